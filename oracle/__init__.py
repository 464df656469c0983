"""CPU oracle for the Ros2 kinetics-diffusion step (TEST INFRASTRUCTURE).

This package restates the reference VULCAN algorithm in numpy so that the
GPU implementation can be checked against it.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s ``cpu_baseline`` / reference
arm import it, and only as the reference results are compared with or as the
timed CPU baseline -- never as the product path.  The product (``vulcan_gb300``) does not import it and
fails loudly when its CUDA library is missing.

Parity pin: the restatement is checked against golden vectors recorded from
the reference itself (tests/golden/golden_*.npz, made by
tests/golden/make_golden.py, which runs the unmodified reference code in a
temporary copy).
"""
