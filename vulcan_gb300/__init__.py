"""vulcan_gb300: GB300-native Ros2 kinetics-diffusion step for VULCAN networks.

Python host code over a ctypes C-ABI (include/vk_ros2.h) to hand-written
sm_103a CUDA kernels.  Modules:
  network   - VULCAN network-file compiler and FP64 rate constants
  column    - atmospheric column set-up (T-P-Kzz, gravity, diffusion)
  configs   - seeded synthetic workloads
  solver    - device handles, column batches and the Ros2GPU drop-in
  batch     - many columns to steady state (vk_run), photochemistry schedule
  photo     - radiative-transfer tables (bins, cross sections, stellar flux)
  warmstart - learned warm start (BF16 MLP), element projection, EQ start
  eqchem    - thermochemical equilibrium (Gibbs minimisation)
  vulio     - .vul output and vulcan_ini restart
  replicas  - one process per GPU over disjoint column sets
  synthnet  - seeded synthetic stress network in the reference's formats
  capi      - the ctypes binding of libvk_gb300.so
"""
from .network import Network  # noqa: F401
from . import column, configs  # noqa: F401


def build(verbose=False):
    """Compile libvk_gb300.so in-tree (nvcc, sm_103a)."""
    from ._build import build as _b
    return _b(verbose=verbose)
