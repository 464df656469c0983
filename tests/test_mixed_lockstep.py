"""Mixed precision against FP64 in lock-step: the precision effect alone.

Two handles hold the same column (the reference's c2conv column and initial
state): one solves every attempt in FP64, the other in mixed precision (FP32
tensor-core block factors + FP64 refinement, routed to FP64 per column where
the refinement fails).  The FP64 path drives the step control exactly as the
reference does (clip, the step_ok test with atom conservation, step halving
on rejection, the step-size rule; op.py:2447-2534, 3091-3125); the mixed path
takes the same step sizes and the same accept/reject decisions from its own
state.  So the two trajectories differ only by the arithmetic of the linear
solves, and their mixing ratios must stay within 1e-3 relative wherever the
FP64 value exceeds 1e-20, from dt = 1e-10 s through the late, stiff steps.
(Runs that take their own decisions fork at the late steps' conditioning
floor and stop at different points of the slow evolution; that is a property
of the reference problem, not of the precision.)
"""
import numpy as np
import pytest

from helpers import golden, network, oracle_net
from oracle import ros2 as O

pytestmark = pytest.mark.gpu

NSTEPS = 700
CHECK_EVERY = 50


def test_mixed_follows_fp64_within_1e3():
    from vulcan_gb300 import _build
    from test_gpu_parity import make_handle
    _build.build()
    g, net, gn, h64, b = make_handle('c2conv', precision=0)
    _, _, _, h32, _ = make_handle('c2conv', precision=1)
    on = oracle_net('c2conv', g)
    tol = O.Tol()
    n0 = g['n_0'][:, None]
    atom_ini = g['atom_ini']
    y64, ym64 = g['y_ini'].copy(), g['ymix_ini'].copy()
    y32, ym32 = y64.copy(), ym64.copy()
    loss_prev = np.zeros(len(atom_ini))
    dt, t = 1e-10, 0.0
    worst, checked, dt_max = 0.0, 0, 0.0
    for step in range(1, NSTEPS + 1):
        while True:
            h64.set_state(y64, ym64)
            h32.set_state(y32, ym32)
            o64 = h64.attempt(dt)
            o32 = h32.attempt(dt)
            c64, cm64 = O.clip(o64['sol'], o64['ymix'], tol)
            loss = (O.atom_sums(on, c64) - atom_ini) / atom_ini
            ok = (np.all(c64 >= 0) and np.amax(np.abs(loss - loss_prev)) < tol.loss_eps
                  and o64['delta'][0] <= tol.rtol)
            if ok or dt * tol.dt_var_min < tol.dt_min:
                break
            dt *= tol.dt_var_min
        c32, cm32 = O.clip(o32['sol'], o32['ymix'], tol)
        loss_prev = loss
        # renormalisation of the reference loop (op.py:894): y = n_0 ymix
        y64, ym64 = n0 * cm64, cm64
        y32, ym32 = n0 * cm32, cm32
        t += dt
        dt_max = max(dt_max, dt)
        if step % CHECK_EVERY == 0:
            m = ym64 > 1e-20
            e = float(np.max(np.abs(ym32[m] - ym64[m]) / ym64[m]))
            worst = max(worst, e)
            checked += 1
            assert e <= 1e-3, (step, t, dt, e)
        dt = O.step_size(dt, o64['delta'][0], tol)
    h64.close()
    h32.close()
    print('lock-step: %d steps to t = %.3e s (dt up to %.2e s), worst ymix rel. diff %.2e'
          % (NSTEPS, t, dt_max, worst))
    assert checked == NSTEPS // CHECK_EVERY
    assert dt_max > 1e2            # the run reached the stiff late phase
