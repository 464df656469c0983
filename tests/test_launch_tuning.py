"""Launch tuning on the device: every CTAs-per-SM setting and every k_lu32
register tiling that covers the network gives the attempt of the default
launch (the work queue hands whole columns to CTAs, and each tiling runs
the same arithmetic on a zero-padded block); a too-small tiling is refused;
the autotuner's pick still reproduces a short vk_run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


def _rel(a, b):
    """max |a-b| / (|b| + 1e-10 of the layer's total): the floor metric."""
    scale = np.abs(b) + 1e-10 * np.abs(b).sum(axis=1, keepdims=True)
    return float(np.max(np.abs(a - b) / scale))


def _handle(precision):
    from test_gpu_parity import make_handle
    return make_handle('c2', ns=[0, 1, 2, 3], precision=precision)


@pytest.mark.parametrize('precision', [0, 1])
def test_launch_settings_leave_results_unchanged(precision):
    from vulcan_gb300 import autotune, capi
    g, net, gn, h, b = _handle(precision)
    dt = g['att_dt'][[0, 1, 2, 3]]
    ref = h.attempt(dt)
    # grids only move whole columns between CTAs (same arithmetic); a tiling
    # could at most change the FP32 factors, which the FP64 refinement
    # absorbs to its tolerance
    tol = 1e-12 if precision == 0 else 1e-10
    kernels = [k for k, (_, paths) in autotune.KERNELS.items() if precision in paths]
    for k in kernels:
        kid = autotune.KERNELS[k][0]
        for c, v in autotune.candidates(k, net.ni):
            h.set_launch(kid, c, v)
            assert h.get_launch(kid) == (c, v if kid == capi.VK_TUNE_LU32 else -1)
            out = h.attempt(dt)
            assert _rel(out['sol'], ref['sol']) <= tol, (k, c, v)
            np.testing.assert_allclose(out['delta'], ref['delta'], rtol=1e3 * tol)
        h.set_launch(kid, 0, -1)
    h.close()


def test_too_small_tiling_refused():
    from vulcan_gb300 import capi
    g, net, gn, h, b = _handle(1)
    with pytest.raises(capi.VkError) as e:
        h.set_launch(capi.VK_TUNE_LU32, 2, 0)        # covers 48 species, the network has 69
    assert e.value.code == capi.VK_EINVAL
    h.close()


def test_tuned_run_matches_default_run():
    from vulcan_gb300 import autotune, configs
    from vulcan_gb300.solver import ctrl_from
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    states = []
    for tuned in (False, True):
        g, net, gn, h, b = _handle(1)
        h.set_atom_ini(np.tile(g['atom_ini'], (b.ncols, 1)))
        h.set_clock(dt=1e-10, t=0.0, count=0)
        if tuned:
            res = autotune.tune(h, 1e-10, repeats=1)
            assert res['_ms'] <= res['_default_ms']
            h.set_columns(b)                       # back to the initial state
            h.set_atom_ini(np.tile(g['atom_ini'], (b.ncols, 1)))
            h.set_clock(dt=1e-10, t=0.0, count=0)
        h.run(ctrl, max_steps=20, timeout_s=300)
        states.append(h.state()['y'].copy())
        h.close()
    assert _rel(states[1], states[0]) <= 1e-10
