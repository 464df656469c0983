"""The tensor-core block factorisation (k_lu_tc: blocked Gauss-Jordan, rank-16
updates as split-TF32 tcgen05 MMAs with the block held in TMEM) against the
CUDA-core FP32 Gauss-Jordan (k_lu32) on the same mixed-precision attempts.

Both invert the same FP32 scaled blocks, so their inverses agree to FP32
rounding amplified by each block's condition number; what the solver needs
from them is that the FP64 refinement converges as fast: the attempts match
the reference's recorded ones to the per-step bar, no column falls back to
FP64, and the refinement needs at most one sweep more.
"""
import numpy as np
import pytest

from helpers import floor_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


def _factors(h, ni, L):
    from vulcan_gb300 import capi
    import ctypes as C
    G = np.empty((L, ni * ni), dtype=np.float32)
    capi.check(capi.lib().vk_get_lu32(h.h, G.ctypes.data_as(C.POINTER(C.c_float))), h.h)
    return G.reshape(L, ni, ni)


@pytest.mark.parametrize('tag,ns', [('c2', [0, 1, 2, 3, 4]), ('c0', [0, 3, 8, 13]),
                                    ('c3s', [0, 1, 2, 3, 4]), ('c2long', [0])])
def test_tensor_core_factors_match_cuda_core_factors(tag, ns):
    from test_gpu_parity import make_handle
    from vulcan_gb300 import capi
    g, net, gn, h, b = make_handle(tag, ns=ns, precision=1)
    dt = g['att_dt'][ns]
    # the CUDA-core kernel: the smallest register tiling that covers ni
    h.set_launch(capi.VK_TUNE_LU32, 0, min(t for t, cap in enumerate(capi.LU32_TILING_CAP[:4])
                                           if cap >= net.ni))
    out_ref = h.attempt(dt)
    sw_ref, fb_ref = h.refine_stats()
    G_ref = _factors(h, net.ni, b.L)
    h.set_launch(capi.VK_TUNE_LU32, 0, capi.LU32_TC)
    out = h.attempt(dt)
    sw, fb = h.refine_stats()
    G = _factors(h, net.ni, b.L)
    h.close()
    # inverses: FP32 agreement scaled by the block's own magnitude
    scale = np.abs(G_ref).max(axis=(1, 2), keepdims=True)
    rel = np.abs(G - G_ref) / scale
    print('%s: max %.2e median %.2e of per-layer max |dG|/max|G|; sweeps %d vs %d, fallbacks %d vs %d'
          % (tag, rel.max(), np.median(rel.max(axis=(1, 2))), sw, sw_ref, fb, fb_ref))
    assert fb <= fb_ref
    if tag == 'c2long':          # late, ill-conditioned blocks: both fall back to FP64
        return
    assert np.isfinite(G).all()
    assert np.median(rel.max(axis=(1, 2))) < 1e-4
    assert sw <= sw_ref + 1
    sols, sols_ref = b.split(out['sol']), b.split(out_ref['sol'])
    for i, n in enumerate(ns):
        assert floor_err(sols[i], sols_ref[i], g['n_0']) <= 1e-10
        assert floor_err(sols[i], g['att_sol'][n], g['n_0']) <= 1e-10


def test_tensor_core_is_the_default_up_to_128_species():
    """Without a launch setting the mixed path factorises on the tensor cores
    (variant -1 resolves to the cooperative-panel variant 5 for ni <= 128):
    its factors equal an explicit variant-4 run bit for bit."""
    from test_gpu_parity import make_handle
    from vulcan_gb300 import capi
    g, net, gn, h, b = make_handle('c2', ns=[0, 1], precision=1)
    dt = g['att_dt'][[0, 1]]
    h.attempt(dt)
    G0 = _factors(h, net.ni, b.L)
    h.set_launch(capi.VK_TUNE_LU32, 0, capi.LU32_TC)
    h.attempt(dt)
    G1 = _factors(h, net.ni, b.L)
    h.close()
    np.testing.assert_array_equal(G0, G1)
    assert capi.LU32_TILING_CAP[capi.LU32_TC] == 128


@pytest.mark.parametrize('tag,ns', [('c2', [0, 1, 2, 3, 4]), ('c3s', [0, 1, 2])])
def test_cooperative_panel_gives_the_same_factors(tag, ns):
    """Variant 5 eliminates each panel with the CTA's four warps instead of
    one; the pivots and every FP32 operation are the same, so the factors and
    the attempt equal variant 4's bit for bit."""
    from test_gpu_parity import make_handle
    from vulcan_gb300 import capi
    g, net, gn, h, b = make_handle(tag, ns=ns, precision=1)
    dt = g['att_dt'][ns]
    h.set_launch(capi.VK_TUNE_LU32, 0, capi.LU32_TC)
    out4 = h.attempt(dt)
    G4 = _factors(h, net.ni, b.L)
    h.set_launch(capi.VK_TUNE_LU32, 0, capi.LU32_TC_COOP)
    out5 = h.attempt(dt)
    G5 = _factors(h, net.ni, b.L)
    h.close()
    np.testing.assert_array_equal(G5, G4)
    np.testing.assert_array_equal(out5['sol'], out4['sol'])
    assert capi.LU32_TILING_CAP[capi.LU32_TC_COOP] == 128
