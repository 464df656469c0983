"""vk_block_solve_noalloc: the block-tridiagonal solve that allocates nothing.

It exists for callers that cannot call cudaMalloc (their device memory is
owned by another allocator, or they are handed buffers by a host program), so
its scratch is a fixed array inside the library.  The test gives it device
buffers it allocates itself (through PyTorch) and checks its answer against
the regular entry point: vk_ros2_attempt solves (c0 I - J) k1 = f on the same
block-tridiagonal matrix, so solving that matrix for b = A k1 must give k1
back, within the per-step tolerance of the parity tests.  Two different
systems are solved back to back (the shared scratch keeps the previous call's
contents), then the first one again, which must reproduce its answer bit for
bit.  A singular and a non-finite block must be reported, and the next good
call must not see their status.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import column_from_golden, floor_err, golden, network
from oracle import ros2 as O

pytestmark = pytest.mark.gpu


def _system(n):
    """Block-tridiagonal matrix of fixture attempt n (from the regular entry
    point's own LHS) and its k1 from vk_ros2_attempt."""
    from vulcan_gb300.solver import ColumnBatch, GPUNetwork, Ros2Handle
    g = golden('c0')
    net = network('c0')
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    b = ColumnBatch([dict(col=column_from_golden(g, n), k=g['k'], y=g['att_y'][n],
                          ymix=g['att_ymix'][n])], net.ni)
    h = Ros2Handle(gn, 1, b.L)
    h.set_columns(b)
    dt = float(g['att_dt'][n])
    out = h.attempt(dt, want_k=True)
    jv, dA, dB, dC = h.lhs()
    h.close()
    rows, cols = gn.jac_pattern()
    nz, ni = b.L, net.ni
    c0 = 1.0 / (O.R_ROS * dt)
    D = np.zeros((nz, ni, ni))
    D[:, rows, cols] = jv
    idx = np.arange(ni)
    D[:, idx, idx] += c0 - dA
    lower, upper = -dC, -dB
    k1 = out['k1']
    rhs = np.einsum('lij,lj->li', D, k1)
    rhs[1:] += lower[1:] * k1[:-1]
    rhs[:-1] += upper[:-1] * k1[1:]
    return D, lower, upper, rhs, k1, g['n_0']


def _solve(lib, D, lower, upper, rhs):
    import torch
    dev = torch.device('cuda:0')
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (D, lower, upper, rhs)]
    x = torch.empty_like(t[3])
    torch.cuda.synchronize()
    nz, ni = rhs.shape
    p = lambda a: C.c_void_p(a.data_ptr())
    rc = lib.vk_block_solve_noalloc(nz, ni, p(t[0]), p(t[1]), p(t[2]), p(t[3]), p(x), None)
    assert rc == 0, lib.vk_last_error(None)
    return x.cpu().numpy()


def test_noalloc_solve_matches_attempt_twice():
    pytest.importorskip('torch')
    from vulcan_gb300 import _build, capi
    _build.build()
    lib = capi.lib()
    s0 = _system(0)
    s1 = _system(2)
    x0 = _solve(lib, *s0[:4])
    assert floor_err(x0, s0[4], s0[5]) <= 1e-10
    x1 = _solve(lib, *s1[:4])                 # second call in a row, other system
    assert floor_err(x1, s1[4], s1[5]) <= 1e-10
    x0b = _solve(lib, *s0[:4])                # scratch reused: same answer again
    np.testing.assert_array_equal(x0b, x0)


def _status(lib, D, lower, upper, rhs):
    """Return code of one call on caller-owned device buffers."""
    import torch
    dev = torch.device('cuda:0')
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (D, lower, upper, rhs)]
    x = torch.empty_like(t[3])
    torch.cuda.synchronize()
    nz, ni = rhs.shape
    p = lambda a: C.c_void_p(a.data_ptr())
    return lib.vk_block_solve_noalloc(nz, ni, p(t[0]), p(t[1]), p(t[2]), p(t[3]), p(x), None), x


def test_noalloc_reports_singular_and_nan_then_recovers():
    """A zero diagonal block gives VK_ESINGULAR and a NaN in a block VK_ENAN;
    the status word lives in the shared scratch, so a good solve right after
    each must return VK_OK with the right answer (the kernel clears it)."""
    pytest.importorskip('torch')
    from vulcan_gb300 import _build, capi
    _build.build()
    lib = capi.lib()
    nz, ni = 2, 3
    rng = np.random.default_rng(3)
    good = np.stack([np.eye(ni) * 4.0 + 0.1 * rng.standard_normal((ni, ni)) for _ in range(nz)])
    lower = 0.1 * rng.standard_normal((nz, ni))
    upper = 0.1 * rng.standard_normal((nz, ni))
    xt = rng.standard_normal((nz, ni))
    rhs = np.einsum('lij,lj->li', good, xt)
    rhs[1:] += lower[1:] * xt[:-1]
    rhs[:-1] += upper[:-1] * xt[1:]
    zero = good.copy()
    zero[0] = 0.0
    nan = good.copy()
    nan[1, 1, 2] = np.nan
    for bad, code in ((zero, capi.VK_ESINGULAR), (nan, capi.VK_ENAN)):
        rc, _ = _status(lib, bad, lower, upper, rhs)
        assert rc == code, (rc, lib.vk_last_error(None))
        rc, x = _status(lib, good, lower, upper, rhs)
        assert rc == capi.VK_OK, lib.vk_last_error(None)
        np.testing.assert_allclose(x.cpu().numpy(), xt, rtol=1e-12, atol=1e-12)


def test_noalloc_rejects_sizes_beyond_scratch():
    from vulcan_gb300 import _build, capi
    _build.build()
    lib = capi.lib()
    rc = lib.vk_block_solve_noalloc(200, 160, C.c_void_p(1), C.c_void_p(1), C.c_void_p(1),
                                    C.c_void_p(1), C.c_void_p(1), None)
    assert rc == capi.VK_EINVAL
    assert b'exceeds the fixed scratch' in lib.vk_last_error(None)
