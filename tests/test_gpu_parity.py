"""GPU Ros2 step vs the reference's recorded attempts and vs the CPU oracle.

Tolerances (see tests/test_oracle.py for the reasoning):
  per attempt  |sol_gpu - sol_ref| <= 1e-10 (|sol_ref| + 1e-10 n_0) and delta to
               1e-6 relative for dt < 1e-2 s; at the late stiff steps 10x the
               reference's own conditioning floor (helpers.reference_floor).
  chemistry    bit-identical to the reference's generated chemdf.
"""
import types

import numpy as np
import pytest

from helpers import (attempt_atm, column_from_golden, floor_err, golden, network,
                     oracle_net, reference_floor, step_tolerance)
from oracle import ros2 as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


def make_handle(tag, ncols=1, ns=None, precision=0):
    from vulcan_gb300.solver import ColumnBatch, GPUNetwork, Ros2Handle
    g = golden(tag)
    net = network(tag)
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    ns = ns if ns is not None else [None] * ncols
    items = []
    for n in ns:
        col = column_from_golden(g, n)
        y = g['y_ini'] if n is None else g['att_y'][n]
        ym = g['ymix_ini'] if n is None else g['att_ymix'][n]
        items.append(dict(col=col, k=g['k'], y=y, ymix=ym))
    b = ColumnBatch(items, net.ni)
    h = Ros2Handle(gn, len(items), b.L, precision)
    h.set_columns(b)
    return g, net, gn, h, b


@pytest.mark.parametrize('tag', ['c0', 'c1', 'c2'])
def test_chem_source_bit_exact(tag):
    g, net, gn, h, b = make_handle(tag)
    np.testing.assert_array_equal(h.chem_source(g['y_ini']), g['chemdf0'])


@pytest.mark.parametrize('tag', ['c0', 'c2'])
def test_lhs_matches_oracle(tag):
    g, net, gn, h, b = make_handle(tag, ns=[0])
    h.attempt(g['att_dt'][0])
    jv, dA, dB, dC = h.lhs()
    on = oracle_net(tag, g)
    y = g['att_y'][0]
    J = O.neg_jac_blocks(on, y, g['M'], g['k'])
    rows, cols = gn.jac_pattern()
    for l in (0, 1, y.shape[0] // 2, y.shape[0] - 1):
        ref = J[l][rows, cols]
        scale = np.abs(J[l]).max()
        assert np.max(np.abs(jv[l] - ref)) <= 1e-14 * scale
    A, B, C, Ai, Bi, Ci = O.diff_coeffs(y, attempt_atm(g, 0), O.Flags())
    # eddy + molecular parts can nearly cancel: compare against their magnitudes
    for got, e, m, sl in ((dA, A, Ai, slice(None)), (dB, B, Bi, slice(0, -1)),
                          (dC, C, Ci, slice(1, None))):
        ref = e[:, None] + m
        mag = np.abs(e[:, None]) + np.abs(m)
        assert np.all(np.abs(got[sl] - ref[sl]) <= 1e-13 * mag[sl])


def _cases():
    out = []
    for tag in ('c0', 'c1', 'c2', 'c2long'):
        try:
            g = golden(tag)
        except FileNotFoundError:
            continue
        out += [(tag, n) for n in range(len(g['att_index']))]
    return out


@pytest.mark.parametrize('tag,n', _cases())
def test_attempt_matches_reference(tag, n):
    g, net, gn, h, b = make_handle(tag, ns=[n])
    out = h.attempt(g['att_dt'][n], want_k=True)
    n0 = g['n_0']
    if g['att_dt'][n] < 1e-2:
        tol, dtol = 1e-10, 1e-6
        yk2_ref = g['att_y'][n] + g['att_k1'][n].reshape(out['k1'].shape) / O.R_ROS
        yk2 = g['att_y'][n] + out['k1'] / O.R_ROS
        assert floor_err(yk2, yk2_ref, n0) <= 1e-9
    else:
        tol, dtol = step_tolerance(*reference_floor(tag, g, n))
    assert floor_err(out['sol'], g['att_sol'][n], n0) <= tol
    assert abs(out['delta'][0] / g['att_delta'][n] - 1) <= dtol
    ym = out['sol'] / out['sol'].sum(axis=1, keepdims=True)
    np.testing.assert_allclose(out['ymix'], ym, rtol=1e-14, atol=0)


@pytest.mark.parametrize('tag,n', _cases())
def test_mixed_attempt_matches_reference(tag, n):
    """FP32 scaled block LU + FP64 refinement: same per-attempt tolerances as
    the FP64 path (refinement runs to 1e-13 of |x| + |y|, or the column is
    redone in FP64)."""
    g, net, gn, h, b = make_handle(tag, ns=[n], precision=1)
    out = h.attempt(g['att_dt'][n], want_k=True)
    n0 = g['n_0']
    if g['att_dt'][n] < 1e-2:
        tol, dtol = 1e-10, 1e-6
    else:
        tol, dtol = step_tolerance(*reference_floor(tag, g, n))
    assert floor_err(out['sol'], g['att_sol'][n], n0) <= tol
    assert abs(out['delta'][0] / g['att_delta'][n] - 1) <= dtol


def test_mixed_matches_fp64_path_batch():
    """Mixed and FP64 solves of the same batch of attempts agree to the
    refinement tolerance (well-conditioned early steps)."""
    g = golden('c0')
    ns = [0, 3, 5, 9]
    dts = np.array([g['att_dt'][n] for n in ns])
    _, _, _, h64, b = make_handle('c0', ns=ns)
    _, _, _, h32, _ = make_handle('c0', ns=ns, precision=1)
    o64 = h64.attempt(dts)
    o32 = h32.attempt(dts)
    for c, n in enumerate(ns):
        n0 = g['n_0']
        sl = slice(b.off[c], b.off[c + 1])
        assert floor_err(o32['sol'][sl], o64['sol'][sl], n0) <= 1e-11
    np.testing.assert_allclose(o32['delta'], o64['delta'], rtol=1e-8)


def test_batch_invariance_and_determinism():
    """Columns in one batch give bit-identical results to single-column runs,
    and repeated runs are bit-identical (no atomics on the FP64 path)."""
    g = golden('c0')
    ns = [0, 5, 9, 13]
    _, _, _, hb, bb = make_handle('c0', ns=ns)
    dts = np.array([g['att_dt'][n] for n in ns])
    ob = hb.attempt(dts)
    ob2 = hb.attempt(dts)
    np.testing.assert_array_equal(ob['sol'], ob2['sol'])
    sols = bb.split(ob['sol'])
    for c, n in enumerate(ns):
        _, _, _, h1, _ = make_handle('c0', ns=[n])
        o1 = h1.attempt(g['att_dt'][n])
        np.testing.assert_array_equal(sols[c], o1['sol'])
        assert ob['delta'][c] == o1['delta'][0]


def test_nan_state_reports_status():
    """A NaN injected into the state is reported as VK_ENAN (host-visible
    status, the context stays usable)."""
    from vulcan_gb300 import capi
    g, net, gn, h, b = make_handle('c0', ns=[0])
    y = g['att_y'][0].copy()
    y[7, 3] = np.nan
    h.set_state(y, g['att_ymix'][0])
    with pytest.raises(capi.VkError) as e:
        h.attempt(g['att_dt'][0])
    assert e.value.code == capi.VK_ENAN
    h.set_state(g['att_y'][0], g['att_ymix'][0])
    out = h.attempt(g['att_dt'][0])
    assert floor_err(out['sol'], g['att_sol'][0], g['n_0']) <= 1e-10


def test_bad_dt_rejected():
    from vulcan_gb300 import capi
    g, net, gn, h, b = make_handle('c0', ns=[0])
    for dt in (0.0, -1.0, np.inf, np.nan):
        with pytest.raises(capi.VkError) as e:
            h.attempt(dt)
        assert e.value.code == capi.VK_EINVAL


def test_dropin_solver_contract():
    """Ros2GPU.solver reads var/atm like op.Ros2.solver and writes var.y,
    var.ymix and para.delta (a stand-in op module; the reference itself is
    not needed on the GPU machine)."""
    from vulcan_gb300.solver import make_ros2gpu
    g = golden('c0')
    net = network('c0')
    n = 3

    class FakeRos2:
        pass

    op = types.SimpleNamespace(Ros2=FakeRos2)
    cfg = types.SimpleNamespace(network=None, use_photo=False, atom_list=list(g['atom_list']),
                                use_moldiff=True, use_topflux=False, use_botflux=False)
    cls = make_ros2gpu(op, cfg, net.species)
    cls._vk_net_cls = types.SimpleNamespace(from_file=lambda path, use_photo: net)
    s = cls()
    var = types.SimpleNamespace(y=g['att_y'][n].copy(), ymix=g['att_ymix'][n].copy(),
                                dt=float(g['att_dt'][n]),
                                k={i: g['k'][i - 1] for i in range(1, net.nr + 1)})
    col = column_from_golden(g, n)
    atm = types.SimpleNamespace(**{k: getattr(col, k) for k in (
        'M', 'n_0', 'Tco', 'g', 'dzi', 'Kzz', 'vz', 'Ti', 'Hpi', 'Hp', 'pico', 'dz', 'Dzz',
        'ms', 'alpha', 'top_flux', 'bot_flux', 'bot_vdep', 'pref_indx')})
    para = types.SimpleNamespace(delta=0.0)
    var, para = s.solver(var, atm, para)
    assert floor_err(var.y, g['att_sol'][n], g['n_0']) <= 1e-10
    assert abs(para.delta / g['att_delta'][n] - 1) <= 1e-6


def test_device_run_tracks_reference_trajectory():
    """vk_run (device accept/reject, step size, update_mu_dz, renormalisation)
    from the reference's initial state reproduces its first 100 steps."""
    from vulcan_gb300 import configs
    from vulcan_gb300.solver import ctrl_from
    g, net, gn, h, b = make_handle('c0')
    h.set_atom_ini(g['atom_ini'][None, :])
    h.set_clock(dt=1e-10, t=0.0, count=0)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    h.run(ctrl, max_steps=100, timeout_s=600)
    st = h.state()
    cnt = h.counters()
    assert st['count'][0] == 100
    assert cnt[0, 0] == g['traj_natt'][99]
    np.testing.assert_allclose(st['t'][0], g['traj_t'][99], rtol=1e-9)
    np.testing.assert_allclose(st['dt'][0], g['traj_dt_next'][99], rtol=1e-8)
    y100 = g['ystep_y'][list(g['ystep_index']).index(99)]
    assert floor_err(st['y'], y100, g['n_0']) <= 1e-8


def test_run_watchdog_returns_timeout():
    from vulcan_gb300 import capi, configs
    from vulcan_gb300.solver import ctrl_from
    g, net, gn, h, b = make_handle('c0')
    h.set_atom_ini(g['atom_ini'][None, :])
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    with pytest.raises(capi.VkError) as e:
        h.run(ctrl, max_steps=1000, timeout_s=1e-9)
    assert e.value.code == capi.VK_ETIMEOUT
    st = h.state()                    # the handle stays usable
    assert np.isfinite(st['y']).all()


def _run_to_steady(tag, precision, count_max=20000, **cfg):
    from vulcan_gb300 import configs
    from vulcan_gb300.solver import ctrl_from
    g, net, gn, h, b = make_handle(tag, precision=precision)
    h.set_atom_ini(g['atom_ini'][None, :])
    mask = np.zeros(net.ni, dtype=np.int32)
    for sp in g['conver_ignore']:
        if str(sp) in net.species:
            mask[net.species.index(str(sp))] = 1
    h.set_conv_ignore(mask)
    h.set_clock(dt=1e-10, t=0.0, count=0)
    ctrl = ctrl_from(cfg, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = count_max
    h.run(ctrl, max_steps=count_max + 10, timeout_s=900)
    return g, h.state()


@pytest.mark.parametrize('precision', [0, 1])
def test_device_run_converges_like_reference(precision):
    """vk_run from the reference's initial state stops by the reference's own
    convergence test (op.py:1018-1085, default criterion).  That test allows
    10 % drift over the last half of the run time once t is large
    (yconv_min = 0.1 with the slope clause), so runs that part at the late
    steps' conditioning floor stop at different points; the step count is
    compared.  Under a tightened criterion (yconv_cri = yconv_min = 1e-3) the
    reference itself does not converge within 12 000 steps (fixture c2tight,
    tests/test_oracle.py), so no reference steady state pins the state
    to 1e-3."""
    g, st = _run_to_steady('c2conv', precision)
    assert st['end_case'][0] == 1
    assert 0.4 * g['final_count'] <= st['count'][0] <= 2.5 * g['final_count']
    # the final state against the reference's, on the entries the
    # convergence test itself judges (op.py:1041-1046: ymix >= mtol_conv,
    # y >= atol, conver_ignore species left out): within the criterion's own
    # tolerances -- yconv_cri (0.01) in the median, yconv_min (0.1 relative
    # change over the last half of the run time) at the 90th percentile
    tol = O.Tol()
    ref, yref = g['final_ymix'], g['final_y']
    m = (ref >= tol.mtol_conv) & (yref >= tol.atol)
    net = network('c2conv')
    for sp in g['conver_ignore']:
        m[:, net.species.index(str(sp))] = False
    rel = np.abs(st['ymix'][m] - ref[m]) / ref[m]
    q50, q90, q99, qmax = np.percentile(rel, [50, 90, 99, 100])
    print('c2conv final ymix vs reference (precision %d, t %.3e vs %.3e s): median %.2e, '
          '90%% %.2e, 99%% %.2e, max %.2e'
          % (precision, st['t'][0], g['final_t'], q50, q90, q99, qmax))
    assert q50 <= tol.yconv_cri and q90 <= tol.yconv_min


@pytest.mark.parametrize('precision', [0, 1])
def test_slow_column_stalls_like_reference(precision):
    """A column that the reference itself does not bring to steady state in
    4000 steps (fixture c2slow: count_max reached at t = 7e6 s with dt ~ 1e3 s,
    the stall the device batch shows on a quarter of the uneven columns):
    the device run stalls the same way -- the stragglers of a batch come from
    the reference algorithm, not from this implementation."""
    from vulcan_gb300 import configs
    from vulcan_gb300.solver import ctrl_from
    g, net, gn, h, b = make_handle('c2slow', precision=precision)
    h.set_atom_ini(g['atom_ini'][None, :])
    mask = np.zeros(net.ni, dtype=np.int32)
    for sp in g['conver_ignore']:
        if str(sp) in net.species:
            mask[net.species.index(str(sp))] = 1
    h.set_conv_ignore(mask)
    h.set_clock(dt=1e-10, t=0.0, count=0)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = int(g['final_count']) - 1
    h.run(ctrl, max_steps=10 * int(g['final_count']), timeout_s=900)
    st = h.state()
    assert g['end_case'] == 3
    assert st['end_case'][0] == 3 and st['count'][0] == g['final_count']
    assert 0.2 * g['final_t'] <= st['t'][0] <= 5.0 * g['final_t']
    dt_ref = np.median(g['traj_dt_used'][-500:])
    assert 0.05 * dt_ref <= st['dt'][0] <= 20 * dt_ref
