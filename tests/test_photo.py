"""Photochemistry radiative transfer: the oracle against the reference's own
compute_tau / compute_flux / compute_J (fixtures c1rt and, with
temperature-dependent cross sections for CO2, H2O and NH3, c1rtT, recorded
with the reference's radiative transfer on), and the device path against
the oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import photo as P


def _fixture(tag='c1rt'):
    d = dict(np.load(os.path.join(GOLDEN, 'golden_%s.npz' % tag), allow_pickle=False))
    spec = [str(s) for s in d['spec_list']]
    d['absp_idx'] = [spec.index(str(s)) for s in d['absp_sp']]
    d['photo_idx'] = [spec.index(str(s)) for s in d['photo_sp']]
    d['scat_idx'] = [spec.index(str(s)) for s in d['scat_sp']]
    absp = [str(s) for s in d['absp_sp']]
    d['cross_photo'] = np.array([d['cross'][absp.index(str(s))] for s in d['photo_sp']])
    d['weights'] = P.j_weights(len(d['bins']), int(d['sflux_din12_indx']), float(d['dbin1']),
                               float(d['dbin2']))
    # temperature-dependent tables keyed by absorber / channel position
    chans = list(zip([str(s) for s in d['ch_sp']], [int(b) for b in d['ch_br']]))
    d['chans'] = chans
    d['cross_T_at'], d['cross_J_T_at'] = {}, {}
    if 'T_cross_sp' in d:
        for i, sp in enumerate(d['T_cross_sp']):
            d['cross_T_at'][absp.index(str(sp))] = d['cross_T'][i]
        for i, c in enumerate(zip([str(s) for s in d['chT_sp']], [int(b) for b in d['chT_br']])):
            d['cross_J_T_at'][chans.index(c)] = d['cross_J_T'][i]
    return d


def _oracle_call(d, y, ymix, dz, du, dd, prev=None):
    tau = P.compute_tau(y, dz, d['absp_idx'], d['cross'], d['scat_idx'], d['cross_scat'],
                        d['cross_T_at'])
    af, _, ch = P.compute_flux(tau, ymix, d['photo_idx'], d['cross_photo'], d['scat_idx'],
                               d['cross_scat'], d['sflux_top'], d['bins'], float(d['sl_angle']),
                               float(d['edd']), du, dd, aflux_prev=prev,
                               flux_atol=float(d['flux_atol']))
    return tau, af, P.compute_J(af, d['cross_J'], d['weights'], d['cross_J_T_at']), ch


def _rel(a, b, floor=1e-300):
    m = np.abs(b) > floor
    return float(np.max(np.abs(a - b)[m] / np.abs(b)[m]))


@pytest.mark.parametrize('tag', ['c1rt', 'c1rtT', 'c1rtA', 'c3rt'])
def test_oracle_matches_reference_records(tag):
    d = _fixture(tag)
    nz, nb = d['rec0_y'].shape[0], len(d['bins'])
    du, dd = np.zeros((nz + 1, nb)), np.zeros((nz + 1, nb))
    # first call (set-up), then the integrator's first update on the same state
    # (the downward sweep reads the first call's upward flux), then count 100
    tau, af, J, _ = _oracle_call(d, d['rec0_y'], d['rec0_ymix'], d['rec0_dz'], du, dd)
    assert _rel(tau, d['rec0_tau']) < 1e-13
    assert _rel(af, d['rec0_aflux'], 1e-30) < 1e-12
    assert _rel(J, d['rec0_J']) < 1e-11
    np.testing.assert_allclose(du, d['rec0_dflux_u'], rtol=1e-10, atol=1e-12 * np.abs(du).max())
    _, af1, J1, ch1 = _oracle_call(d, d['rec0_y'], d['rec0_ymix'], d['rec0_dz'], du, dd, af)
    assert _rel(af1, d['rec1_aflux'], 1e-30) < 1e-12 and _rel(J1, d['rec1_J']) < 1e-11
    assert abs(ch1 / float(d['rec1_aflux_change']) - 1) < 1e-10
    np.testing.assert_allclose(du, d['rec1_dflux_u'], rtol=1e-10, atol=1e-12 * np.abs(du).max())
    if int(d['n_rec']) > 2:
        _, af2, J2, _ = _oracle_call(d, d['rec2_y'], d['rec2_ymix'], d['rec2_dz'], du, dd, af1)
        assert _rel(af2, d['rec2_aflux'], 1e-30) < 1e-12 and _rel(J2, d['rec2_J']) < 1e-11
    if d['cross_J_T_at']:             # the per-layer tables change J well above rounding
        e = dict(d, cross_T_at={}, cross_J_T_at={})
        du, dd = np.zeros((nz + 1, nb)), np.zeros((nz + 1, nb))
        _, _, J0, _ = _oracle_call(e, d['rec0_y'], d['rec0_ymix'], d['rec0_dz'], du, dd)
        assert _rel(J0, d['rec0_J']) > 1e-3


def test_host_tables_match_the_reference_set_up():
    """vulcan_gb300.photo.PhotoTables.from_reference_files against the tables
    the reference's make_bins_read_cross / read_sflux built from the same
    files (differences recorded by the fixture generator)."""
    d = _fixture()
    assert bool(d['setup_same_layout'])
    for key in ('bins', 'cross', 'cross_J', 'cross_scat', 'sflux_top'):
        assert float(d['setup_rel_' + key]) <= 1e-15, key
    # T-dependent per-layer tables (photo.TCross) for the c1 column's
    # 973-2535 K: CO2 above its hottest table for the upper layers and
    # between tables below, H2O between tables, NH3 above its hottest
    t = _fixture('c1rtT')
    assert bool(t['setup_same_layout'])
    for key in ('cross', 'cross_J', 'cross_T', 'cross_J_T'):
        assert float(t['setup_rel_' + key]) <= 1e-15, key
    # dbin_12trans beyond the bins (index -1), 2 nm bins
    a = _fixture('c1rtA')
    assert bool(a['setup_same_layout']) and int(a['sflux_din12_indx']) == -1
    for key in ('bins', 'cross', 'cross_J', 'cross_scat', 'sflux_top'):
        assert float(a['setup_rel_' + key]) <= 1e-15, key
    # the sulfur network: 37 absorbers, 60 channels, a branching-ratio table
    # whose last rows are out of order (CH3SH; interp1d sorts, so do we)
    sn = _fixture('c3rt')
    assert bool(sn['setup_same_layout']) and len(sn['absp_sp']) == 37 and len(sn['ch_sp']) == 60
    for key in ('bins', 'cross', 'cross_J', 'cross_scat', 'sflux_top'):
        assert float(sn['setup_rel_' + key]) <= 1e-15, key


def _tcross(temps, base=2e-18):
    """photo.TCross over synthetic tables: one absorber with two branches
    (ratios 0.25 / 0.75), tables at ``temps`` of constant cross section
    1e-18 x T/100 over 100-200 nm (disso = 0.5 x cross), bins 50-250 nm."""
    from vulcan_gb300 import photo
    bins = np.arange(50., 250., 10.)
    inside = (bins >= 100.) & (bins <= 200.)
    t = photo.PhotoTables(bins=bins, dbin1=10., dbin2=10., i12=-1, sflux_top=np.ones_like(bins),
                          absp_sp=['X'], cross=np.full((1, bins.size), base), scat_sp=[],
                          cross_scat=np.zeros((0, bins.size)), ch_sp=['X', 'X'], ch_br=[1, 2],
                          cross_J=np.array([np.full(bins.size, base * 0.25),
                                            np.full(bins.size, base * 0.75)]),
                          sl_angle=0.5, edd=0.5, f_diurnal=1.0, flux_atol=1.0)
    lam = np.linspace(100., 200., 11)
    raw = {T: (lam, np.full(11, 1e-18 * T / 100.), np.full(11, 0.5e-18 * T / 100.))
           for T in temps}
    raw[300] = (lam, np.full(11, base), np.full(11, base))
    ratio = {('X', 1): np.full(bins.size, 0.25), ('X', 2): np.full(bins.size, 0.75)}
    return photo.TCross(t, {'X': raw}, ratio), inside, bins


def test_tcross_cases():
    """The reference's three temperature cases (op.py:649-747) on synthetic
    tables: log-linear in T between two tables inside their common
    wavelengths; the nearest table at or beyond either end; the
    T-independent values outside a table's wavelengths or where the end
    table is the 300 K one."""
    base = 2e-18
    tc, inside, bins = _tcross([100, 500], base)
    ct, cj = tc.for_column(np.array([200., 50., 900., 100.]))
    c = ct['X']
    # 200 K between 100 K (1e-18) and 300 K (base): log-linear at a half
    want = 10 ** (np.log10(1e-18) + 0.5 * (np.log10(base) - np.log10(1e-18)))
    np.testing.assert_allclose(c[0][inside], want, rtol=1e-14)
    assert np.all(c[0][~inside] == base)
    # disso between 0.5e-18 and base, times the branch ratio
    wj = 10 ** (np.log10(0.5e-18) + 0.5 * (np.log10(base) - np.log10(0.5e-18)))
    np.testing.assert_allclose(cj[('X', 2)][0][inside], 0.75 * wj, rtol=1e-14)
    assert np.all(cj[('X', 1)][0][~inside] == base * 0.25)
    # 50 K: below every table -> the 100 K table; 900 K: above -> 500 K table
    assert np.all(c[1][inside] == 1e-18) and np.all(c[1][~inside] == base)
    assert np.all(c[2][inside] == 5e-18) and np.all(cj[('X', 1)][2][inside] == 0.25 * 2.5e-18)
    # exactly at the lowest table: between it and the next (the reference's <= / >)
    np.testing.assert_allclose(c[3][inside], 1e-18, rtol=1e-14)
    # the 300 K table at an end: T-independent values
    tc, inside, _ = _tcross([500], base)
    ct, cj = tc.for_column(np.array([250.]))
    assert np.all(ct['X'][0] == base) and np.all(cj[('X', 2)][0] == base * 0.75)
    tc, inside, _ = _tcross([100], base)
    ct, _ = tc.for_column(np.array([400.]))
    assert np.all(ct['X'][0] == base)


def test_tcross_zero_cross_sections():
    """A zero table value is log10 -100: both tables zero gives 0, one zero
    gives a vanishing interpolant (the reference's -100 convention)."""
    tc, inside, bins = _tcross([100], 2e-18)
    tc.raw['X'][100] = (tc.raw['X'][100][0], np.zeros(11), np.zeros(11))
    ct, cj = tc.for_column(np.array([200.]))
    v = ct['X'][0][inside]
    assert np.all((v > 0) & (v < 1e-50))
    tc.raw['X'][300] = (tc.raw['X'][300][0], np.zeros(11), np.zeros(11))
    ct, cj = tc.for_column(np.array([200.]))
    assert np.all(ct['X'][0][inside] == 0) and np.all(cj[('X', 1)][0][inside] == 0)


def test_tcross_batch_layout():
    tc, inside, bins = _tcross([100, 500])
    Ts = [np.array([200., 900.]), np.array([50., 250., 600.])]
    ct, cj = tc.for_columns(Ts)
    assert ct['X'].shape == (5, bins.size) and cj[('X', 1)].shape == (5, bins.size)
    one, _ = tc.for_column(Ts[1])
    np.testing.assert_array_equal(ct['X'][2:], one['X'])


def test_j_weights_follow_the_reference_sums():
    """The weights reproduce the reference's four-part trapezoid sums, also
    when the dbin switch lies outside the bins (index -1)."""
    rng = np.random.default_rng(0)
    for i12 in (5, -1):
        f = rng.random(20)
        ref = (np.sum(f[:i12]) * 0.1 - 0.5 * (f[0] + f[i12 - 1]) * 0.1
               + np.sum(f[i12:]) * 2.0 - 0.5 * (f[i12] + f[-1]) * 2.0)
        assert abs(f @ P.j_weights(20, i12, 0.1, 2.0) - ref) < 1e-13


def _attach(h, d, net):
    """The fixture's tables on a handle whose batch is the c1 column."""
    from vulcan_gb300 import photo
    photo.attach(h, photo.PhotoTables.from_fixture(d), net)
    if 'T_cross_sp' in d:
        photo.attach_cross_T(
            h, {str(sp): d['cross_T'][i] for i, sp in enumerate(d['T_cross_sp'])},
            {(str(sp), int(br)): d['cross_J_T'][i]
             for i, (sp, br) in enumerate(zip(d['chT_sp'], d['chT_br']))})


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['c1rt', 'c1rtT'])
def test_device_radiative_transfer_matches_oracle(tag):
    """vk_photo_update on the c1 column (the reference's set-up arrays) from
    the recorded states: tau, actinic flux, J and the k slots, over the three
    recorded calls (the diffuse fluxes persist between calls); c1rtT with
    per-layer cross sections (vk_photo_set_cross_T)."""
    from test_gpu_parity import make_handle
    from vulcan_gb300 import _build
    from vulcan_gb300.capi import ATM_DZ
    _build.build()
    d = _fixture(tag)
    g, net, gn, h, b = make_handle('c1')
    np.testing.assert_allclose(g['dz'], d['rec0_dz'], rtol=1e-14)
    np.testing.assert_array_equal(g['Tco'], d['Tco'])
    _attach(h, d, net)
    nz = d['rec0_y'].shape[0]
    nb = len(d['bins'])
    du, dd = np.zeros((nz + 1, nb)), np.zeros((nz + 1, nb))
    prev = None
    states = [(d['rec0_y'], d['rec0_ymix']), (d['rec0_y'], d['rec0_ymix'])]
    if int(d['n_rec']) > 2:
        states.append((d['rec2_y'], d['rec2_ymix']))
    for rec, (y, ym) in enumerate(states):
        dz = d['rec2_dz'] if rec == 2 else d['rec0_dz']
        if rec == 2:                  # update_mu_dz changed dz by count 100
            atm = b.atm.copy()
            atm[:, ATM_DZ] = dz
            h.set_atm(atm)
        h.set_state(y, ym)
        change = h.photo_update()
        tau_d, af_d, J_d = h.photo_get()
        tau, af, J, ch = _oracle_call(d, y, ym, dz, du, dd, prev)
        prev = af
        assert _rel(tau_d[:nz + 1], tau) < 1e-13
        assert _rel(af_d, af, 1e-30) < 1e-11
        assert _rel(J_d.T, J) < 1e-10
        if rec > 0:
            assert abs(change[0] / ch - 1) < 1e-9
        k = h.k()
        for c, ki in enumerate(d['ch_kindex']):
            np.testing.assert_allclose(k[:, int(ki) - 1], J_d[:, c] * float(d['f_diurnal']), rtol=1e-15)
    h.close()


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['c1rt', 'c1rtT'])
def test_device_run_with_photo_tracks_reference(tag):
    """vk_run with the reference's photochemistry schedule from the c1rt
    (c1rtT: T-dependent cross sections) set-up: J recomputed at count 0
    (twice, as the reference's set-up and its first loop iteration do), the
    state after 100 steps and the J of the update at count 100 against the
    reference's records."""
    from helpers import floor_err
    from test_gpu_parity import make_handle
    from vulcan_gb300 import _build, batch, configs
    from vulcan_gb300.solver import ctrl_from
    _build.build()
    d = _fixture(tag)
    g, net, gn, h, b = make_handle('c1')
    h.set_atom_ini(g['atom_ini'][None, :])
    h.set_clock(dt=1e-10, t=0.0, count=0)
    _attach(h, d, net)
    h.photo_update()                                   # the set-up call
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    st = batch.run_with_photo(h, ctrl, max_steps=100)
    assert st['count'][0] == 100
    assert floor_err(st['y'], d['rec2_y'], g['n_0']) <= 1e-8
    h.photo_update()                                   # the update at count 100
    _, _, J = h.photo_get()
    m = d['rec2_J'] > 1e-300
    assert float(np.max(np.abs(J.T - d['rec2_J'])[m] / d['rec2_J'][m])) <= 1e-6
    h.close()


def test_photo_schedule_follows_the_reference():
    """batch.run_with_photo on a stand-in handle: J before the steps whose
    count is a multiple of update_photo_frq (100, then 5 once longdy < 10
    yconv_min and longdydt < 1e-6), per column."""
    from types import SimpleNamespace
    from vulcan_gb300 import batch

    class FakeHandle:
        def __init__(self):
            self.batch = SimpleNamespace(ncols=2)
            self.count = np.zeros(2, dtype=int)
            self.updates = []

        def state(self):
            return {'count': self.count.copy(), 'end_case': np.where(self.count >= 300, 1, 0)}

        def conv_stats(self):
            # column 1 is near steady state from count 150 on
            ld = np.array([1.0, 1e-3 if self.count[1] >= 150 else 1.0])
            return ld, ld * 1e-9

        def photo_update(self, mask=None):
            self.updates.append((self.count.copy(), np.asarray(mask).copy()))

        def run(self, ctrl, max_steps=0, timeout_s=0.0):
            self.count += max_steps * (self.count < 300)

    h = FakeHandle()
    batch.run_with_photo(h, SimpleNamespace(yconv_min=0.1), max_steps=300)
    col0 = [int(c[0]) for c, m in h.updates if m[0]]
    col1 = [int(c[1]) for c, m in h.updates if m[1]]
    assert col0 == [0, 100, 200]
    assert col1[:2] == [0, 100] and col1[2:] == list(range(150, 300, 5))


def _dropin(d, net, g, use_ion=False):
    """Ros2GPU over a stand-in op module whose own radiative transfer records
    its calls, with the c1 column's set-up arrays as var/atm."""
    import types
    from helpers import column_from_golden
    from vulcan_gb300.solver import make_ros2gpu
    calls = []

    class FakeRos2:
        def compute_tau(self, var, atm):
            calls.append('tau')

        def compute_flux(self, var, atm):
            calls.append('flux')

        def compute_J(self, var, atm):
            calls.append('J')

    op = types.SimpleNamespace(Ros2=FakeRos2)
    cfg = types.SimpleNamespace(
        network=None, use_photo=True, atom_list=[str(a) for a in g['atom_list']],
        use_moldiff=True, use_topflux=False, use_botflux=False,
        T_cross_sp=[str(sp) for sp in d.get('T_cross_sp', [])],
        use_ion=use_ion, scat_sp=[str(s) for s in d['scat_sp']], sl_angle=float(d['sl_angle']),
        edd=float(d['edd']), f_diurnal=float(d['f_diurnal']), flux_atol=float(d['flux_atol']),
        remove_list=[])
    cls = make_ros2gpu(op, cfg, net.species)
    cls._vk_net_cls = types.SimpleNamespace(from_file=lambda path, use_photo: net)
    chans = list(zip([str(s) for s in d['ch_sp']], [int(b) for b in d['ch_br']]))
    absp = [str(s) for s in d['absp_sp']]
    var = types.SimpleNamespace(
        y=d['rec0_y'].copy(), ymix=d['rec0_ymix'].copy(), dt=1e-10,
        k={i: g['k'][i - 1].copy() for i in range(1, net.nr + 1)},
        bins=d['bins'], dbin1=float(d['dbin1']), dbin2=float(d['dbin2']),
        sflux_din12_indx=int(d['sflux_din12_indx']), sflux_top=d['sflux_top'],
        photo_sp=set(str(s) for s in d['photo_sp']),
        pho_rate_index={c: int(ki) for c, ki in zip(chans, d['ch_kindex'])},
        cross={sp: d['cross'][i] for i, sp in enumerate(absp)},
        cross_scat={str(sp): d['cross_scat'][i] for i, sp in enumerate(d['scat_sp'])},
        cross_J={c: d['cross_J'][i] for i, c in enumerate(chans)},
        aflux=np.zeros((d['rec0_y'].shape[0], len(d['bins']))))
    if 'T_cross_sp' in d:
        var.cross_T = {str(sp): d['cross_T'][i] for i, sp in enumerate(d['T_cross_sp'])}
        var.cross_J_T = {(str(sp), int(br)): d['cross_J_T'][i]
                         for i, (sp, br) in enumerate(zip(d['chT_sp'], d['chT_br']))}
    col = column_from_golden(g)
    atm = types.SimpleNamespace(**{k: getattr(col, k) for k in (
        'M', 'n_0', 'Tco', 'g', 'dzi', 'Kzz', 'vz', 'Ti', 'Hpi', 'Hp', 'pico', 'dz', 'Dzz',
        'ms', 'alpha', 'top_flux', 'bot_flux', 'bot_vdep', 'pref_indx')})
    return cls(), var, atm, chans, calls


def test_dropin_radiative_transfer_dispatch():
    """Ros2GPU keeps the reference's own compute_tau / compute_flux /
    compute_J where the device path does not apply (photoionisation);
    otherwise compute_tau and compute_flux leave var alone and the device
    work happens in compute_J."""
    from helpers import golden, network
    d = _fixture()
    s, var, atm, _, calls = _dropin(d, network('c1'), golden('c1'), use_ion=True)
    for f in (s.compute_tau, s.compute_flux, s.compute_J):
        f(var, atm)
    assert calls == ['tau', 'flux', 'J']
    s, var, atm, _, calls = _dropin(d, network('c1'), golden('c1'))
    s.compute_tau(var, atm)
    s.compute_flux(var, atm)
    assert calls == [] and not hasattr(var, 'tau')


@pytest.mark.gpu
@pytest.mark.parametrize('tag', ['c1rt', 'c1rtT'])
def test_dropin_radiative_transfer_matches_reference(tag):
    """Ros2GPU.compute_tau / compute_flux / compute_J in the reference's call
    order on the c1 column: var.tau, var.aflux, var.J_sp and the photolysis
    k against the reference's records of its set-up call and its first
    update (whose aflux_change reads the set-up call's flux).  The absorbers
    are summed in this process's set order, not the recording's, so the
    actinic flux is held to 1e-10 here (1.6e-11 seen); the kernel's own
    parity on identical tables is test_device_radiative_transfer_matches_oracle.
    c1rtT: CO2, H2O and NH3 with the reference's per-layer cross sections."""
    from helpers import golden, network
    from vulcan_gb300 import _build
    _build.build()
    d = _fixture(tag)
    g = golden('c1')
    s, var, atm, chans, calls = _dropin(d, network('c1'), g)
    nz = d['rec0_y'].shape[0]
    for rec in ('rec0', 'rec1'):
        for f in (s.compute_tau, s.compute_flux, s.compute_J):
            f(var, atm)
        if rec == 'rec0':
            assert _rel(var.tau, d['rec0_tau']) < 1e-13
        assert _rel(var.aflux, d[rec + '_aflux'], 1e-30) < 1e-10
        J = np.array([var.J_sp[c] for c in chans])
        assert _rel(J, d[rec + '_J']) < 1e-10
        for c, ki in var.pho_rate_index.items():
            np.testing.assert_array_equal(var.k[ki], var.J_sp[c] * float(d['f_diurnal']))
        for sp in var.photo_sp:
            tot = sum(var.J_sp[c] for c in chans if c[0] == sp)
            np.testing.assert_allclose(var.J_sp[(sp, 0)], tot, rtol=1e-14)
    assert abs(var.aflux_change / float(d['rec1_aflux_change']) - 1) < 1e-9
    assert var.tau.shape == (nz + 1, len(d['bins'])) and calls == []
    s._vk_h.close()


def test_attach_cross_T_checks_shapes_and_slots():
    """photo.attach_cross_T (host side): per-layer tables must be [L, nbins]
    of the handle's batch; absorber and channel slots follow the tables'
    lists (checked on a stand-in library)."""
    import types
    from vulcan_gb300 import capi, photo
    d = _fixture('c1rtT')
    t = photo.PhotoTables.from_fixture(d)
    calls = []

    class FakeLib:
        def vk_photo_set_cross_T(self, *a):
            calls.append(a)
            return 0

    h = types.SimpleNamespace(h=None, photo_tables=t, batch=types.SimpleNamespace(L=150))
    orig_lib, orig_check = capi.lib, capi.check
    capi.lib, capi.check = (lambda: FakeLib()), (lambda rc, hh=None: None)
    try:
        ct = {str(sp): d['cross_T'][i] for i, sp in enumerate(d['T_cross_sp'])}
        cj = {(str(sp), int(br)): d['cross_J_T'][i]
              for i, (sp, br) in enumerate(zip(d['chT_sp'], d['chT_br']))}
        photo.attach_cross_T(h, ct, cj)
        a = calls[-1]
        assert a[1] == 3 and a[4] == 7
        assert [t.absp_sp[a[2][i]] for i in range(a[1])] == list(ct)
        chans = list(zip(t.ch_sp, t.ch_br))
        assert [chans[a[5][i]] for i in range(a[4])] == list(cj)
        with pytest.raises(ValueError):
            photo.attach_cross_T(h, {k: v[:-1] for k, v in ct.items()}, cj)
        photo.attach_cross_T(h, {}, {})                  # removes the tables
        assert calls[-1][1] == 0 and calls[-1][4] == 0
    finally:
        capi.lib, capi.check = orig_lib, orig_check
