"""`.vul` output / `vulcan_ini` restart (the reference's save_out layout)."""
import os
import pickle

import numpy as np

from helpers import GOLDEN, network
from vulcan_gb300 import batch, configs, vulio

ATOMS = ['H', 'O', 'C', 'He', 'N']
BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), '_build', 'tests')


def test_write_read_round_trip():
    net = network('c2')
    specs = configs.config2_columns(ncols=2, seed=3, nz_range=(40, 50))
    items = batch.build_items(specs, net)
    L = sum(it['col'].nz for it in items)
    rng = np.random.default_rng(0)
    y = np.concatenate([it['y'] for it in items]) * (1 + 0.1 * rng.random((L, net.ni)))
    ymix = y / y.sum(axis=1, keepdims=True)
    state = dict(y=y, ymix=ymix, t=np.array([1e9, 2e9]), dt=np.array([1e7, 2e7]),
                 count=np.array([900, 1100], dtype=np.int32), end_case=np.array([1, 3], dtype=np.int32),
                 delta=np.array([0.1, 0.2]))
    os.makedirs(BUILD, exist_ok=True)
    paths = [os.path.join(BUILD, 'col%d.vul' % c) for c in range(2)]
    vulio.write_batch(paths, net, items, state, ATOMS)
    with open(paths[1], 'rb') as f:
        d = pickle.load(f)
    v = d['variable']
    assert set(d) == {'variable', 'atm', 'parameter'}
    assert v['species'] == net.species and v['nr'] == net.nr
    nz0 = items[0]['col'].nz
    np.testing.assert_array_equal(v['ymix'], ymix[nz0:])
    np.testing.assert_array_equal(v['k'][1], items[1]['k'][0])
    assert v['Rf'][1] == net.reactions[0].text
    assert d['parameter']['end_case'] == 3 and d['parameter']['count'] == 1100
    np.testing.assert_array_equal(d['atm']['pco'], items[1]['col'].pco)
    assert abs(v['atom_loss']['H']) < 0.2
    # restart (ini_mix = 'vulcan_ini'): by species name, into another order
    order = list(reversed(net.species)) + ['XYZ']
    yr, missing = vulio.read_vul_y(paths[1], order, nz=items[1]['col'].nz)
    assert missing == ['XYZ']
    np.testing.assert_array_equal(yr[:, :-1], y[nz0:][:, ::-1])
    np.testing.assert_array_equal(yr[:, -1], 0.0)


# what the reference saves (store.py:83-86) and what its plot_py scripts read
REF_VAR_SAVE = ['k', 'y', 'ymix', 'y_ini', 't', 'dt', 'longdy', 'longdydt', 'atom_ini',
                'atom_sum', 'atom_loss', 'atom_conden', 'aflux_change', 'Rf']
REF_PHOTO_SAVE = ['nbin', 'bins', 'dbin1', 'dbin2', 'tau', 'sflux', 'aflux', 'cross',
                  'cross_scat', 'cross_J', 'J_sp', 'n_branch']
PLOT_ATM = ['pco', 'zco', 'zmco', 'pico', 'dz', 'Tco', 'Kzz']
PLOT_VAR = ['species', 'ymix', 'y', 'y_ini']
PLOT_VAR_PHOTO = ['bins', 'cross_scat', 'aflux', 'cross', 'tau']


def test_layout_has_what_the_reference_saves_and_plots():
    from conftest import GOLDEN
    from vulcan_gb300 import photo
    net = network('c2')
    specs = configs.config2_columns(ncols=2, seed=3, nz_range=(40, 50))
    items = batch.build_items(specs, net)
    L = sum(it['col'].nz for it in items)
    y = np.concatenate([it['y'] for it in items])
    state = dict(y=y, ymix=y / y.sum(axis=1, keepdims=True), t=np.ones(2), dt=np.ones(2),
                 count=np.ones(2, dtype=np.int32), end_case=np.ones(2, dtype=np.int32),
                 delta=np.zeros(2))
    tables = photo.PhotoTables.from_fixture(dict(np.load(os.path.join(GOLDEN, 'golden_c1rt.npz'))))
    nb, nch = len(tables.bins), len(tables.ch_sp)
    rng = np.random.default_rng(1)
    tau, aflux, J = rng.random((L + 2, nb)), rng.random((L, nb)), rng.random((L, nch))
    os.makedirs(BUILD, exist_ok=True)
    paths = [os.path.join(BUILD, 'ph%d.vul' % c) for c in range(2)]
    vulio.write_batch(paths, net, items, state, ATOMS, photo=(tables, tau, aflux, J))
    with open(paths[1], 'rb') as f:
        d = pickle.load(f)
    v, atm = d['variable'], d['atm']
    for key in REF_VAR_SAVE + REF_PHOTO_SAVE + PLOT_VAR + PLOT_VAR_PHOTO:
        assert key in v, key
    for key in PLOT_ATM:
        assert key in atm, key
    nz0, nz1 = items[0]['col'].nz, items[1]['col'].nz
    # staggered rows of the second column start at nz0 + 1
    np.testing.assert_array_equal(v['tau'], tau[nz0 + 1:nz0 + 1 + nz1 + 1])
    np.testing.assert_array_equal(v['aflux'], aflux[nz0:])
    ch = list(zip(tables.ch_sp, tables.ch_br))
    sp, br = ch[0]
    np.testing.assert_array_equal(v['J_sp'][(sp, br)], J[nz0:, 0])
    tot = sum(J[nz0:, i] for i, c in enumerate(ch) if c[0] == sp)
    np.testing.assert_allclose(v['J_sp'][(sp, 0)], tot, rtol=1e-14)
    np.testing.assert_allclose(atm['zmco'], 0.5 * (atm['zco'][:-1] + atm['zco'][1:]))
    assert atm['zmco'].size == nz1


def test_matches_a_file_the_reference_wrote():
    """golden_c0vul.vul is the reference's own save_out (op.py:3216-3256) after
    20 steps of config 0 (tests/golden/make_golden.py c0vul).  Written from
    the same state, this package's file has every variable and atm entry of
    the reference's, with the same set-up arrays, rate constants, reaction
    texts and initial state; its parameter entries are a subset of the
    reference's (the run-internal ones it does not track -- nega_y, small_y,
    pic_count, where_varies_most, start_time, the plot palette -- are left
    out); and the reference's file restarts a run (vulcan_ini) through
    read_vul_y.  The column geometry that diffusion updates (mu, g, Hp, dz,
    zco, zmco, dzi: update_mu_dz every update_frq steps, the first time after
    step 1) is the reference's at its last update and the column item's here
    (the set-up): they agree to the drift of one step, 1e-5."""
    g = dict(np.load(os.path.join(GOLDEN, 'golden_c0vul.npz'), allow_pickle=False))
    with open(os.path.join(GOLDEN, 'golden_c0vul.vul'), 'rb') as f:
        ref = pickle.load(f)
    net = network('c0')
    atoms = [str(a) for a in g['atom_list']]
    item = batch.build_items([configs.config0()], net)[0]
    ours = vulio.vul_dict(net, item, g['final_y'], g['final_ymix'], float(g['final_t']), 1e-9,
                          int(g['final_count']), int(g['end_case']), atoms,
                          counters=np.array([26, 6, 0, 0, 0, 20]))
    rv, ov = ref['variable'], ours['variable']
    assert set(rv) <= set(ov)
    assert set(ref['atm']) <= set(ours['atm'])
    assert set(ours['parameter']) <= set(ref['parameter'])
    assert ov['species'] == list(rv['species']) and ov['nr'] == rv['nr']
    assert ov['Rf'] == rv['Rf']
    assert set(ov['k']) == set(rv['k'])
    for i in rv['k']:
        np.testing.assert_array_equal(ov['k'][i], rv['k'][i])
    np.testing.assert_array_equal(ov['y_ini'], rv['y_ini'])
    for a in atoms:
        assert abs(ov['atom_ini'][a] / rv['atom_ini'][a] - 1) < 1e-12
        assert ov['atom_conden'][a] == rv['atom_conden'][a] == 0.0
    for key in ('pco', 'pico', 'Tco', 'Kzz', 'M', 'n_0', 'Dzz', 'Dzz_cen', 'ms', 'alpha', 'Ti',
                'top_flux', 'bot_flux', 'bot_vdep', 'vz', 'vm', 'vs', 'bot_fix_sp'):
        np.testing.assert_allclose(np.asarray(ours['atm'][key], float),
                                   np.asarray(ref['atm'][key], float), rtol=1e-13, atol=0, err_msg=key)
    for key in ('mu', 'g', 'Hp', 'dz', 'zco', 'zmco', 'dzi', 'Hpi'):
        o, r = np.asarray(ours['atm'][key], float), np.asarray(ref['atm'][key], float)
        assert o.shape == r.shape, key
        assert np.abs(o - r).max() <= 1e-5 * np.abs(r).max(), key
    assert ours['atm']['pref_indx'] == ref['atm']['pref_indx']
    assert ours['atm']['gs'] == ref['atm']['gs']
    assert list(ours['atm']['gas_indx']) == list(ref['atm']['gas_indx'])
    for key in vulio.CONDENSE_DICT_KEYS:
        assert ours['atm'][key] == ref['atm'][key] == {}
    p = ref['parameter']
    assert ours['parameter']['count'] == p['count'] and ours['parameter']['end_case'] == p['end_case']
    assert ours['parameter']['delta_count'] == p['delta_count']
    # the reference's file as a restart: its y by species name
    y, missing = vulio.read_vul_y(os.path.join(GOLDEN, 'golden_c0vul.vul'), net.species)
    assert not missing
    np.testing.assert_array_equal(y, rv['y'])
