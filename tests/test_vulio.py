"""`.vul` output / `vulcan_ini` restart (the reference's save_out layout)."""
import os
import pickle

import numpy as np

from helpers import network
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
