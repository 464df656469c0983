"""Device chemistry and Ros2 attempts on the reference's 89-species sulfur
network: the chemical source equals the reference's generated chemdf bit for
bit at a seeded positive state (fixture snchok), and the attempts match the
reference's recorded ones (fixture c3s)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_sulfur_network_chemical_source_bit_exact():
    import dataclasses
    from vulcan_gb300 import _build, batch, configs
    from vulcan_gb300.network import Network
    _build.build()
    g = np.load(os.path.join(GOLDEN, 'golden_snchok.npz'))
    net = Network.from_npz(os.path.join(GOLDEN, 'net_SNCHO_photo.npz'))
    atoms = ['H', 'O', 'C', 'He', 'N', 'S']
    spec = dataclasses.replace(configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0],
                               const_mix={'H2': 0.85, 'He': 0.15}, atom_list=atoms)
    items = batch.build_items([spec], net)
    # the fixture's own M and k: the seeded column is rebuilt with numpy's
    # exp/log, whose last bit differs between x86 and Arm builds of numpy,
    # and a one-ulp change of M moves every termolecular rate by an ulp
    items[0]['col'].M = g['M'].copy()
    items[0]['k'] = g['k']
    h, b = batch.make_batch_handle(net, items, atoms)
    np.testing.assert_array_equal(h.chem_source(g['y_rand']), g['chemdf_rand'])
    h.close()


@pytest.mark.parametrize('precision', [0, 1])
def test_sulfur_network_attempts_match_reference(precision):
    """Device Ros2 attempts on the sulfur network against the reference's
    recorded attempts (fixture c3s), FP64 and mixed."""
    from helpers import column_from_golden, floor_err, golden, network
    from vulcan_gb300 import _build
    from vulcan_gb300.solver import ColumnBatch, GPUNetwork, Ros2Handle
    _build.build()
    g = golden('c3s')
    net = network('c3s')
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    items = [dict(col=column_from_golden(g, n), k=g['k'], y=g['att_y'][n], ymix=g['att_ymix'][n])
             for n in range(len(g['att_index']))]
    b = ColumnBatch(items, net.ni)
    h = Ros2Handle(gn, len(items), b.L, precision)
    h.set_columns(b)
    out = h.attempt(g['att_dt'])
    sols = b.split(out['sol'])
    for n in range(len(items)):
        assert floor_err(sols[n], g['att_sol'][n], g['n_0']) <= 1e-10, n
        assert abs(out['delta'][n] / g['att_delta'][n] - 1) <= 1e-6, n
    h.close()
