"""Device chemistry on the reference's 89-species sulfur network: the
chemical source equals the reference's generated chemdf bit for bit at a
seeded positive state (fixture snchok)."""
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
    items[0]['k'] = g['k']
    h, b = batch.make_batch_handle(net, items, atoms)
    np.testing.assert_array_equal(h.chem_source(g['y_rand']), g['chemdf_rand'])
    h.close()
