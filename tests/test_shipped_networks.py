"""Every network file the reference ships that its own set-up can use (15 of
17; CHO, NCHO, SNCHO and TiSNCHO families, 38-99 species, up to 1 284 rate
slots), pinned to the reference itself: fixtures n_<network> record its
species order, rate constants (read_rate, rev_rate), and its generated
chemistry source (chemdf) and sympy Jacobian (neg_symjac) at a seeded
positive state with seeded J in the photolysis slots
(tests/golden/make_golden.py).

Checked here, on the CPU: this package's parser gives the reference's
species order and rate slots; its host rate constants are bit-identical; the
oracle's chemdf is bit-identical and its -J within 1e-14 of the block scale;
and the device tables' gather form -- what the rate kernel evaluates,
operations and order included, run on the host by vk_network_eval_host --
gives the reference's chemdf bit for bit on every layer and its -J within
1e-14."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import ros2 as O

TAGS = sorted(os.path.basename(f)[7:-4] for f in glob.glob(os.path.join(GOLDEN, 'golden_n_*.npz')))


def _load(tag):
    from vulcan_gb300.network import Network
    g = dict(np.load(os.path.join(GOLDEN, 'golden_%s.npz' % tag), allow_pickle=False))
    path = os.path.join(GOLDEN, 'net_%s.npz' % tag[2:])
    return g, path, Network.from_npz(path), [str(a) for a in g['atom_list']]


def test_every_usable_shipped_network_has_a_fixture():
    assert len(TAGS) == 15


@pytest.mark.parametrize('tag', TAGS)
def test_species_and_rate_constants(tag):
    g, path, net, atoms = _load(tag)
    assert [str(s) for s in g['spec_list']] == list(net.species)
    assert int(g['nr']) == net.nr
    photo = np.zeros(net.nr, dtype=bool)
    for idx in net.photo_index().values():
        photo[idx - 1] = True
    with np.errstate(over='ignore'):
        k = net.rate_constants(g['Tco'], g['M'])
    np.testing.assert_array_equal(k[~photo], g['k'][~photo])


@pytest.mark.parametrize('tag', TAGS)
def test_oracle_chemistry(tag):
    g, path, net, atoms = _load(tag)
    on = O.OracleNet.from_npz(path, atoms)
    np.testing.assert_array_equal(O.chemdf(on, g['y_rand'], g['M'], g['k']), g['chemdf_rand'])
    J = O.neg_jac_blocks(on, g['y_rand'], g['M'], g['k'])
    for i, l in enumerate(g['negjac_layers']):
        ref = g['negjac_blocks'][i]
        assert np.abs(J[l] - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize('tag', TAGS)
def test_device_tables_gather_form(tag):
    from vulcan_gb300 import _build, capi
    from vulcan_gb300.solver import GPUNetwork
    _build.build()
    g, path, net, atoms = _load(tag)
    gn = GPUNetwork(net, atoms)
    rows, cols = gn.jac_pattern()
    lib = capi.lib()
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    layers = list(g['negjac_layers'])
    for l in range(g['y_rand'].shape[0]):
        y = np.ascontiguousarray(g['y_rand'][l])
        k = np.ascontiguousarray(g['k'][:, l])
        f, jv = np.zeros(net.ni), np.zeros(gn.nnz)
        assert lib.vk_network_eval_host(gn.handle, p(y), p(k), float(g['M'][l]), p(f), p(jv)) == 0
        np.testing.assert_array_equal(f, g['chemdf_rand'][l], err_msg='layer %d' % l)
        if l in layers:
            ref = g['negjac_blocks'][layers.index(l)]
            J = np.zeros((net.ni, net.ni))
            J[rows, cols] = jv
            assert np.abs(J - ref).max() <= 1e-14 * np.abs(ref).max(), 'layer %d' % l
