"""Rate constants on the device (vk_compute_k) against the host restatement
of the reference's read_rate / rev_rate (network.Network.rate_constants)."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, network
from vulcan_gb300 import batch, configs, synthnet
from vulcan_gb300.network import Network

pytestmark = pytest.mark.gpu
ATOMS = ['H', 'O', 'C', 'He', 'N']


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


def _check(net, specs, atoms):
    items = batch.build_items(specs, net)
    h, b = batch.make_batch_handle(net, items, atoms)
    host = np.concatenate([it['k'].T for it in items])           # [L, nr]
    h.set_rate_params(net)
    h.compute_k()
    dev = h.k()
    h.close()
    # exp / pow / log of two math libraries: a few ulp, more where exp's
    # argument is large (reverse rates through Keq = exp(-dg))
    np.testing.assert_allclose(dev, host, rtol=2e-12, atol=1e-290)
    return items, dev


def test_thermo_network_columns_of_different_temperature():
    net = network('c2')
    _check(net, configs.config2_columns(ncols=6, seed=5, nz_range=(30, 60)), ATOMS)


def test_special_and_photo_slots():
    """NCHO photo network: the OH + CH3 + M pressure-dependent form, and the
    photolysis forward slots keep the uploaded frozen J."""
    net = Network.from_npz(os.path.join(GOLDEN, 'net_NCHO_photo.npz'))
    spec = configs.config1(sorted(net.photo_index()), nz=40)
    items, dev = _check(net, [spec], ATOMS)
    pidx = net.photo_index()
    for key, J in spec.photo_J.items():
        np.testing.assert_array_equal(dev[:, pidx[key] - 1], J)


def test_synthetic_150_species():
    d = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), '_build', 'tests', 'syn150')
    net = Network.from_file(synthnet.generate(d), use_photo=True)
    _check(net, configs.config4_columns(sorted(net.photo_index()), ncols=2, nz=40), ATOMS)


def test_low_temperature_caps():
    """use_lowT_limit_rates on a 150-450 K column: the device against the
    host restatement (itself bit-exact to the reference, fixture lowT), and
    the caps removed again give the plain rates."""
    from helpers import golden
    g = golden('lowT')
    net = network('c2')
    spec = configs.config2_columns(ncols=1, seed=2, nz_range=(40, 40))[0]
    spec.Tco = g['Tco'].copy()
    items = batch.build_items([spec], net)
    h, b = batch.make_batch_handle(net, items, ATOMS)
    from vulcan_gb300.capi import ATM_M, ATM_TCO
    np.testing.assert_array_equal(b.atm[:, ATM_TCO], g['Tco'])
    M = b.atm[:, ATM_M]
    np.testing.assert_allclose(M, g['M'], rtol=1e-15)
    h.set_rate_params(net, use_lowT_limit_rates=True)
    h.compute_k()
    capped = h.k()
    h.set_rate_params(net)
    h.compute_k()
    plain = h.k()
    h.close()
    host_c = net.rate_constants(g['Tco'], M, use_lowT_limit_rates=True).T
    host_p = net.rate_constants(g['Tco'], M).T
    np.testing.assert_allclose(capped, host_c, rtol=2e-12, atol=1e-290)
    np.testing.assert_allclose(plain, host_p, rtol=2e-12, atol=1e-290)
    assert np.any(np.abs(capped - plain) > 1e-3 * np.abs(plain))
