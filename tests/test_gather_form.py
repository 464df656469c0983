"""The compiled network's gather form (vk_network.cpp) -- what the rate
kernel k_rates evaluates, one FP64 instruction per gathered term -- checked
on the CPU through vk_network_eval_host, which runs the same tables with the
kernel's operations and order.  Against the oracle (itself pinned bit for bit
to the reference's generated chemdf and to its sympy Jacobian): the chemical
source is bit-identical and the -J entries agree to 1e-14 of the block's
largest entry, on every shipped-network fixture (CHO, NCHO thermo and
photo, the 89-species sulfur network) and the 150-species synthetic stress
network, at random states spanning the mixing-ratio range of a column."""
import ctypes as C
import os

import numpy as np
import pytest

from helpers import GOLDEN
from oracle import ros2 as O

NETS = [('CHO_thermo', ['H', 'O', 'C', 'He']), ('NCHO_thermo', ['H', 'O', 'C', 'He', 'N']),
        ('NCHO_photo', ['H', 'O', 'C', 'He', 'N']), ('SNCHO_photo', ['H', 'O', 'C', 'He', 'N', 'S'])]


def _eval(lib, gn, net, y, k, M):
    f = np.zeros(net.ni)
    jv = np.zeros(gn.nnz)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.vk_network_eval_host(gn.handle, p(y), p(k), M, p(f), p(jv)) == 0
    rows, cols = gn.jac_pattern()
    J = np.zeros((net.ni, net.ni))
    J[rows, cols] = jv
    return f, J


def _check(lib, net, on, gn, seed):
    rng = np.random.default_rng(seed)
    for _ in range(3):
        y = 10.0 ** rng.uniform(-5, 19, net.ni)
        y[rng.random(net.ni) < 0.2] = 0.0              # absent species
        k = 10.0 ** rng.uniform(-35, -5, net.nr)
        M = float(10.0 ** rng.uniform(14, 20))
        f, J = _eval(lib, gn, net, y, k, M)
        fo = O.chemdf(on, y[None, :], np.array([M]), k[:, None])[0]
        Jo = O.neg_jac_blocks(on, y[None, :], np.array([M]), k[:, None])[0]
        np.testing.assert_array_equal(f, fo)
        assert np.abs(J - Jo).max() <= 1e-14 * np.abs(Jo).max()


@pytest.mark.parametrize('name,atoms', NETS)
def test_gather_form_matches_oracle(name, atoms):
    from vulcan_gb300 import _build, capi
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import GPUNetwork
    _build.build()
    path = os.path.join(GOLDEN, 'net_%s.npz' % name)
    net = Network.from_npz(path)
    _check(capi.lib(), net, O.OracleNet.from_npz(path, atoms), GPUNetwork(net, atoms), 1)


def test_gather_form_synthetic_150_species(tmp_path):
    from vulcan_gb300 import _build, capi, synthnet
    from vulcan_gb300.network import Network
    from vulcan_gb300.solver import GPUNetwork
    _build.build()
    net = Network.from_file(synthnet.generate(str(tmp_path / 'syn150')), use_photo=True)
    on = O.OracleNet(list(net.species), [(r.reac, r.prod) for r in net.reactions],
                     np.zeros((net.ni, 1)), np.zeros(net.ni))
    _check(capi.lib(), net, on, GPUNetwork(net, list(synthnet.ATOMS)), 2)
