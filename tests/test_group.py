"""Several networks in one launch: a group of handles (the 69-species
NCHO-thermo network and the 150-species synthetic network, each with its
own uneven columns) run by one graph per replay.

The group places each handle's kernels on its own stream inside one graph;
the kernels and their inputs are those of the handle's own vk_run, so every
column's state, step count and time must equal, bit for bit, those of the
handle run alone -- for the one-step graph (max_steps = 1) and the
eight-attempt graph, and across repeated calls (graph reuse).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ATOMS = ['H', 'O', 'C', 'He', 'N']
BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), '_build', 'tests')


@pytest.fixture(scope='module')
def nets():
    from conftest import GOLDEN
    from vulcan_gb300 import _build, batch, configs, synthnet
    from vulcan_gb300.network import Network
    _build.build()
    ncho = Network.from_npz(os.path.join(GOLDEN, 'net_NCHO_thermo.npz'))
    items_a = batch.build_items(configs.config2_columns(ncols=3, seed=7, nz_range=(40, 90)), ncho)
    syn = Network.from_file(synthnet.generate(os.path.join(BUILD, 'syn150')), use_photo=True)
    specs = configs.config4_columns(sorted(syn.photo_index()), ncols=2, nz=40)
    items_b = batch.build_items(specs, syn)
    return [(ncho, items_a), (syn, items_b)]


def _handles(nets, precision):
    from vulcan_gb300 import batch
    return [batch.make_batch_handle(net, items, ATOMS, precision) for net, items in nets]


def _snap(h):
    st = h.state()
    return {k: st[k].copy() for k in ('y', 'ymix', 'dt', 't', 'count', 'end_case')}


@pytest.mark.parametrize('precision', [0, 1])
def test_group_matches_each_network_alone(nets, precision):
    from vulcan_gb300 import configs
    from vulcan_gb300.solver import Ros2Group, ctrl_from
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    calls = (1, 20, 20)
    alone = []
    for h, b in _handles(nets, precision):
        snaps = []
        for m in calls:
            h.run(ctrl, max_steps=m, timeout_s=300)
            snaps.append(_snap(h))
        alone.append(snaps)
        h.close()
    hb = _handles(nets, precision)
    g = Ros2Group([h for h, _ in hb])
    together = [[] for _ in hb]
    for m in calls:
        g.run(ctrl, max_steps=m, timeout_s=300)
        for i, (h, _) in enumerate(hb):
            together[i].append(_snap(h))
    ms, launches = g.timing()
    assert ms > 0 and launches > 0
    g.close()
    for h, _ in hb:
        h.close()
    for i in range(len(hb)):
        for call, (a, t) in enumerate(zip(alone[i], together[i])):
            assert (t['count'] >= 1).all()
            for k in a:
                np.testing.assert_array_equal(a[k], t[k], err_msg='network %d call %d %s' % (i, call, k))
