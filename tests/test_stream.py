"""Continuous batching on the device: the slotted layout and vk_refill.

A column's arithmetic never depends on the other columns of its batch (the
per-layer kernels read its own layers, the per-column kernels take whole
columns from a work queue), so a column must give the same bits whether it
sits packed, in a slot of a larger layout, or arrives later in a slot that
another column has left.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from vulcan_gb300 import _build
    _build.build()


def _items(n, seed=2, nz_range=(40, 90)):
    from vulcan_gb300 import batch, configs
    from vulcan_gb300.network import Network
    import os
    from conftest import GOLDEN
    net = Network.from_npz(os.path.join(GOLDEN, 'net_NCHO_thermo.npz'))
    specs = configs.config2_columns(ncols=n, seed=seed, nz_range=nz_range)
    return net, batch.build_items(specs, net)


ATOMS = ['H', 'O', 'C', 'He', 'N']


@pytest.mark.parametrize('precision', [0, 1])
def test_slotted_layout_matches_packed(precision):
    """Attempts and a 30-step run give the same bits in the packed and the
    slotted layout."""
    from vulcan_gb300 import batch, configs
    from vulcan_gb300.solver import ctrl_from
    net, items = _items(4)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    outs = []
    for cap in (0, 100):
        h, b = batch.make_batch_handle(net, items, ATOMS, precision, slot_cap=cap)
        a = h.attempt(np.full(b.ncols, 1e-8))
        h.run(ctrl, max_steps=30, timeout_s=300)
        st = h.state()
        outs.append((b.split(a['sol']), b.split(st['y']), st['count'].copy(), st['t'].copy()))
        h.close()
    (s0, y0, c0, t0), (s1, y1, c1, t1) = outs
    for c in range(len(items)):
        np.testing.assert_array_equal(s0[c], s1[c])
        np.testing.assert_array_equal(y0[c], y1[c])
    np.testing.assert_array_equal(c0, c1)
    np.testing.assert_array_equal(t0, t1)


@pytest.mark.parametrize('precision,chunk_attempts', [(0, None), (1, None), (0, 16), (1, 16)])
def test_refilled_column_runs_as_in_its_own_batch(precision, chunk_attempts):
    """Three columns through two slots (count_max 60, so the first two end
    together and the third is refilled into a slot they left): every column's
    final state, step count and time equal those of the column alone -- with
    refills every 20 steps, and every 16 attempts of the batch
    (vk_run_budget: a run that stops mid-step resumes exactly)."""
    from vulcan_gb300 import batch, configs
    from vulcan_gb300.solver import ctrl_from
    net, items = _items(3, seed=5)
    ctrl = ctrl_from(None, gs=configs.GS, Rp=configs.RP)
    ctrl.count_max = 60
    res, wall = batch.run_stream(net, items, ATOMS, nslots=2, ctrl=ctrl, precision=precision,
                                 slot_cap=100, chunk=20, keep_state=True,
                                 chunk_attempts=chunk_attempts)
    assert sorted(res) == [0, 1, 2]
    for i, it in enumerate(items):
        h, b = batch.make_batch_handle(net, [it], ATOMS, precision)
        h.run(ctrl, max_steps=1000, timeout_s=300)
        st = h.state()
        h.close()
        r = res[i]
        assert r['end_case'] == st['end_case'][0] == 3
        assert r['count'] == st['count'][0]
        assert r['t'] == st['t'][0]
        np.testing.assert_array_equal(r['y'], st['y'])


def test_refill_rejects_bad_slots():
    from vulcan_gb300 import batch, capi
    net, items = _items(3)
    h, b = batch.make_batch_handle(net, items[:2], ATOMS, 0, slot_cap=100)
    with pytest.raises(capi.VkError):
        h.refill([5], items[2:], np.stack([items[2]['atom_ini']]))      # no such slot
    with pytest.raises(capi.VkError):
        h.refill([0, 0], items[1:], np.stack([it['atom_ini'] for it in items[1:]]))   # repeated
    h.close()
    h, b = batch.make_batch_handle(net, items[:2], ATOMS, 0)            # packed layout
    with pytest.raises(capi.VkError):
        h.refill([0], items[2:], np.stack([items[2]['atom_ini']]))
    h.close()
