"""Host logic of continuous batching (batch.run_stream) on the CPU, with a
stand-in for the device handle: every item ends exactly once, an ended slot
takes the next item in order, results are keyed by item, the attempt budget
is passed through, and the step / attempt statistics add up.  The device
side of the same loop (slotted layout, vk_refill, vk_run_budget) is checked
bit for bit in tests/test_stream.py on the GPU."""
import types

import numpy as np
import pytest

from vulcan_gb300 import batch, capi


class FakeBatch:
    def __init__(self, ncols, slot_cap, ni):
        self.ncols = ncols
        self.off = np.arange(ncols) * slot_cap
        self.end = self.off + slot_cap
        self.L = ncols * slot_cap
        self.ni = ni


class FakeHandle:
    """Each slot holds an item that ends after `need` accepted steps (two
    attempts per step); a run advances every live slot by `max_steps` steps,
    or by max_attempts // 2 steps under an attempt budget."""

    def __init__(self, items, slot_cap, ni, log):
        self.b = FakeBatch(len(items), slot_cap, ni)
        self.ni = ni
        self.log = log
        self.need = [it['need'] for it in items]
        self.count = np.zeros(len(items), dtype=np.int32)
        self.att = np.zeros(len(items), dtype=np.int32)
        self.end_case = np.zeros(len(items), dtype=np.int32)
        self.tag = [it['tag'] for it in items]
        self.closed = False
        self.route = None

    def set_route(self, dt0):
        self.route = dt0

    def run(self, ctrl, max_steps=0, timeout_s=0.0, max_attempts=0):
        self.log.append(('run', max_steps, max_attempts))
        adv = max_attempts // 2 if max_attempts else max_steps
        for c in range(self.b.ncols):
            if self.end_case[c] == 0 and self.need[c] is not None:
                take = min(adv, self.need[c] - self.count[c])
                self.count[c] += take
                self.att[c] += 2 * take
                if self.count[c] >= self.need[c]:
                    self.end_case[c] = 1

    def timing(self):
        return dict(rates=5.0, lu=0.0, solve=0.0, stage=0.0, launches=0)

    def state(self):
        L, ni = self.b.L, self.ni
        y = np.zeros((L, ni))
        for c in range(self.b.ncols):            # the slot's layers carry its item's tag
            y[self.b.off[c]:self.b.end[c]] = self.tag[c]
        return dict(end_case=self.end_case.copy(), count=self.count.copy(),
                    t=self.count.astype(float), y=y, ymix=y.copy())

    def counters(self):
        c = np.zeros((self.b.ncols, capi.NCOUNTERS), dtype=np.int32)
        c[:, 0] = self.att
        return c

    def refill(self, slots, nitems, atom_ini, masks):
        assert len(slots) == len(nitems) == atom_ini.shape[0] == masks.shape[0]
        self.log.append(('refill', list(slots), [it['tag'] for it in nitems]))
        for c, it in zip(slots, nitems):
            assert self.end_case[c] != 0              # only ended slots are refilled
            self.need[c] = it['need']
            self.tag[c] = it['tag']
            self.count[c] = 0
            self.att[c] = 0
            self.end_case[c] = 0

    def close(self):
        self.closed = True


def _items(needs):
    col = types.SimpleNamespace(nz=4)
    return [dict(col=col, atom_ini=np.ones(2), ignore=[], need=n, tag=i)
            for i, n in enumerate(needs)]


@pytest.fixture
def fake(monkeypatch):
    log, made = [], []

    def make(net, items, atom_list, precision=0, slot_cap=0):
        h = FakeHandle(items, slot_cap, net.ni, log)
        made.append(h)
        return h, h.b

    monkeypatch.setattr(batch, 'make_batch_handle', make)
    return log, made


NET = types.SimpleNamespace(ni=3, species=['A', 'B', 'C'])


@pytest.mark.parametrize('chunk_attempts', [None, 8])
def test_every_item_ends_once_in_order(fake, chunk_attempts):
    log, made = fake
    needs = [3, 9, 4, 2, 7, 5, 1]
    stats = {}
    res, wall = batch.run_stream(NET, _items(needs), ['H', 'O'], nslots=3, ctrl=None,
                                 chunk=2, keep_state=True, stats=stats,
                                 chunk_attempts=chunk_attempts)
    assert sorted(res) == list(range(len(needs)))
    for i, n in enumerate(needs):
        assert res[i]['end_case'] == 1
        assert res[i]['count'] == n                  # its own steps, from its own start
        assert np.all(res[i]['y'] == i)               # the state read from its own slot
    # refills hand out the items in order, each to a slot that had just ended
    handed = [t for e in log if e[0] == 'refill' for t in e[2]]
    assert handed == list(range(3, len(needs)))
    assert stats['steps'] == sum(needs)
    assert stats['attempts'] == 2 * sum(needs)
    runs = [e for e in log if e[0] == 'run']
    if chunk_attempts:
        assert all(e[1] == 0 and e[2] == chunk_attempts for e in runs)
    else:
        assert all(e[1] == 2 and e[2] == 0 for e in runs)
    assert stats['device_s'] == pytest.approx(5e-3 * len(runs))
    assert made[0].closed


def test_fewer_items_than_slots(fake):
    log, made = fake
    res, _ = batch.run_stream(NET, _items([2, 3]), ['H'], nslots=4, ctrl=None, chunk=1)
    assert sorted(res) == [0, 1]
    assert not [e for e in log if e[0] == 'refill']
    assert made[0].b.ncols == 2


def test_budget_stops_with_live_slots_counted(fake):
    """A zero wall budget stops before the first run; the statistics then
    count the live slots' (zero) steps rather than failing."""
    log, made = fake
    stats = {}
    res, _ = batch.run_stream(NET, _items([5, 5, 5]), ['H'], nslots=2, ctrl=None, chunk=1,
                              budget_s=0.0, stats=stats)
    assert res == {}
    assert stats['steps'] == 0 and stats['attempts'] == 0
    assert not [e for e in log if e[0] == 'run']
    assert made[0].closed


def test_route_only_for_mixed(fake):
    log, made = fake
    batch.run_stream(NET, _items([1]), ['H'], nslots=1, ctrl=None, chunk=1, route_dt0=1e-6,
                     precision=capi.VK_PREC_FP64)
    batch.run_stream(NET, _items([1]), ['H'], nslots=1, ctrl=None, chunk=1, route_dt0=1e-6,
                     precision=capi.VK_PREC_MIXED)
    assert made[0].route is None and made[1].route == 1e-6
