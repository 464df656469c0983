"""Launch autotuner: search logic and cache on a stand-in handle (CPU); the
launch settings themselves on the device (GPU test in
tests/test_launch_tuning.py)."""
import pytest

from vulcan_gb300 import autotune, capi


class FakeHandle:
    """Attempt time = 10 ms + a per-kernel cost of its (ctas, variant); the
    cheapest settings are known."""

    def __init__(self, ni, cost):
        self.ni = ni
        self.cost = cost
        self.launch = {}
        self.calls = 0

    def set_launch(self, kernel, ctas_per_sm=0, variant=-1):
        if kernel == capi.VK_TUNE_LU32 and variant != -1 and \
                capi.LU32_TILING_CAP[variant] < self.ni:
            raise capi.VkError(capi.VK_EINVAL, 'tiling too small')
        self.launch[kernel] = (ctas_per_sm, variant)

    def attempt(self, dt, flags=capi.VK_F_MOLDIFF):
        self.calls += 1

    def timing(self):
        ms = 10.0 + sum(self.cost(k, *v) for k, v in self.launch.items())
        return dict(rates=1.0, lu=ms - 3.0, solve=1.5, stage=0.5, launches=12)


def _cost(kernel, ctas, variant):
    best = {capi.VK_TUNE_LU32: (2, 2), capi.VK_TUNE_REFINE: (4, -1),
            capi.VK_TUNE_LU64: (1, -1), capi.VK_TUNE_SWEEP64: (3, -1)}[kernel]
    if ctas == 0:                     # the built-in default sits in the middle
        return 1.0
    return 0.3 * abs(ctas - best[0]) + (0.2 * abs(variant - best[1]) if variant >= 0 else 0.0)


def test_candidates_cover_ni():
    assert autotune.candidates('lu32', 69) == [(c, t) for t in (1, 2, 3, 4, 5) for c in (1, 2, 3, 4)]
    assert [t for _, t in autotune.candidates('lu32', 150)] == [3] * 4
    assert autotune.candidates('lu64', 69) == [(1, -1), (2, -1), (3, -1), (4, -1)]


def test_tune_finds_the_cheapest_settings():
    h = FakeHandle(69, _cost)
    res = autotune.tune(h, 1e-3, precision=capi.VK_PREC_MIXED, repeats=1)
    assert res['lu32'] == (2, 2) and res['refine'] == (4, -1)
    assert res['lu64'] == (1, -1) and res['sweep64'] == (3, -1)
    assert res['_ms'] == pytest.approx(10.0) and res['_default_ms'] == pytest.approx(14.0)
    # the winners stay applied on the handle
    assert h.launch[capi.VK_TUNE_LU32] == (2, 2)


def test_fp64_path_tunes_only_its_kernels():
    h = FakeHandle(69, _cost)
    res = autotune.tune(h, 1e-3, precision=capi.VK_PREC_FP64, repeats=1)
    assert set(k for k in res if not k.startswith('_')) == {'lu64', 'sweep64'}


def test_default_kept_when_nothing_is_faster():
    h = FakeHandle(69, lambda k, c, v: 0.0 if c == 0 else 1.0)
    res = autotune.tune(h, 1e-3, repeats=1)
    assert all(res[k] == (0, -1) for k in ('lu32', 'refine', 'lu64', 'sweep64'))


def test_cache_roundtrip(tmp_path):
    path = str(tmp_path / 'tuning.json')
    key = autotune.cache_key('GB300', 69, 512, capi.VK_PREC_MIXED)
    assert autotune.load(path, key) is None
    settings = {'lu32': (2, 1), 'refine': (3, -1), '_ms': 12.5}
    autotune.save(path, key, settings)
    autotune.save(path, autotune.cache_key('GB300', 150, 128, 1), {'lu32': (1, 3)})
    got = autotune.load(path, key)
    assert got['lu32'] == (2, 1) and got['refine'] == (3, -1) and got['_ms'] == 12.5
    h = FakeHandle(69, _cost)
    autotune.apply(h, got)
    assert h.launch == {capi.VK_TUNE_LU32: (2, 1), capi.VK_TUNE_REFINE: (3, -1)}
