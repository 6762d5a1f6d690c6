"""The schedule autotuner's selection and cache logic, on a fake pipeline
whose frame time depends on the schedule (no GPU)."""
import json

from puresoft3d_gb300.autotune import Autotuner


class _FakeCb:
    def __init__(self, pipe):
        self.pipe = pipe

    def submit(self):
        self.pipe.submits += 1

    def destroy(self):
        pass


class _FakePipe:
    COST = {8: 3.0, 16: 1.5, 32: 2.0}

    def __init__(self):
        self.bw = 32
        self.occ = 0
        self.cull = 1
        self.split = 1
        self.warp = 0
        self.items = 0
        self.lazy = 0
        self.submits = 0
        self.recorded = 0

    def setBinWidth(self, w):
        assert w in self.COST
        self.bw = w

    def setRasterOccupancy(self, o):
        assert o in (0, 8)
        self.occ = o

    def setSpanCulling(self, on):
        self.cull = int(on)

    def setRowSplit(self, n):
        assert n in (1, 2, 4, 8)
        self.split = n

    def setWarpBins(self, on):
        self.warp = int(on)

    def setSpanItems(self, on):
        self.items = int(on)

    def setLazyVaryings(self, on):
        self.lazy = int(on)

    def beginCommands(self):
        pass

    def endCommands(self):
        return _FakeCb(self)

    def finish(self):
        pass

    def scrubL2(self):
        pass

    def timerBegin(self):
        pass

    def timerEnd(self):
        return (self.COST[self.bw] - (0.25 if self.occ == 8 else 0.0) - (0.125 if self.cull == 0 else 0.0)
                - (0.0625 if self.split == 4 else 0.0) - (0.5 if self.warp and self.bw == 8 else 0.0)
                + (0.01 if self.items else 0.0) - (0.03125 if self.lazy else 0.0))


def _record(pipe):
    pipe.recorded += 1


def test_picks_fastest_and_sets_it(tmp_path):
    t = Autotuner(cache_path=str(tmp_path / "tune.json"))
    p = _FakePipe()
    best, ms = t.tune(p, _record, key="w1", candidates=(8, 16, 32), second_stage=False)
    assert best == (16, 0, 1, 1, 0, 0, 0) and p.bw == 16
    assert ms == {"8/0/1/1/0": 3.0, "16/0/1/1/0": 1.5, "32/0/1/1/0": 2.0}
    assert p.recorded == 3


def test_width_occupancy_culling_split_and_warp_bins(tmp_path):
    t = Autotuner(cache_path=str(tmp_path / "tune.json"))
    p = _FakePipe()
    best, ms = t.tune(p, _record, key="w1")
    # second stage: span items are slower here and dropped, deferred varyings faster and kept
    assert best == (16, 8, 0, 4, 0, 0, 1) and (p.bw, p.occ, p.cull, p.split, p.warp, p.items, p.lazy) == best
    assert len(ms) == 34 and p.recorded == 34
    assert ms["8/0/0/4/1"] == 3.0 - 0.125 - 0.0625 - 0.5
    assert ms["16/8/0/4/0/1/0"] > ms["16/8/0/4/0"] > ms["16/8/0/4/0/0/1"]


def test_cache_is_reused_and_keyed(tmp_path):
    path = str(tmp_path / "tune.json")
    Autotuner(cache_path=path).tune(_FakePipe(), _record, key="w1")
    table = json.load(open(path))
    assert len(table) == 1 and list(table.values())[0]["best"] == [16, 8, 0, 4, 0, 0, 1]
    p = _FakePipe()
    best, _ = Autotuner(cache_path=path).tune(p, _record, key="w1")
    assert best == (16, 8, 0, 4, 0, 0, 1) and p.lazy == 1 and p.bw == 16 and p.cull == 0 and p.split == 4 and p.recorded == 0  # from the cache
    p2 = _FakePipe()
    Autotuner(cache_path=path).tune(p2, _record, key="w2", candidates=(8, 32))
    assert p2.bw == 32 and p2.recorded == 4
    assert len(json.load(open(path))) == 2


def test_retune_ignores_cache(tmp_path):
    path = str(tmp_path / "tune.json")
    Autotuner(cache_path=path).tune(_FakePipe(), _record, key="w1")
    p = _FakePipe()
    Autotuner(cache_path=path).tune(p, _record, key="w1", retune=True)
    assert p.recorded == 34
