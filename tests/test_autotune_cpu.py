"""Autotuner host logic (xfluids_gb300/autotune.py) against a fake ensemble: coordinate descent
finds the fastest schedule, skips size classes that are absent, and caches by signature."""
import json

from xfluids_gb300 import autotune
from xfluids_gb300.mesh import make_block, make_scheme


class FakeEnsemble:
    """Timing model: ms per step = sum of per-knob costs; the cheapest value is known."""
    COST = {"tile_2d_large": {5: 3.0, 6: 1.0, 7: 2.0, 4: 4.0, 3: 5.0}, "tile_2d_small": {5: 1.0, 6: 2.0, 7: 3.0, 4: 0.5},
            "tile_3d": {5: 1.0, 6: 0.2, 4: 2.0}, "tile_1d": {7: 1.0, 6: 2.0, 5: 3.0},
            "fused_faces": {0: 1.0, 1: 0.4}, "largest_first": {1: 0.1, 0: 0.2}, "graph_steps": {1: 0.3, 4: 0.1}}

    def __init__(self, blocks, precision=1):
        self.blocks = dict(enumerate(blocks))
        self.scheme = make_scheme(precision=precision)
        self.sched = {"largest_first": 1, "fused_faces": 0, "graph_steps": 1, "tile_1d": 7, "tile_2d_small": 5,
                      "tile_2d_large": 5, "tile_3d": 5}
        self.steps = 0

    def schedule(self):
        return dict(self.sched)

    def set_schedule(self, s):
        self.sched.update(s)

    def advance(self, n):
        self.steps += n
        return 0, n * sum(self.COST[k][v] for k, v in self.sched.items())


def blocks():
    return [make_block((512, 512, 0), (1, 1, 1), [2] * 6), make_block((128, 128, 0), (1, 1, 1), [2] * 6),
            make_block((1024, 0, 0), (1, 1, 1), [2] * 6)]


def test_coordinate_descent_finds_the_cheapest_schedule(tmp_path, monkeypatch):
    monkeypatch.setenv("XFG_TUNE_CACHE", str(tmp_path / "c.json"))
    e = FakeEnsemble(blocks())
    best, rep = autotune.tune(e, steps=2)
    assert rep["source"] == "search"
    assert best == {"largest_first": 1, "fused_faces": 1, "graph_steps": 4, "tile_1d": 7, "tile_2d_small": 4,
                    "tile_2d_large": 6, "tile_3d": 5}  # no 3D member: its knob stays at the default
    assert e.schedule() == best
    assert all(s["tile_3d"] == 5 for s, _ in rep["trials"])
    data = json.load(open(tmp_path / "c.json"))
    assert list(data.values())[0]["schedule"] == best


def test_cache_hit_sets_schedule_without_trials(tmp_path, monkeypatch):
    monkeypatch.setenv("XFG_TUNE_CACHE", str(tmp_path / "c.json"))
    best, _ = autotune.tune(FakeEnsemble(blocks()), steps=1)
    e2 = FakeEnsemble(blocks())
    best2, rep = autotune.tune(e2, steps=1)
    assert rep["source"] == "cache" and best2 == best and e2.steps == 0 and e2.schedule() == best
    # another size mix or precision is another key
    e3 = FakeEnsemble(blocks()[:2], precision=0)
    _, rep3 = autotune.tune(e3, steps=1)
    assert rep3["source"] == "search"


def test_signature_classes():
    e = FakeEnsemble(blocks() + [make_block((32, 16, 8), (1, 1, 1), [2] * 6)])
    sig = autotune.signature(e, "GB300")
    assert sig.startswith("GB300|p1|o5|") and "tile_1d:10:1" in sig and "tile_2d_large:18:1" in sig
    assert "tile_2d_small:14:1" in sig and "tile_3d:12:1" in sig
