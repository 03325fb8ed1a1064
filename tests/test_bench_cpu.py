"""Host logic of bench.py on CPU: the committed algorithmic flop counts against a recount on the
oracle, and the accuracy leg (GPU runs + oracle checker) driven by an oracle-backed stand-in for the
CUDA handle on a small vortex."""
import numpy as np
import pytest

import bench
from oracle import xfo
from xfluids_gb300 import cases


def test_flop_constants_match_oracle_count():
    n = bench.FLOP_COUNT_SIZE
    b, s, th, U, T = cases.isentropic_vortex(n)
    c = xfo.count_flops(b, s, th, U, T, 1)
    per_face_x = c["faces_x"] / 3.0 / ((n + 1) * n)   # three RK stages, (n+1) x faces per row
    per_cell_update = sum(c.values()) / float(n * n)
    assert per_face_x == bench.FLOPS_PER_FACE_X
    assert per_cell_update == bench.FLOPS_PER_CELL_UPDATE


class _OracleFluid:
    """The subset of Fluid that bench.accuracy_gpu uses, run by the oracle (precision ignored)."""

    def __init__(self, b, s, th, device=0):
        self.b, self.s, self.th = b, s, th

    def InitialU(self, U, T):
        self.o = xfo.Oracle(self.b, self.s, self.th, U, T)

    def initialize(self):
        self.o.initialize()
        self.t = 0.0

    def advance(self, nsteps, target_t):
        k = 0
        while k < nsteps and self.t < target_t:
            self.t, _ = self.o.step(target_t)
            k += 1
        return 0, self.t, k

    def get(self, name):
        return self.o.get(name)

    def close(self):
        pass


def test_accuracy_leg_with_oracle_stand_in(monkeypatch):
    from xfluids_gb300 import fluid
    monkeypatch.setattr(fluid, "Fluid", _OracleFluid)
    runs = bench.accuracy_gpu(0, n=24, t_end=0.05)
    val, steps, el, acc = bench.cpu_leg(2, runs, size=32, min_seconds=0.2)
    assert val > 0 and steps >= 1 and el >= 0.2
    assert acc["steps"] > 0
    for name in ("fp64", "mixed"):
        r = acc[name]
        assert r["steps"] == acc["steps"]
        assert r["l1_vs_oracle"] == 0.0 and r["max_normwise_vs_oracle"] == 0.0
        assert r["l1_rho_vs_exact"] == pytest.approx(acc["oracle_l1_rho_vs_exact"])
        assert np.isfinite(r["linf_rho_vs_exact"]) and r["linf_rho_vs_exact"] > 0.0


def test_hbm_context_reads_the_measured_peak_or_falls_back(tmp_path):
    peaks = tmp_path / "peaks.json"
    peaks.write_text('{"hbm_gbs": 6000.0}')
    h = bench.hbm_context(3.0e9, 20.0, peaks_path=str(peaks))
    assert h["dram_gbs"] == pytest.approx(150.0) and h["hbm_peak_gbs"] == 6000.0
    assert h["frac"] == pytest.approx(0.025) and h["peak_source"].startswith("of measured")
    h = bench.hbm_context(3.0e9, 20.0, peaks_path=str(tmp_path / "absent.json"))
    assert h["hbm_peak_gbs"] == 6800.0 and h["peak_source"].startswith("of fallback")
    assert bench.hbm_context(None, 20.0) is None


def test_batched_mixing_members_are_seeded_and_sized_like_the_single_layer():
    """The members of the batched mixing-layer ensemble: 16 temporal mixing layers of seeded sizes
    32a x 16b x 16c, a, b, c in [4, 8], together about the single 512 x 256 x 256 layer's cells."""
    s, th, ms = bench.mixing_members(16)
    sizes = [(b.X_inner, b.Y_inner, b.Z_inner) for b, _, _ in ms]
    assert sizes == [(b.X_inner, b.Y_inner, b.Z_inner) for b, _, _ in bench.mixing_members(16)[2]]
    assert all(x % 32 == 0 and 128 <= x <= 256 and y % 16 == 0 and 64 <= y <= 128 and z % 16 == 0 and 64 <= z <= 128
               for x, y, z in sizes)
    cells = sum(x * y * z for x, y, z in sizes)
    assert 0.8 * 512 * 256 * 256 <= cells <= 1.2 * 512 * 256 * 256
    assert s.cop == 1 and s.num_species == 5 and s.scheme_order == 7
    for b, U, T in ms:
        assert U.size == b.Xmax * b.Ymax * b.Zmax * 9 and T.size == b.Xmax * b.Ymax * b.Zmax


def test_per_component_names_the_worst_relative_component():
    from xfluids_gb300.workloads import per_component
    r = np.array([[1.0, 2.0, 0.0], [3.0, 2.0, 0.0]])
    a = r + np.array([[1e-6, 0.0, 5e-9], [1e-6, 4e-6, 0.0]])
    out = per_component(a, r, ["a", "b", "z"])
    assert out["a"]["l1_rel"] == pytest.approx(1e-6 / 2.0)
    assert out["b"]["l1_rel"] == pytest.approx(2e-6 / 2.0)
    assert out["z"]["l1_rel"] is None and out["z"]["l1"] == pytest.approx(2.5e-9)   # zero reference: absolute only
    assert out["worst"] == "b"
