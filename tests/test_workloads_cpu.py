"""Host logic of the workload runner: the vortex horizon report, driven by an oracle-backed
stand-in for the CUDA handle (same methods as xfluids_gb300.fluid.Fluid), on a small grid."""
import numpy as np
import pytest

from oracle import xfo
from xfluids_gb300 import workloads


class _OracleFluid:
    """The subset of Fluid that vortex_horizon uses, run by the oracle (precision ignored)."""

    def __init__(self, b, s, th, device=0):
        self.b, self.s, self.th = b, s, th

    def InitialU(self, U, T):
        self.o = xfo.Oracle(self.b, self.s, self.th, U, T)

    def initialize(self):
        self.o.initialize()
        self.t = 0.0

    def advance_timed(self, nsteps, target_t):
        k = 0
        while k < nsteps and self.t < target_t:
            self.t, _ = self.o.step(target_t)
            k += 1
        return 0, self.t, k, 1.0

    def get(self, name):
        return self.o.get(name)

    def close(self):
        pass


def test_vortex_horizon_report(monkeypatch):
    import xfluids_gb300.fluid as fluid
    monkeypatch.setattr(fluid, "Fluid", _OracleFluid)
    xfo.set_threads(2)
    out = workloads.vortex_horizon(16, 1, precisions=(0, workloads.MIXED), chunk=50)
    for name in ("fp64", "mixed"):
        r = out[name]
        assert r["status"] == 0 and r["t"] == pytest.approx(10.0, abs=1e-12)
        assert r["steps"] > 100 and abs(r["mass_drift_rel"]) < 1e-13
        assert 0.0 < r["l1_rho_vs_exact"] < r["linf_rho_vs_exact"]
    # the stand-in runs the same arithmetic for both, so the comparison is exactly zero
    assert out["mixed_vs_fp64"]["l1_rel"] == [0.0] * 5
    assert out["mixed_vs_fp64"]["linf_normwise"] == 0.0
    assert np.isfinite(out["mixed_vs_fp64"]["linf_normwise"])
