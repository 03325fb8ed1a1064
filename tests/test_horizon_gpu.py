"""Whole solves at the horizons the workloads are quoted on, through the C ABI.

- Sod shock tube, 1024 cells to t = 0.2: the strict form and the FP64 form run free next to the
  oracle for every step of the solve; the density is compared with the exact Riemann solution.
- 2D isentropic vortex, 10 periods (t = 100, the exact solution is the initial state): the FP64
  form against the oracle on a 32^2 grid (about 3700 steps), and the mixed form against FP64 at
  64^2, 128^2, 512^2 (and 1024^2 on request): L1 per conserved component within 1e-6 of its mean.

Every measured figure is printed before it is checked. The bounds are drift bounds over the whole
solve, not the per-stage parity bound.
"""
import os

import numpy as np
import pytest

import helpers as H
from oracle import xfo
from oracle.xfo import Oracle
from xfluids_gb300 import cases
from xfluids_gb300.abi import MIXED, FP64, FP64_STRICT

pytestmark = pytest.mark.gpu


def _gpu_solve(b, s, th, U, T, t_end, chunk=1024):
    from xfluids_gb300.fluid import Fluid
    f = Fluid(b, s, th)
    try:
        f.InitialU(U, T)
        f.initialize()
        t, k, st = 0.0, 0, 0
        while t < t_end and st == 0:
            st, t, kk = f.advance(chunk, t_end)
            k += kk
        return st, t, k, H.inner_aos(b, f.get("U"), s.Emax)
    finally:
        f.close()


def _oracle_solve(b, s, th, U, T, t_end):
    o = Oracle(b, s, th, U, T)
    o.initialize()
    t, k = 0.0, 0
    while t < t_end:
        t, _ = o.step(t_end)
        k += 1
    return t, k, H.inner_aos(b, o.get("U"), s.Emax)


def test_sod_1024_whole_solve(cuda_lib):
    xfo.set_threads(4)
    b, s, th, U, T = cases.sod(1024)
    t_o, k_o, ref = _oracle_solve(b, s, th, U, T, 0.2)
    X, _, _ = cases.cell_centres(b)
    ex = cases.sod_exact_density(X[b.inner_slices()].ravel(), 0.2)
    res = {}
    for name, prec in (("strict", FP64_STRICT), ("fp64", FP64)):
        s.precision = prec
        st, t, k, g = _gpu_solve(b, s, th, U, T, 0.2)
        res[name] = (st, t, k, float(H.normwise(g, ref, 5).max()), float(np.abs(g[:, 0] - ex).mean()))
    print(f"Sod 1024 to t = 0.2, oracle {k_o} steps (L1 rho vs exact {np.abs(ref[:, 0] - ex).mean():.3e}); "
          + "; ".join(f"{n}: {r[2]} steps, normwise vs oracle {r[3]:.3e}, L1 rho vs exact {r[4]:.3e}"
                      for n, r in res.items()))
    for name, (st, t, k, nw, l1) in res.items():
        assert st == 0 and k == k_o and t == t_o, (name, st, k, k_o, t, t_o)
        assert l1 < 3e-3, (name, l1)
    assert res["strict"][3] <= 1e-13, res["strict"]
    assert res["fp64"][3] <= 1e-9, res["fp64"]


def test_vortex_ten_periods_fp64_against_oracle(cuda_lib):
    xfo.set_threads(4)
    b, s, th, U, T = cases.isentropic_vortex(32)
    t_o, k_o, ref = _oracle_solve(b, s, th, U, T, 100.0)
    res = {}
    for name, prec in (("strict", FP64_STRICT), ("fp64", FP64)):
        s.precision = prec
        st, t, k, g = _gpu_solve(b, s, th, U, T, 100.0)
        d = np.abs(g - ref)
        res[name] = (st, t, k, float(H.normwise(g, ref, 5).max()), float(d.mean()))
    print(f"vortex 32^2, 10 periods, oracle {k_o} steps; "
          + "; ".join(f"{n}: {r[2]} steps, normwise vs oracle {r[3]:.3e}, L1 vs oracle {r[4]:.3e}"
                      for n, r in res.items()))
    for name, (st, t, k, nw, l1) in res.items():
        assert st == 0 and k == k_o and abs(t - t_o) <= 1e-12 * t_o, (name, st, k, k_o, t, t_o)
    assert res["strict"][3] <= 1e-12, res["strict"]
    assert res["fp64"][3] <= 1e-9, res["fp64"]


MIXED_L1_BOUND = 1e-6   # mixed against FP64, L1 per conserved component over its own mean


@pytest.mark.parametrize("n", [
    64, 128, 512,
    pytest.param(1024, marks=pytest.mark.skipif(
        not os.environ.get("XFG_HORIZON_1024"),
        reason="the FP64 reference solve of 1024^2 over 10 periods takes about 18 min; set XFG_HORIZON_1024=1")),
])
def test_vortex_ten_periods_mixed_against_fp64(n, cuda_lib):
    """The vortex over its 10 periods (t = 100) in FP64 and in the mixed form: every conserved
    component of the mixed state within 1e-6 of the FP64 state in L1 relative to its own mean, and
    the totals kept to the FP64 stage arithmetic's level."""
    from xfluids_gb300.workloads import vortex_horizon
    out = vortex_horizon(n, 10, precisions=(FP64, MIXED), chunk=2048)
    print(out)
    for name in ("fp64", "mixed"):
        assert out[name]["status"] == 0 and abs(out[name]["t"] - 100.0) <= 1e-12, out[name]
        # the FP64 stage sums move the total mass by about 4e-17 per step (rounding of the stage
        # arithmetic); the FP32 face fluxes must add nothing to that
        assert abs(out[name]["mass_drift_rel"]) <= 2e-16 * out[name]["steps"], out[name]
    assert out["fp64"]["steps"] == out["mixed"]["steps"] or abs(out["fp64"]["steps"] - out["mixed"]["steps"]) <= 1
    pc = out["mixed_vs_fp64"]["per_component"]
    for nm in ("rho", "rho_u", "rho_v", "E"):
        assert pc[nm]["l1_rel"] <= MIXED_L1_BOUND, (nm, pc)
    assert pc["rho_w"]["linf"] == 0.0   # a 2D flow without w keeps rho w = 0 exactly
