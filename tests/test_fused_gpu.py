"""The fused mixed stage of two-dimensional single-gas blocks (xfg_fused.cuh): primitive recovery,
both face sweeps, divergence and RK update in one kernel per stage, reconstructing deviations from
each face's left cell in FP32.

- Its right-hand side (xfg_compute_lu through the fused kernel) against the FP64 path's on the same
  state, per component normwise; blocks whose sizes are not multiples of the 32 x 7 tile,
  periodic, outflow, symmetry and wall sides, LLF and Roe.
- Free-running steps against the FP64 path, and the stage-by-stage API (BoundaryCondition +
  UpdateFluidStates + ComputeFluidLU + UpdateFluidURK3) against the fused steps.
- Conservation: a face flux shared by two tiles is computed by both with the same instructions,
  and the divergence takes it exactly, so the total of every conserved quantity of a periodic
  block moves only by the FP64 stage arithmetic.
"""
import numpy as np
import pytest

import helpers as H
from xfluids_gb300 import cases
from xfluids_gb300.abi import FP64, MIXED, LLF, ROE, OUTFLOW, PERIODIC, SYMMETRY, NSLIPWALL, SLIPWALL, INFLOW
from xfluids_gb300.mesh import make_block

pytestmark = pytest.mark.gpu

# The deviation form's rounding acts on a few cells' variation of the flux, so its right-hand side
# stays within 1e-6 of the FP64 one per component (normwise over the block)
LU_TOL = 1e-5


def _vortex(nx, ny, bc=PERIODIC):
    """The isentropic vortex on an nx x ny block of [0,10]^2 (cell sizes differ in x and y)."""
    b, s, th, _, _ = cases.isentropic_vortex(16)
    b = make_block((nx, ny, 0), (10.0, 10.0, 1.0), [bc] * 6, cfl=0.5)
    X, Y, _ = cases.cell_centres(b)
    xv, yv = X - 5.0, Y - 5.0
    r2 = xv * xv + yv * yv
    inter1 = 25.0 * np.exp(1.0 - r2) / 28.0 / np.pi / np.pi
    inter2 = 0.5 * 5.0 * np.exp(0.5 * (1.0 - r2)) / np.pi
    rho = (1.0 - inter1) ** 2.5
    U = cases.conserved_ideal(rho, 1.0 - inter2 * yv, 1.0 + inter2 * xv, 0.1 * np.sin(X), rho ** 1.4)
    return b, s, th, U, None


def _riemann(n, bcs, artificial=LLF, seed=3):
    b, s, th, U, T = H.riemann_small(n, seed=seed, artificial=artificial)
    for q in range(6):
        b.Boundarys[q] = bcs[q]
    return b, s, th, U, T


CASES = {
    "vortex64": lambda: _vortex(64, 64),
    "vortex45x23": lambda: _vortex(45, 23),
    "vortex33x8_roe": lambda: _vortex(33, 8),
    "riemann48_outflow": lambda: _riemann(48, [OUTFLOW] * 6),
    "riemann37_walls": lambda: _riemann(37, [SYMMETRY, NSLIPWALL, SLIPWALL, NSLIPWALL, OUTFLOW, OUTFLOW]),
    "riemann40_roe_inflow": lambda: _riemann(40, [INFLOW, OUTFLOW, OUTFLOW, INFLOW, OUTFLOW, OUTFLOW], artificial=ROE),
}


def _make(name, prec):
    b, s, th, U, T = CASES[name]()
    if name.endswith("_roe"):
        s.artificial_type = ROE
    s.precision = prec
    return b, s, th, U, T


def _fluid(b, s, th, U, T):
    from xfluids_gb300.fluid import Fluid
    f = Fluid(b, s, th)
    f.InitialU(U, T)
    return f


def _lu(name, prec):
    b, s, th, U, T = _make(name, prec)
    f = _fluid(b, s, th, U, T)
    f.BoundaryCondition(0)
    f.UpdateFluidStates(0)
    f.ComputeFluidLU(0)
    lu = H.inner_aos(b, f.get("LU"), 5)
    f.close()
    return b, lu


@pytest.mark.parametrize("name", list(CASES))
def test_fused_rhs_close_to_fp64(name, cuda_lib):
    b, ref = _lu(name, FP64)
    _, got = _lu(name, MIXED)
    r = H.normwise(got, ref, 5)
    print(f"{name}: fused mixed LU vs FP64, normwise per component {r}")
    assert np.all(r <= LU_TOL), r


@pytest.mark.parametrize("name", ["vortex45x23", "riemann37_walls", "riemann40_roe_inflow"])
def test_fused_steps_close_to_fp64_and_to_the_stage_api(name, cuda_lib):
    b, s, th, U, T = _make(name, FP64)
    f64 = _fluid(b, s, th, U, T)
    f64.initialize()
    st, t64, n = f64.advance(12)
    assert st == 0 and n == 12
    ref = H.inner_aos(b, f64.get("U"), 5)
    f64.close()
    b, s, th, U, T = _make(name, MIXED)
    fm = _fluid(b, s, th, U, T)
    fm.initialize()
    st, tm, n = fm.advance(40, t64)
    assert st == 0 and abs(tm - t64) <= 1e-12 * t64
    got = H.inner_aos(b, fm.get("U"), 5)
    fm.close()
    r = H.normwise(got, ref, 5)
    print(f"{name}: fused mixed vs FP64 after {n} steps, normwise {r}")
    assert np.all(r <= 1e-5), r
    # one step through the stage-by-stage API of class Fluid against one fused step (the same dt:
    # both take the maxima of the initial UpdateFluidStates)
    fa = _fluid(b, s, th, U, T)
    fb = _fluid(b, s, th, U, T)
    fa.initialize(), fb.initialize()
    dt = fa.GetFluidDt()
    for flag in (1, 2, 3):
        fa.stage(flag, dt)
    fb.advance(1)
    ra = H.inner_aos(b, fa.get("U"), 5)
    rb = H.inner_aos(b, fb.get("U"), 5)
    fa.close(), fb.close()
    assert np.all(H.normwise(ra, rb, 5) <= 1e-13), H.normwise(ra, rb, 5)


def test_fused_step_conserves_on_a_periodic_block(cuda_lib):
    """Every conserved total of a periodic 200 x 90 vortex (tiles of 32 x 7 do not divide it) after
    20 fused steps: moved only by the FP64 stage arithmetic (pairwise sums)."""
    b, s, th, U, T = _vortex(200, 90)
    s.precision = MIXED
    f = _fluid(b, s, th, U, T)
    f.initialize()
    st, t, n = f.advance(20)
    assert st == 0 and n == 20
    a = H.inner_aos(b, f.get("U"), 5)
    f.close()
    a0 = H.inner_aos(b, U, 5)
    tot = lambda x: np.array([np.sum(np.sort(x[:, q])) for q in range(5)])
    rel = np.abs(tot(a) - tot(a0)) / np.abs(a0).sum(axis=0)
    print("relative drift of the conserved totals", rel)
    assert np.all(rel <= 2e-16 * 20 * 4), rel


def test_fused_launches_and_phases(cuda_lib):
    b, s, th, U, T = _make("vortex64", MIXED)
    f = _fluid(b, s, th, U, T)
    f.initialize()
    assert f.launches_per_step == 1 + 3 * 3 + 1
    ph = f.time_phases()
    assert ph["faces_x"] > 0 and ph["states"] == 0 and ph["div_rk"] == 0
    # primitives of the last UpdateFluidStates (stage 3's input) are readable after the step
    rho = f.get("rho").reshape(b.Ymax, b.Xmax)
    assert np.all(rho > 0.3) and np.all(rho < 1.1)
    f.close()


@pytest.mark.parametrize("name", ["vortex200x90", "riemann40_roe_inflow", "riemann48_outflow"])
def test_tma_staged_kernel_equals_one_tile_per_cta(name, cuda_lib, monkeypatch):
    """With XFG_FUSED_TMA=1 at handle creation, blocks with an even Xmax run the persistent kernel
    whose state arrives by TMA copies (k_fused_stage_tma) instead of the one-tile-per-CTA kernel.
    Both compute every tile with the same instructions from the same values: the states after
    free-running steps (LU included, through a stage-API step) are bitwise equal."""
    make = (lambda: _vortex(200, 90)) if name == "vortex200x90" else CASES[name]
    out = []
    for env in ("1", "0"):
        monkeypatch.setenv("XFG_FUSED_TMA", env)
        b, s, th, U, T = make()
        if name.endswith("_roe"):
            s.artificial_type = ROE
        s.precision = MIXED
        assert b.Xmax % 2 == 0
        f = _fluid(b, s, th, U, T)
        f.initialize()
        st, t, n = f.advance(10)
        assert st == 0 and n == 10
        dt = f.GetFluidDt()
        for flag in (1, 2, 3):
            f.stage(flag, dt)
        out.append((f.get("U").copy(), f.get("LU").copy(), t))
        f.close()
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
