"""Parity of the CUDA FP64 path with the oracle, stage by stage, through the C ABI.

Bound: every stage's U / U1 / LU and primitives agree with the oracle to PARITY_TOL (1e-12)
normwise relative per component; fused steps (xfg_step) and graph replays (xfg_advance) agree
with the stage-by-stage oracle run to the same bound.

Mixtures in the FP64 form contract the face sweeps into FMAs (the ill-conditioned Roe sound speed
excepted, which keeps the reference's rounding); they are compared on identical inputs per RK
stage: before every stage the oracle's U, U1 and T (the warm start of the temperature Newton
iteration, whose stopping test |dT| <= 1e-6 turns a 1e-15 change of the energy into a different
iterate) are loaded into the handle, and the right-hand side is compared through the stage
increment it makes (dt LU against the state; see _check_increment), the stage results per
component. The strict form (no contraction anywhere) runs free next to the oracle, bit for bit.
"""
import numpy as np
import pytest

import helpers as H
from oracle.xfo import Oracle
from xfluids_gb300.abi import ROE, GLF, MIXED, FP64, FP64_STRICT

pytestmark = pytest.mark.gpu


def _fluid(b, s, th, U, T):
    from xfluids_gb300.fluid import Fluid
    f = Fluid(b, s, th)
    f.InitialU(U, T)
    return f


def _check(name, a, b, ncomp, tol=H.PARITY_TOL):
    r = H.normwise(a, b, ncomp)
    assert np.all(r <= tol), f"{name}: normwise relative error {r} > {tol}"
    return float(r.max())


def _check_increment(name, lu_a, lu_b, U, dt, ncomp, tol=H.PARITY_TOL):
    """The right-hand side through the stage increment it makes: max|dt (LU_a - LU_b)| / max|U| per
    component. LU is a difference of face fluxes, so a rounding change of a flux of size |F| moves it
    by ~eps |F| / dx whatever its own size; where the fluxes are pressure-dominated (1e5 Pa) and
    nearly cancel, its per-component ratio measures that cancellation, the increment does not."""
    a, b, u = (np.asarray(x).reshape(-1, ncomp) for x in (lu_a, lu_b, U))
    num, den = np.abs(dt * (a - b)).max(axis=0), np.abs(u).max(axis=0)
    r = np.where(den > 0, num / np.where(den > 0, den, 1.0), num)
    assert np.all(r <= tol), f"{name}: stage increment relative error {r} > {tol}"
    return float(r.max())


def _compare_stage(block, f, o, E, tag, cop, lu_dt=None):
    """lu_dt: compare LU through the stage increment with this dt (mixtures in the FP64 form, whose
    face sweeps are contracted); otherwise per component."""
    worst = 0.0
    worst = max(worst, _check(f"{tag} U", H.inner_aos(block, f.get("U"), E), H.inner_aos(block, o.get("U"), E), E))
    worst = max(worst, _check(f"{tag} U1", H.inner_aos(block, f.get("U1"), E), H.inner_aos(block, o.get("U1"), E), E))
    if lu_dt is None:
        worst = max(worst, _check(f"{tag} LU", H.inner_aos(block, f.get("LU"), E), H.inner_aos(block, o.get("LU"), E), E))
    else:
        worst = max(worst, _check_increment(f"{tag} LU", H.inner_aos(block, f.get("LU"), E),
                                            H.inner_aos(block, o.get("LU"), E), H.inner_aos(block, o.get("U"), E),
                                            lu_dt, E))
    names = ["rho", "p", "u", "v", "w", "c", "H"] + (["T"] if cop else [])
    for nm in names:
        worst = max(worst, _check(f"{tag} {nm}", f.get(nm), o.get(nm), 1))
    return worst


def resync(f, o, cop):
    """Load the oracle's stage inputs into the handle (identical inputs per RK stage)."""
    f.set("U", o.get("U"))
    f.set("U1", o.get("U1"))
    if cop:
        f.set("T", o.get("T"))


def needs_resync(s, precision):
    """Mixtures in the FP64 form with contracted faces (with the positivity limiter on they keep
    the no-contraction faces: its theta amplifies the flux's rounding)."""
    return bool(s.cop) and precision == FP64 and not s.positivity


def run_stagewise(case, steps=2, precision=FP64, transport=None):
    b, s, th, U, T = case
    s.precision = precision
    E = s.Emax
    f = _fluid(b, s, th, U, T) if transport is None else None
    if f is None:
        from xfluids_gb300.fluid import Fluid
        f = Fluid(b, s, th)
        f.set_transport(transport)
        f.InitialU(U, T)
    o = Oracle(b, s, th, U, T, transport=transport)
    f.initialize()
    o.initialize()
    sync = needs_resync(s, precision)
    worst = 0.0
    for step in range(steps):
        dt_g, dt_o = f.GetFluidDt(), o.get_dt()
        assert abs(dt_g - dt_o) <= 1e-12 * dt_o, (dt_g, dt_o)
        for flag in (1, 2, 3):
            if sync:
                resync(f, o, s.cop)
            f.stage(flag, dt_o)
            o.stage(flag, dt_o)
            worst = max(worst, _compare_stage(b, f, o, E, f"step {step} stage {flag}", s.cop,
                                              lu_dt=dt_o if sync else None))
    f.close()
    return worst


CASES = {
    "sod_weno5_llf": lambda: H.sod_like(128),
    "sod_weno7_llf": lambda: H.sod_like(128, order=7),
    "sod_weno5_roe": lambda: H.sod_like(96, artificial=ROE),
    "sod_weno5_glf": lambda: H.sod_like(96, artificial=GLF),
    "vortex64": lambda: __import__("xfluids_gb300.cases", fromlist=["x"]).isentropic_vortex(64),
    "riemann2d_weno5": lambda: H.riemann_small(40),
    "riemann2d_weno7_sym": lambda: H.riemann_small(36, order=7, bc=2),
    "blast3d_weno5": lambda: H.blast3d(),
    "blast3d_weno7_glf": lambda: H.blast3d(order=7, artificial=GLF),
    "insert_st_ghost_nasa": lambda: H.insert_st(120),
    "insert_st_janaf_weno7": lambda: H.insert_st(100, order=7, ghost=False, thermo_kind=0),
    "mixing5_weno7_janaf": lambda: H.mixing_small(),
    "mixing5_weno5_nasa_roe": lambda: H.mixing_small((16, 12, 8), order=5, thermo_kind=1, artificial=ROE),
    # WENO-CU6
    "riemann2d_cu6_llf": H.with_order(lambda: H.riemann_small(40), 6),
    "blast3d_cu6_glf": H.with_order(lambda: H.blast3d(artificial=GLF), 6),
    "mixing5_cu6_janaf_roe": H.with_order(lambda: H.mixing_small((16, 12, 8), order=5, artificial=ROE), 6),
    # positivity limiter on (cases where it acts: without it the first two turn negative)
    "pp_riemann88": H.with_positivity(lambda: H.riemann_member(88, 32)),
    "pp_riemann1d": H.with_positivity(H.riemann1d_strong),
    "pp_mixing5_weno5_janaf": H.with_positivity(lambda: H.mixing_small((12, 8, 6), order=5)),
    "pp_blast3d_weno7": H.with_positivity(lambda: H.blast3d(order=7)),
    "pp_insert_st_ghost_nasa": H.with_positivity(lambda: H.insert_st(120)),
}


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("name", list(CASES))
def test_stagewise_parity(name, precision, cuda_lib):
    worst = run_stagewise(CASES[name](), steps=2, precision=precision)
    print(f"{name}: worst normwise relative difference {worst:.3e}")


@pytest.mark.parametrize("name", ["vortex64", "blast3d_weno7_glf", "riemann2d_weno7_sym", "mixing5_weno7_janaf",
                                  "pp_riemann88", "pp_mixing5_weno5_janaf", "riemann2d_cu6_llf", "mixing5_cu6_janaf_roe"])
def test_strict_is_bitwise(name, cuda_lib):
    """Without contraction the CUDA path performs the reference's operation sequence: every array
    of every stage is bit-identical to the oracle (no log/exp on these cases)."""
    worst = run_stagewise(CASES[name](), steps=2, precision=FP64_STRICT)
    assert worst == 0.0


@pytest.mark.parametrize("name", ["vortex64", "sod_weno5_llf", "mixing5_weno7_janaf", "blast3d_weno5", "pp_riemann88",
                                  "pp_mixing5_weno5_janaf"])
def test_fused_step_and_graph(name, cuda_lib):
    """Fused steps and graph replays against the free-running oracle (mixtures: the strict form,
    see the module docstring), and for mixtures in the FP64 form against the same handle's
    stage-by-stage calls."""
    b, s, th, U, T = CASES[name]()
    E = s.Emax
    if s.cop:
        s.precision = FP64
        f0, f1 = _fluid(b, s, th, U, T), _fluid(b, s, th, U, T)
        f0.initialize(), f1.initialize()
        for q in range(3):
            dt = f0.GetFluidDt()
            for flag in (1, 2, 3):
                f0.stage(flag, dt)
        st, _, n = f1.advance(3)
        assert st == 0 and n == 3
        _check("FP64 graph vs stage calls", H.inner_aos(b, f1.get("U"), E), H.inner_aos(b, f0.get("U"), E), E,
               tol=1e-15)
        f0.close(), f1.close()
        s.precision = FP64_STRICT
    o = Oracle(b, s, th, U, T)
    o.initialize()
    f1 = _fluid(b, s, th, U, T)
    f1.initialize()
    f2 = _fluid(b, s, th, U, T)
    f2.initialize()
    nsteps = 4
    for q in range(nsteps):
        to, dto = o.step()
        st, t1, dt1 = f1.step()
        assert st == 0
        assert abs(dt1 - dto) <= 1e-12 * dto
    st, t2, n2 = f2.advance(nsteps)
    assert st == 0 and n2 == nsteps
    assert abs(t2 - to) <= 1e-12 * to
    ref = H.inner_aos(b, o.get("U"), E)
    _check("fused U", H.inner_aos(b, f1.get("U"), E), ref, E)
    _check("graph U", H.inner_aos(b, f2.get("U"), E), ref, E)
    f1.close(), f2.close()


def test_advance_stops_at_target(cuda_lib):
    b, s, th, U, T = H.sod_like(64)
    o = Oracle(b, s, th, U, T)
    o.initialize()
    t_end = 0.01
    t = 0.0
    n_o = 0
    while t < t_end:
        t, _ = o.step(t_end)
        n_o += 1
    f = _fluid(b, s, th, U, T)
    f.initialize()
    st, tg, n = f.advance(n_o + 5, t_end)   # extra replays past the target must do nothing
    assert st == 0 and n == n_o and tg == t
    _check("U at t_end", H.inner_aos(b, f.get("U"), 5), H.inner_aos(b, o.get("U"), 5), 5)
    f.close()


def test_mixed_mixture_close_to_fp64(cuda_lib):
    """Mixed form on the 5-species mixing layer: FP32 projection / WENO with the FP64 Roe sound
    speed of the mixture and the FP64 Newton temperature."""
    b, s, th, U, T = H.mixing_small((24, 16, 8))
    f64 = _fluid(b, s, th, U, T)
    s2 = H.mixing_small((24, 16, 8))[1]
    s2.precision = MIXED
    fmx = _fluid(b, s2, th, U, T)
    f64.initialize(), fmx.initialize()
    st1, t1, n1 = f64.advance(5)
    st2, t2, n2 = fmx.advance(50, t1)
    assert st1 == 0 and st2 == 0 and t1 == t2
    a, r = H.inner_aos(b, fmx.get("U"), 9), H.inner_aos(b, f64.get("U"), 9)
    num, den = np.abs(a - r).mean(axis=0), np.abs(r).mean(axis=0)
    rel = np.where(den > 0, num / np.where(den > 0, den, 1.0), num)   # H2O is identically zero
    print("mixed mixture L1 relative per component", rel)
    assert np.all(rel < 1e-4), rel
    f64.close(), fmx.close()


def test_mixed_precision_close_to_fp64(cuda_lib):
    from xfluids_gb300 import cases
    b, s, th, U, T = cases.isentropic_vortex(128)
    f64 = _fluid(b, s, th, U, T)
    s2 = cases.isentropic_vortex(128, precision=MIXED)[1]
    fmx = _fluid(b, s2, th, U, T)
    f64.initialize(), fmx.initialize()
    f64.advance(20)
    fmx.advance(20)
    a, r = H.inner_aos(b, fmx.get("U"), 5), H.inner_aos(b, f64.get("U"), 5)
    l1 = np.abs(a - r).mean(axis=0)
    assert np.all(l1 < 1e-5), l1
    f64.close(), fmx.close()


def test_nan_detection(cuda_lib):
    b, s, th, U, T = H.sod_like(64)
    U = U.copy().reshape(-1)
    U[5 * 40 + 4] = np.nan     # energy of one inner cell
    f = _fluid(b, s, th, U, T)
    err = f.initialize()
    assert err                  # EstimatePrimitiveVar-style capture (p is NaN)
    st, t, dt = f.step()
    assert st > 0
    f.close()


def test_positivity_limiter_acts_and_keeps_density_positive(cuda_lib):
    """Without the limiter the first stage of this member drives the density negative (status
    10000); with it the run goes on and the density stays positive, FP64 and mixed form."""
    for prec in (FP64, MIXED):
        b, s, th, U, T = H.riemann_member(88, 32)
        s.precision = prec
        f = _fluid(b, s, th, U, T)
        f.initialize()
        st, _, _ = f.advance(3)
        assert st != 0
        f.close()
        s.positivity = 1
        f = _fluid(b, s, th, U, T)
        f.initialize()
        st, t, n = f.advance(20)
        assert st == 0 and n == 20
        assert H.inner_aos(b, f.get("U"), 5)[:, 0].min() > 0.0
        f.close()


def test_mixed_cu6_close_to_fp64(cuda_lib):
    """The mixed form with WENO-CU6 reconstruction stays close to the FP64 path."""
    b, s, th, U, T = H.with_order(lambda: H.riemann_small(64), 6)()
    f64 = _fluid(b, s, th, U, T)
    b2, s2, _, _, _ = H.with_order(lambda: H.riemann_small(64), 6)()
    s2.precision = MIXED
    fmx = _fluid(b2, s2, th, U, T)
    f64.initialize(), fmx.initialize()
    st1, t1, n1 = f64.advance(10)
    st2, t2, n2 = fmx.advance(40, t1)
    assert st1 == 0 and st2 == 0
    a, r = H.inner_aos(b, fmx.get("U"), 5), H.inner_aos(b, f64.get("U"), 5)
    num, den = np.abs(a - r).mean(axis=0), np.abs(r).mean(axis=0)
    rel = np.where(den > 0, num / np.where(den > 0, den, 1.0), num)   # rho w is zero in 2D
    assert np.all(rel < 1e-4), rel
    f64.close(), fmx.close()


def test_mixed_single_gas_glf_and_primitives(cuda_lib):
    """Single-gas mixed form: the GLF maxima come from its FP32 primitives (the form writes no FP64
    primitives during the step) and the primitives a caller reads back are those of the last
    UpdateFluidStates; both close to the FP64 path."""
    b, s, th, U, T = H.blast3d(artificial=GLF)
    f64 = _fluid(b, s, th, U, T)
    b2, s2, _, _, _ = H.blast3d(artificial=GLF)
    s2.precision = MIXED
    fmx = _fluid(b2, s2, th, U, T)
    f64.initialize(), fmx.initialize()
    st1, t1, n1 = f64.advance(5)
    st2, t2, n2 = fmx.advance(30, t1)
    assert st1 == 0 and st2 == 0 and abs(t2 - t1) <= 1e-12 * t1
    a, r = H.inner_aos(b, fmx.get("U"), 5), H.inner_aos(b, f64.get("U"), 5)
    num, den = np.abs(a - r).mean(axis=0), np.abs(r).mean(axis=0)
    assert np.all(num / den < 1e-5), num / den
    for nm in ("rho", "p", "u", "c", "H"):
        x, y = fmx.get(nm), f64.get(nm)
        assert np.abs(x - y).max() <= 1e-4 * np.abs(y).max(), nm
    f64.close(), fmx.close()


def _visc_case(name):
    """A viscous case and the reference's fitted transport data (from its golden fixture)."""
    import os
    z = np.load(os.path.join(H.GOLDEN, "visc_mixing5_12x8x6_janaf_w5.npz"))
    tr = H.transport_of(z)
    mk = {"visc3d": lambda: H.mixing_small((16, 12, 8), order=5),
          "visc2d_weno7": lambda: H.mixing_small((24, 16, 0), order=7),
          "visc3d_heat_only": lambda: H.mixing_small((12, 8, 6), order=5)}[name]
    b, s, th, U, T = mk()
    s.viscous = 3 if name == "visc3d_heat_only" else 7
    return b, s, th, U, T, tr


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("name", ["visc3d", "visc2d_weno7", "visc3d_heat_only"])
def test_viscous_stagewise_parity(name, precision, cuda_lib):
    """Viscous stress and heat conduction (and the diffusion terms, zero in a single block) agree
    with the oracle per stage; exp / log / pow differ from the host's by an ulp, so the bound is
    the parity bound, not bit equality."""
    from xfluids_gb300.fluid import Fluid
    b, s, th, U, T, tr = _visc_case(name)
    s.precision = precision
    run_stagewise((b, s, th, U, T), steps=2, precision=precision, transport=tr)
    # the graph replay against the free-running oracle (strict) or the same form's stage calls
    E = s.Emax
    f, g = Fluid(b, s, th), Fluid(b, s, th)
    o = Oracle(b, s, th, U, T, transport=tr)
    for h in (f, g):
        h.set_transport(tr)
        h.InitialU(U, T)
        h.initialize()
    o.initialize()
    for step in range(2):
        dt, dt_o = f.GetFluidDt(), o.get_dt()
        for flag in (1, 2, 3):
            f.stage(flag, dt)
            o.stage(flag, dt_o)
    st, t, n = g.advance(2)
    assert st == 0 and n == 2
    _check("graph U vs stage calls", H.inner_aos(b, g.get("U"), E), H.inner_aos(b, f.get("U"), E), E, tol=1e-15)
    if not needs_resync(s, precision):
        _check("graph U vs oracle", H.inner_aos(b, g.get("U"), E), H.inner_aos(b, o.get("U"), E), E)
    f.close(), g.close()


def test_viscous_needs_transport_and_a_mixture(cuda_lib):
    from xfluids_gb300.abi import XfgError
    from xfluids_gb300.fluid import Fluid
    b, s, th, U, T, tr = _visc_case("visc3d")
    f = Fluid(b, s, th)
    f.InitialU(U, T)
    f.initialize()
    with pytest.raises(XfgError):
        f.advance(1)                      # no transport data yet
    f.close()
    b2, s2, th2, U2, T2 = H.sod_like(64)
    s2.viscous = 1
    with pytest.raises(XfgError):
        Fluid(b2, s2, th2)                # single gas: no temperature for the transport fits


def test_mixed_viscous_close_to_fp64(cuda_lib):
    from xfluids_gb300.fluid import Fluid
    b, s, th, U, T, tr = _visc_case("visc3d")
    runs = {}
    for prec in (FP64, MIXED):
        s.precision = prec
        f = Fluid(b, s, th)
        f.set_transport(tr)
        f.InitialU(U, T)
        f.initialize()
        st, t, n = f.advance(3)
        assert st == 0
        runs[prec] = H.inner_aos(b, f.get("U"), 9)
        f.close()
    a, r = runs[MIXED], runs[FP64]
    num, den = np.abs(a - r).mean(axis=0), np.abs(r).mean(axis=0)
    rel = np.where(den > 0, num / np.where(den > 0, den, 1.0), num)
    assert np.all(rel < 1e-4), rel


def test_fp64_mixture_drift_against_strict(cuda_lib):
    """The FP64 form of a mixture (contracted face sweeps) running free next to the strict form:
    the difference stays at the level the temperature Newton's stopping test lets through."""
    b, s, th, U, T = H.mixing_small()
    E = s.Emax
    runs = {}
    for prec in (FP64, FP64_STRICT):
        s.precision = prec
        f = _fluid(b, s, th, U, T)
        f.initialize()
        st, t, n = f.advance(10)
        assert st == 0 and n == 10
        runs[prec] = H.inner_aos(b, f.get("U"), E)
        f.close()
    r = H.normwise(runs[FP64], runs[FP64_STRICT], E)
    l1 = np.abs(runs[FP64] - runs[FP64_STRICT]).mean(axis=0) / np.maximum(np.abs(runs[FP64_STRICT]).mean(axis=0), 1e-300)
    print(f"FP64 vs strict after 10 steps: normwise {r.max():.3e}, L1 relative {l1.max():.3e}")
    assert np.all(r <= 1e-8), r
