"""Size-independent properties of the CUDA path at the benchmark sizes, where the oracle is too slow
for a stage-by-stage comparison:

- conservation: on a periodic domain the flux divergence telescopes, so the sum of every conserved
  component over the inner cells changes only by rounding (4096^2 vortex; 512x256x256 five-species
  mixing layer made periodic in y, inviscid and with viscous stress and heat conduction);
- free-stream preservation: the right-hand side of a uniform periodic state is exactly zero (every
  face flux is the same number);
- checkpoint round trip: a state written and read back is the same state, and continues bit for
  bit like a run set to that state.
"""
import numpy as np
import pytest

import helpers as H
from xfluids_gb300 import cases
from xfluids_gb300.abi import FP64, MIXED, PERIODIC
from xfluids_gb300.mesh import make_block, make_scheme, empty_thermal

pytestmark = pytest.mark.gpu

# relative change of a conserved sum over a few steps: rounding of the stage updates only
CONSERVATION_TOL = {FP64: 1e-12, MIXED: 1e-10}


def _sums(b, f, E):
    """Per-component sums over the inner cells. Each component is summed as one contiguous row
    (numpy's pairwise summation, error ~eps*log2(N)); a reduction over axis 0 of the (cells, E)
    array would add the rows one after another and its rounding (~N*eps for positive values,
    1e-10 at 33 M cells) would swamp the property checked here."""
    U = np.ascontiguousarray(H.inner_aos(b, f.get("U"), E).T)
    return U.sum(axis=1), np.abs(U).sum(axis=1)


def _run_conservation(b, s, th, U, T, steps, transport=None):
    from xfluids_gb300.fluid import Fluid
    E = s.Emax
    f = Fluid(b, s, th)
    try:
        if transport is not None:
            f.set_transport(transport)
        f.InitialU(U, T)
        f.initialize()
        s0, a0 = _sums(b, f, E)
        st, t, n = f.advance(steps)
        assert st == 0 and n == steps, (st, n)
        s1, _ = _sums(b, f, E)
        U1 = H.inner_aos(b, f.get("U"), E)
        assert np.all(np.isfinite(U1))
    finally:
        f.close()
    live = a0 > 0
    rel = np.abs(s1 - s0)[live] / a0[live]
    return rel


@pytest.mark.parametrize("precision", [FP64, MIXED], ids=["fp64", "mixed"])
def test_vortex_4096_conserves(precision, cuda_lib):
    b, s, th, U, T = cases.isentropic_vortex(4096, precision=precision)
    rel = _run_conservation(b, s, th, U, T, steps=3)
    assert np.all(rel <= CONSERVATION_TOL[precision]), rel


@pytest.mark.parametrize("precision", [FP64, MIXED], ids=["fp64", "mixed"])
def test_free_stream_4096(precision, cuda_lib):
    """Every stage's right-hand side of a uniform periodic state is exactly zero; the state itself
    moves only by the rounding of the RK combinations (0.75 U + 0.25 U1, U/3 + 2 U1/3)."""
    from xfluids_gb300.fluid import Fluid
    n = 4096
    b = make_block((n, n, 0), (10.0, 10.0, 1.0), [PERIODIC] * 6, cfl=0.5)
    s = make_scheme(cop=False, scheme_order=5, precision=precision)
    m = b.Xmax * b.Ymax
    one = np.ones(m)
    U = cases.conserved_ideal(1.0 * one, 0.3 * one, -0.2 * one, 0.0 * one, 1.0 * one)
    U0 = H.inner_aos(b, U, 5)
    f = Fluid(b, s, empty_thermal())
    try:
        f.InitialU(U)
        f.initialize()
        for step in range(2):
            dt = f.GetFluidDt()
            for flag in (1, 2, 3):
                f.stage(flag, dt)
                assert not np.any(f.get("LU")), f"step {step} stage {flag}: non-zero LU"
        got = H.inner_aos(b, f.get("U"), 5)
    finally:
        f.close()
    assert np.all(np.abs(got - U0) <= 8 * np.finfo(np.float64).eps * np.abs(U0))


def _mixing_periodic(precision, viscous=0):
    th = H.thermal(cases.MIXING_SPECIES, 0)
    b, s, th, U, T = cases.mixing_layer((512, 256, 256), thermal=th, precision=precision, ybc=PERIODIC)
    s.viscous = viscous
    return b, s, th, U, T


def test_mixing_layer_512x256x256_conserves(cuda_lib):
    rel = _run_conservation(*_mixing_periodic(FP64), steps=2)
    assert np.all(rel <= CONSERVATION_TOL[FP64]), rel


def test_mixing_layer_512x256x256_viscous_mixed_conserves(cuda_lib):
    import os
    tr = H.transport_of(np.load(os.path.join(H.GOLDEN, "visc_mixing5_12x8x6_janaf_w5.npz")))
    rel = _run_conservation(*_mixing_periodic(MIXED, viscous=7), steps=2, transport=tr)
    assert np.all(rel <= CONSERVATION_TOL[MIXED]), rel


def test_checkpoint_round_trip_4096(cuda_lib, tmp_path):
    """A restart recomputes the primitives from the stored U (the reference's Read_Ubak followed by
    the initial UpdateStates), so the restarted run equals a run set to the same U, not the
    continuing one (whose first dt uses the previous stage's primitives)."""
    from xfluids_gb300.fluid import Fluid
    b, s, th, U, T = cases.isentropic_vortex(4096)
    path = tmp_path / "ubak.bin"
    f, g, h = Fluid(b, s, th), Fluid(b, s, th), Fluid(b, s, th)
    try:
        f.InitialU(U)
        f.initialize()
        f.advance(2)
        f.write_checkpoint(path, 2, 0.125, 1.5)
        Uf = f.get("U")
        g.InitialU(U)
        step, t, dur = g.read_checkpoint(path)
        assert (step, t, dur) == (2, 0.125, 1.5)
        g.initialize()
        # inner cells: the ghost layers of the continuing run hold the last stage's boundary fill
        assert np.array_equal(H.inner_aos(b, g.get("U"), 5), H.inner_aos(b, Uf, 5))
        h.InitialU(Uf)
        h.initialize()
        g.advance(2)
        h.advance(2)
        assert np.array_equal(H.inner_aos(b, g.get("U"), 5), H.inner_aos(b, h.get("U"), 5))
    finally:
        f.close()
        g.close()
        h.close()
