"""Seeded random cases against the oracle, stage by stage (the bound and the comparison of
test_parity_gpu.run_stagewise): dimension 1 / 2 / 3 with small sizes, WENO5 / WENO-CU6 / WENO7,
LLF / Roe / GLF splitting, a boundary kind per side (periodic per axis), single gas or the
5-species mixture (JANAF or NASA-9), the positivity limiter on or off; smooth states with a mild
jump, so that every case runs without a numerical stop.

The ghost cells of a mixture start with the temperature of the cell the boundary fill copies into
them (the warm start of the temperature Newton iteration). Across a mirror or outflow boundary the
two cells of the wall face then carry the same bits and the Roe-linearised sound speed sees zero
jumps; with a warm start that differs between them, each side's Newton ends a few ulps apart and
that face's sound-speed correction divides the difference by the sum of squared jumps (+1e-19),
which turns last-bit noise (the GPU's log against the host's, NASA-9) into 1e-4 flux changes.
"""
import numpy as np
import pytest

import helpers as H
from test_parity_gpu import run_stagewise
from xfluids_gb300 import cases, thermo
from xfluids_gb300.abi import (FP64, FP64_STRICT, GLF, INFLOW, LLF, NSLIPWALL, OUTFLOW, PERIODIC, ROE,
                               SLIPWALL, SYMMETRY, VISCWALL)
from xfluids_gb300.mesh import empty_thermal, make_block, make_scheme

pytestmark = pytest.mark.gpu

SIDES = [OUTFLOW, SYMMETRY, SLIPWALL, NSLIPWALL, VISCWALL, INFLOW]


def _field(rng, b, X, Y, Z, base, amp, jump):
    """base * (1 + smooth modes + a step of relative size `jump` across a random plane)."""
    f = np.zeros_like(X)
    for _ in range(3):
        k = rng.integers(1, 4, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        f += rng.uniform(-amp, amp) * np.sin(2 * np.pi * k[0] * X + ph[0]) * np.sin(2 * np.pi * k[1] * Y + ph[1]) * \
            np.cos(2 * np.pi * k[2] * Z + ph[2])
    nrm = rng.normal(size=3)
    plane = nrm[0] * (X - 0.5) + nrm[1] * (Y - 0.5) * b.DimY + nrm[2] * (Z - 0.5) * b.DimZ
    return base * (1.0 + f + jump * (plane > 0))


def fill_ghosts_like_bc(b, A):
    """Copy into the ghost cells of the per-cell field A (Zmax, Ymax, Xmax) the cell the boundary
    fill of U copies there (FluidBCKernelX/Y/Z, X then Y then Z; Y and Z leave viscWall and
    slipWall ghosts alone)."""
    dims, bws, inner = (b.DimX, b.DimY, b.DimZ), (b.Bwidth_X, b.Bwidth_Y, b.Bwidth_Z), (b.X_inner, b.Y_inner, b.Z_inner)
    for d in range(3):
        if not dims[d]:
            continue
        ax = 2 - d  # numpy axis of direction d
        bw, n = bws[d], inner[d]
        nmax = n + 2 * bw
        for side in range(2):
            kind = b.Boundarys[2 * d + side]
            for g in range(bw):
                cn = g if side == 0 else g + nmax - bw
                mo = 0 if side == 0 else n
                if kind == PERIODIC:
                    src = cn + n if side == 0 else cn - n
                elif kind == OUTFLOW:
                    src = bw if side == 0 else nmax - bw - 1
                elif kind == SYMMETRY or kind == NSLIPWALL or (d == 0 and kind in (SLIPWALL, VISCWALL)):
                    src = 2 * (bw + mo) - 1 - cn
                else:
                    continue
                dst = [slice(None)] * 3
                srs = [slice(None)] * 3
                dst[ax], srs[ax] = cn, src
                A[tuple(dst)] = A[tuple(srs)]
    return A


def random_case(seed, cop=None, order=None, art=None, pos=None, thermo_kind=None):
    """Seeded random block, boundary kinds, scheme and state. The keyword arguments, when given,
    replace the drawn choice after it was drawn, so the other draws of a seed stay the same."""
    rng = np.random.default_rng(7000 + seed)
    ndim = int(rng.choice([1, 2, 3], p=[0.3, 0.4, 0.3]))
    res = {1: lambda: (int(rng.integers(16, 65)), 0, 0), 2: lambda: (int(rng.integers(12, 41)), int(rng.integers(12, 41)), 0),
           3: lambda: tuple(int(x) for x in rng.integers(8, 17, 3))}[ndim]()
    bc = []
    for a in range(3):
        if rng.random() < 0.3:
            bc += [PERIODIC, PERIODIC]
        else:
            bc += [int(rng.choice(SIDES)), int(rng.choice(SIDES))]
    drawn = (rng.random() < 0.35, int(rng.choice([5, 6, 7])), int(rng.choice([LLF, ROE, GLF])),
             bool(rng.random() < 0.3))
    cop, order, art, pos = (d if o is None else o for d, o in zip(drawn, (cop, order, art, pos)))
    b = make_block(res, (1.0, 1.0, 1.0), bc, cfl=float(rng.uniform(0.3, 0.6)))
    X, Y, Z = cases.cell_centres(b)
    vel = [_field(rng, b, X, Y, Z, 1.0, 0.3, 0.0) - 1.0 for _ in range(3)]
    if not cop:
        s = make_scheme(cop=False, scheme_order=order, artificial_type=art, positivity=pos)
        rho = _field(rng, b, X, Y, Z, 1.0, 0.15, float(rng.uniform(-0.4, 0.4)))
        p = _field(rng, b, X, Y, Z, 1.0, 0.15, float(rng.uniform(-0.4, 0.4)))
        u, v, w = [0.5 * vv if d else 0.0 * vv for vv, d in zip(vel, (b.DimX, b.DimY, b.DimZ))]
        return b, s, empty_thermal(), cases.conserved_ideal(rho, u, v, w, p), None
    tk = int(rng.integers(0, 2))
    tk = tk if thermo_kind is None else thermo_kind
    th = H.thermal(cases.MIXING_SPECIES, tk)
    s = make_scheme(cop=True, num_species=5, scheme_order=order, artificial_type=art, thermo=tk,
                    ghost_species=False, positivity=pos)
    T = fill_ghosts_like_bc(b, _field(rng, b, X, Y, Z, 800.0, 0.2, float(rng.uniform(-0.4, 0.4))))
    p = _field(rng, b, X, Y, Z, 1.0e5, 0.1, float(rng.uniform(-0.2, 0.2)))
    Yw = np.stack([_field(rng, b, X, Y, Z, float(rng.uniform(0.2, 1.0)), 0.2, float(rng.uniform(-0.3, 0.3)))
                   for _ in range(5)], axis=-1)
    Ys = Yw / Yw.sum(-1, keepdims=True)
    R = thermo.RU * sum(Ys[..., q] / th.Wi[q] for q in range(5))
    rho = p / (R * T)
    h = sum(Ys[..., q] * cases.species_cp_h(th, q, T, nasa=bool(tk))[1] for q in range(5))
    u, v, w = [60.0 * vv if d else 0.0 * vv for vv, d in zip(vel, (b.DimX, b.DimY, b.DimZ))]
    E = rho * (h - R * T + 0.5 * (u * u + v * v + w * w))
    U = np.concatenate([np.stack([rho, rho * u, rho * v, rho * w, E], axis=-1), rho[..., None] * Ys[..., :4]], axis=-1)
    return b, s, th, np.ascontiguousarray(U.reshape(-1, 9)), np.ascontiguousarray(T.reshape(-1))


GHOST_SPECIES = ["H2", "O2", "AR", "N2"]


def ghost_species_case(seed):
    """Random block and boundary kinds of random_case(seed) with a random 4-species NASA-9 state
    (H2, O2, AR, N2), the last species a ghost species (not transported: its mass fraction is
    1 minus the others)."""
    b, _, _, _, _ = random_case(seed, cop=False, order=5, art=LLF, pos=False)
    rng = np.random.default_rng(9000 + seed)
    th = H.thermal(GHOST_SPECIES, 1)
    s = make_scheme(cop=True, num_species=4, scheme_order=5, artificial_type=LLF, thermo=1, ghost_species=True)
    X, Y, Z = cases.cell_centres(b)
    T = fill_ghosts_like_bc(b, _field(rng, b, X, Y, Z, 900.0, 0.2, float(rng.uniform(-0.4, 0.4))))
    p = _field(rng, b, X, Y, Z, 1.0e5, 0.1, float(rng.uniform(-0.2, 0.2)))
    Ys = np.stack([_field(rng, b, X, Y, Z, float(rng.uniform(0.05, 0.3)), 0.2, float(rng.uniform(-0.3, 0.3)))
                   for _ in range(3)], axis=-1)
    Ys = np.concatenate([Ys, 1.0 - Ys.sum(-1, keepdims=True)], axis=-1)
    R = thermo.RU * sum(Ys[..., q] / th.Wi[q] for q in range(4))
    rho = p / (R * T)
    h = sum(Ys[..., q] * cases.species_cp_h(th, q, T, nasa=True)[1] for q in range(4))
    u, v, w = [60.0 * (_field(rng, b, X, Y, Z, 1.0, 0.3, 0.0) - 1.0) * d for d in (b.DimX, b.DimY, b.DimZ)]
    E = rho * (h - R * T + 0.5 * (u * u + v * v + w * w))
    U = np.concatenate([np.stack([rho, rho * u, rho * v, rho * w, E], axis=-1), rho[..., None] * Ys[..., :3]], axis=-1)
    return b, s, th, np.ascontiguousarray(U.reshape(-1, 8)), np.ascontiguousarray(T.reshape(-1))


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("seed", range(16))
def test_random_case_matches_oracle(seed, precision, cuda_lib):
    b, s, th, U, T = random_case(seed)
    worst = run_stagewise((b, s, th, U, T), steps=2, precision=precision)
    print(f"seed {seed}: dims {b.DimX}{b.DimY}{b.DimZ} cop {s.cop} order {s.scheme_order} art {s.artificial_type} "
          f"pos {s.positivity} bc {list(b.Boundarys)}: worst {worst:.2e}")


def _advance(case, precision, steps):
    from xfluids_gb300.fluid import Fluid
    b, s, th, U, T = case
    s.precision = precision
    f = Fluid(b, s, th)
    try:
        f.InitialU(U, T)
        f.initialize()
        st, t, n = f.advance(steps)
        assert st == 0 and n == steps, (st, n)
        return H.inner_aos(b, f.get("U"), s.Emax), t
    finally:
        f.close()


@pytest.mark.parametrize("seed", range(16))
def test_random_case_mixed_close_to_fp64(seed, cuda_lib):
    """The mixed form on the same random cases: L1 of the state after 2 steps against the FP64
    form, per component over its state scale (density for the density and the species, the mean
    momentum magnitude for the momenta, the mean energy), within 1e-5."""
    from xfluids_gb300.abi import MIXED
    case = random_case(seed)
    ref, t64 = _advance(case, FP64, 2)
    got, tmx = _advance(random_case(seed), MIXED, 2)
    assert abs(tmx - t64) <= 1e-5 * t64
    d = np.abs(got - ref).mean(axis=0)
    rho = np.abs(ref[:, 0]).mean()
    mom = np.sqrt((ref[:, 1:4] ** 2).sum(axis=1)).mean()
    scale = np.array([rho, mom, mom, mom, np.abs(ref[:, 4]).mean()] + [rho] * (ref.shape[1] - 5))
    rel = d / scale
    print(f"seed {seed}: mixed vs FP64 state-scaled L1 {rel.max():.2e}")
    assert np.all(rel <= 1e-5), rel


def _tiny_case(res, dom, bc, order, cop=False):
    rng = np.random.default_rng(sum(res) * 31 + order)
    b = make_block(res, dom, bc, cfl=0.5)
    X, Y, Z = cases.cell_centres(b)
    vel = [_field(rng, b, X, Y, Z, 1.0, 0.3, 0.0) - 1.0 for _ in range(3)]
    u, v, w = [0.4 * vv if d else 0.0 * vv for vv, d in zip(vel, (b.DimX, b.DimY, b.DimZ))]
    if not cop:
        s = make_scheme(cop=False, scheme_order=order)
        rho = _field(rng, b, X, Y, Z, 1.0, 0.1, 0.2)
        p = _field(rng, b, X, Y, Z, 1.0, 0.1, -0.2)
        return b, s, empty_thermal(), cases.conserved_ideal(rho, u, v, w, p), None
    th = H.thermal(cases.MIXING_SPECIES, 0)
    s = make_scheme(cop=True, num_species=5, scheme_order=order, thermo=0, ghost_species=False)
    T = fill_ghosts_like_bc(b, _field(rng, b, X, Y, Z, 700.0, 0.1, 0.2))
    p = _field(rng, b, X, Y, Z, 1.0e5, 0.05, 0.1)
    Ys = np.stack([_field(rng, b, X, Y, Z, 0.2 + 0.1 * q, 0.1, 0.1) for q in range(5)], axis=-1)
    Ys = Ys / Ys.sum(-1, keepdims=True)
    R = thermo.RU * sum(Ys[..., q] / th.Wi[q] for q in range(5))
    rho = p / (R * T)
    h = sum(Ys[..., q] * cases.species_cp_h(th, q, T, nasa=False)[1] for q in range(5))
    E = rho * (h - R * T + 0.5 * (3600 * (u * u + v * v + w * w)))
    U = np.concatenate([np.stack([rho, 60 * rho * u, 60 * rho * v, 60 * rho * w, E], axis=-1),
                        rho[..., None] * Ys[..., :4]], axis=-1)
    return b, s, th, np.ascontiguousarray(U.reshape(-1, 9)), np.ascontiguousarray(T.reshape(-1))


TINY = {
    "1d_min_periodic_w7": ((4, 0, 0), (1.0, 1.0, 1.0), [PERIODIC] * 6, 7, False),
    "1d_min_outflow_w5": ((4, 0, 0), (1.0, 1.0, 1.0), [OUTFLOW] * 6, 5, False),
    "2d_min_walls_w7": ((4, 4, 0), (1.0, 3.0, 1.0), [SYMMETRY, NSLIPWALL, SLIPWALL, OUTFLOW, 0, 0], 7, False),
    "2d_ragged_w6": ((5, 7, 0), (0.7, 1.9, 1.0), [PERIODIC, PERIODIC, OUTFLOW, SYMMETRY, 0, 0], 6, False),
    "3d_min_w5": ((4, 4, 4), (1.0, 2.0, 0.5), [PERIODIC, PERIODIC, OUTFLOW, OUTFLOW, SYMMETRY, NSLIPWALL], 5, False),
    "3d_ragged_w7": ((5, 6, 7), (1.0, 1.3, 0.4), [OUTFLOW, SLIPWALL, PERIODIC, PERIODIC, INFLOW, OUTFLOW], 7, False),
    "3d_min_mixture_w7": ((4, 4, 4), (0.01, 0.02, 0.01), [PERIODIC, PERIODIC, OUTFLOW, NSLIPWALL, SYMMETRY, OUTFLOW], 7, True),
    "2d_ragged_mixture_w5": ((5, 9, 0), (0.01, 0.013, 1.0), [SLIPWALL, OUTFLOW, PERIODIC, PERIODIC, 0, 0], 5, True),
}


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("name", list(TINY))
def test_smallest_and_ragged_blocks_match_oracle(name, precision, cuda_lib):
    """Blocks at the minimum size (inner = Bwidth = 4 per active direction), odd and unequal sizes,
    unequal spacings."""
    res, dom, bc, order, cop = TINY[name]
    worst = run_stagewise(_tiny_case(res, dom, bc, order, cop), steps=2, precision=precision)
    print(f"{name}: worst {worst:.2e}")


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("seed", range(8))
def test_random_viscous_case_matches_oracle(seed, precision, cuda_lib):
    """Viscous stress, heat conduction and species diffusion on the random blocks and boundary
    kinds of the reference-pinned viscous cases (walls, inflow, symmetry included; the 5-species
    JANAF mixture, WENO5 LLF), with transport data fitted for the block's spacing."""
    from xfluids_gb300 import transport
    b, s, th, U, T = random_case(200 + seed, cop=True, order=5, art=LLF, pos=False, thermo_kind=0)
    s.viscous = 7
    tr = transport.fit_transport(cases.MIXING_SPECIES, th, 0, tables_json=H.TRANSPORT_JSON,
                                 inv_spacing=(b._dx, b._dy, b._dz))
    worst = run_stagewise((b, s, th, U, T), steps=2, precision=precision, transport=tr)
    print(f"viscous seed {seed}: dims {b.DimX}{b.DimY}{b.DimZ} bc {list(b.Boundarys)}: worst {worst:.2e}")


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
@pytest.mark.parametrize("seed", range(8))
def test_random_ghost_species_case_matches_oracle(seed, precision, cuda_lib):
    """GhostSpecies (renormalised mass fractions written back into U) with NASA-9 polynomials on
    the random blocks and boundary kinds of the reference-pinned GhostSpecies cases."""
    b, s, th, U, T = ghost_species_case(300 + seed)
    worst = run_stagewise((b, s, th, U, T), steps=2, precision=precision)
    print(f"ghost seed {seed}: dims {b.DimX}{b.DimY}{b.DimZ} bc {list(b.Boundarys)}: worst {worst:.2e}")
