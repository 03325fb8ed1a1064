"""Shared test helpers: workload builders and the parity norm."""
from __future__ import annotations

import os

import numpy as np

from xfluids_gb300 import cases, thermo
from xfluids_gb300.abi import OUTFLOW, PERIODIC, SYMMETRY, SLIPWALL, LLF
from xfluids_gb300.mesh import make_block, make_scheme, empty_thermal

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
THERMO_JSON = os.path.join(GOLDEN, "thermo_tables.json")
TRANSPORT_JSON = os.path.join(GOLDEN, "transport_tables.json")

# per-stage parity bound of the FP64 path against the oracle (normwise relative, per component)
PARITY_TOL = 1e-12


def parity_tol(scheme):
    return PARITY_TOL


def thermal(species, th=1):
    return thermo.load_thermal(species, th, tables_json=THERMO_JSON)


def normwise(a, b, ncomp):
    """max over cells |a-b| / max over cells |b| for each component of AoS arrays."""
    a = np.asarray(a).reshape(-1, ncomp)
    b = np.asarray(b).reshape(-1, ncomp)
    num = np.abs(a - b).max(axis=0)
    den = np.abs(b).max(axis=0)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)


def inner_aos(block, arr, ncomp):
    a = np.asarray(arr).reshape(block.Zmax, block.Ymax, block.Xmax, ncomp)
    return a[block.inner_slices()].reshape(-1, ncomp)


def inner_soa(block, arr):
    a = np.asarray(arr).reshape(block.Zmax, block.Ymax, block.Xmax)
    return a[block.inner_slices()].reshape(-1)


def sod_like(n=128, order=5, artificial=LLF, bc=OUTFLOW):
    b, s, th, U, T = cases.sod(n, order=order)
    s.artificial_type = artificial
    for q in range(6):
        b.Boundarys[q] = bc
    return b, s, th, U, T


def riemann_small(n=48, seed=3, artificial=LLF, order=5, bc=OUTFLOW):
    rng = np.random.default_rng(seed)
    states = cases.riemann_states(rng)
    b, s, th, U, T = cases.riemann2d(n, states)
    s.artificial_type = artificial
    s.scheme_order = order
    for q in range(6):
        b.Boundarys[q] = bc
    return b, s, th, U, T


def blast3d(n=(20, 12, 10), order=5, bc=(OUTFLOW, OUTFLOW, SYMMETRY, SLIPWALL, PERIODIC, PERIODIC), artificial=LLF):
    """Small 3D single-gas problem with a smooth pressure bump and a shear (exercises all 3 sweeps
    and the non-periodic boundary kinds)."""
    b = make_block(n, (1.0, 0.6, 0.5), bc, cfl=0.5)
    s = make_scheme(cop=False, scheme_order=order, artificial_type=artificial)
    X, Y, Z = cases.cell_centres(b)
    r2 = (X - 0.5) ** 2 + (Y - 0.3) ** 2 + (Z - 0.25) ** 2
    rho = 1.0 + 0.5 * np.exp(-r2 / 0.02)
    p = 1.0 + 2.0 * np.exp(-r2 / 0.01)
    u = 0.3 * np.sin(2 * np.pi * Y)
    v = 0.2 * np.cos(2 * np.pi * Z)
    w = 0.1 * np.sin(2 * np.pi * X)
    U = cases.conserved_ideal(rho, u, v, w, p)
    return b, s, empty_thermal(), U, None


def mixing_small(shape=(24, 16, 8), order=7, thermo_kind=0, artificial=LLF):
    th = thermal(cases.MIXING_SPECIES, thermo_kind)
    b, s, th, U, T = cases.mixing_layer(shape, thermal=th, order=order, noise=0.05, thermo_kind=thermo_kind)
    s.artificial_type = artificial
    return b, s, th, U, T


def insert_st(n=200, order=5, ghost=True, thermo_kind=1):
    """1D 4-species (H2, O2, AR, N2) shock tube in a T/p jump, GhostSpecies like the reference's
    1d-mc-insert-shock-tube mixture (runtime.dat/1d-mc-insert-shock-tube)."""
    sp = ["H2", "O2", "AR", "N2"]
    th = thermal(sp, thermo_kind)
    b = make_block((n, 0, 0), (0.1, 1.0, 1.0), [OUTFLOW] * 6, cfl=0.5)
    s = make_scheme(cop=True, num_species=4, scheme_order=order, artificial_type=LLF, thermo=thermo_kind,
                    ghost_species=ghost)
    X, _, _ = cases.cell_centres(b)
    left = X < 0.05
    Y = np.zeros(X.shape + (4,))
    Y[..., 0] = np.where(left, 0.01, 0.03)
    Y[..., 1] = np.where(left, 0.2, 0.1)
    Y[..., 2] = np.where(left, 0.5, 0.6)
    Y[..., 3] = 1.0 - Y[..., :3].sum(-1) if not ghost else 0.0
    if ghost:
        Y[..., :3] /= Y[..., :3].sum(-1, keepdims=True)
    T = np.where(left, 1500.0, 400.0)
    p = np.where(left, 4.0e5, 1.0e5)
    R = thermo.RU * sum(Y[..., q] / th.Wi[q] for q in range(4))
    rho = p / (R * T)
    h = np.zeros_like(T)
    for q in range(4):
        h += Y[..., q] * cases.species_cp_h(th, q, T, nasa=bool(thermo_kind))[1]
    e = h - R * T
    U = np.concatenate([np.stack([rho, 0 * rho, 0 * rho, 0 * rho, rho * e], axis=-1), rho[..., None] * Y[..., :3]], axis=-1)
    return b, s, th, np.ascontiguousarray(U.reshape(-1, 8)), np.ascontiguousarray(T.reshape(-1))




def riemann_member(q, n, seed=0):
    """Quadrant states of member q of the seeded 256-member Riemann ensemble on an n^2 grid."""
    _, rng = cases.ensemble_sizes(256, seed)
    for _ in range(q):
        cases.riemann_states(rng)
    return cases.riemann2d(n, cases.riemann_states(rng))


def with_positivity(mk):
    def build():
        b, s, th, U, T = mk()
        s.positivity = 1
        return b, s, th, U, T
    return build


def riemann1d_strong(n=108):
    """1D two-state Riemann problem whose first RK stage drives the density negative without the
    positivity limiter (rho, u, p) = (1.84, -0.494, 0.0911) | (0.189, -0.503, 0.656)."""
    return cases.riemann1d(n, (1.8397073266913917, -0.4944626440950872, 0.09109694116558763),
                           (0.18863925211238564, -0.5028604535820342, 0.6556118842537302))


def with_order(mk, order):
    def build():
        b, s, th, U, T = mk()
        s.scheme_order = order
        return b, s, th, U, T
    return build


def with_viscous(mk, flags=7):
    def build():
        b, s, th, U, T = mk()
        s.viscous = flags
        return b, s, th, U, T
    return build


def transport_of(z):
    """xfg_transport from a fixture holding the reference's fitted transport data."""
    if "tr_visc" not in z:
        return None
    ns = z["tr_chara"].size // 9
    return thermo.transport_from_arrays(ns, z["tr_visc"], z["tr_therm"], z["tr_dkj"], z["tr_chara"], *z["tr_limits"])
