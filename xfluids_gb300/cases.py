"""Initial states of the benchmark workloads (synthetic, seeded, built on the host in numpy).

Each function returns (block, scheme, thermal, U, T): U in the reference layout (AoS, Emax per
cell, all cells including ghosts) and T the temperature that warm-starts the multi-component
Newton iteration (None without COP). The same arrays feed the CUDA path and the oracle.
"""
from __future__ import annotations

import math

import numpy as np

from .abi import OUTFLOW, PERIODIC, LLF
from .mesh import make_block, make_scheme, empty_thermal
from .thermo import RU


def cell_centres(b, domain_min=(0.0, 0.0, 0.0)):
    """Cell-centre coordinates on all cells, x = (i - Bwidth + 0.5) dx + xmin (as the samples'
    InitialUFKernel computes them)."""
    x = (np.arange(b.Xmax) - b.Bwidth_X + 0.5) * b.dx + domain_min[0] if b.DimX else np.zeros(1)
    y = (np.arange(b.Ymax) - b.Bwidth_Y + 0.5) * b.dy + domain_min[1] if b.DimY else np.zeros(1)
    z = (np.arange(b.Zmax) - b.Bwidth_Z + 0.5) * b.dz + domain_min[2] if b.DimZ else np.zeros(1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return X, Y, Z


def conserved_ideal(rho, u, v, w, p, gamma=1.4):
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    U = np.stack([rho, rho * u, rho * v, rho * w, E], axis=-1)
    return np.ascontiguousarray(U.reshape(-1, 5))


def isentropic_vortex(n=1024, cfl=0.5, precision=0, beta=5.0):
    """2D isentropic Euler vortex on the periodic [0,10]^2 (free stream rho=1, u=v=1, p=1),
    the formula of the reference sample 2D-EulerVortex/ini_sample.hpp:14-89."""
    b = make_block((n, n, 0), (10.0, 10.0, 1.0), [PERIODIC] * 6, cfl=cfl)
    s = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=precision)
    X, Y, _ = cell_centres(b)
    xv, yv = X - 5.0, Y - 5.0
    r2 = xv * xv + yv * yv
    inter1 = beta * beta * np.exp(1.0 - r2) / 28.0 / math.pi / math.pi
    inter2 = 0.5 * beta * np.exp(0.5 * (1.0 - r2)) / math.pi
    rho = (1.0 - inter1) ** 2.5
    p = rho ** 1.4
    u = 1.0 - inter2 * yv
    v = 1.0 + inter2 * xv
    U = conserved_ideal(rho, u, v, np.zeros_like(u), p)
    return b, s, empty_thermal(), U, None


def isentropic_vortex_exact(b, t, beta=5.0):
    """Exact density of the vortex at time t: the initial vortex carried by the free stream
    (1, 1) on the periodic [0,10]^2."""
    X, Y, _ = cell_centres(b)
    xv = np.mod(X - t, 10.0) - 5.0
    yv = np.mod(Y - t, 10.0) - 5.0
    r2 = xv * xv + yv * yv
    return (1.0 - beta * beta * np.exp(1.0 - r2) / 28.0 / math.pi / math.pi) ** 2.5


def sod(n=1024, cfl=0.5, precision=0, order=5):
    """1D Sod shock tube on [0,1]: (1, 0, 1) | (0.125, 0, 0.1) at x = 0.5, transmissive ends."""
    b = make_block((n, 0, 0), (1.0, 1.0, 1.0), [OUTFLOW] * 6, cfl=cfl)
    s = make_scheme(cop=False, scheme_order=order, artificial_type=LLF, precision=precision)
    X, _, _ = cell_centres(b)
    left = X < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    z = np.zeros_like(rho)
    U = conserved_ideal(rho, z, z, z, p)
    return b, s, empty_thermal(), U, None


def sod_exact_density(x, t, gamma=1.4):
    """Exact density of the Sod problem at time t (interface at x = 0.5): the star pressure from
    Newton's method on the pressure functions of the exact Riemann solver (Toro, ch. 4), then a
    left rarefaction, the contact and a right shock."""
    rl, pl, rr, pr = 1.0, 1.0, 0.125, 0.1
    g = gamma
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)

    def f(p, rk, pk, ck):
        if p > pk:
            A, B = 2 / ((g + 1) * rk), (g - 1) / (g + 1) * pk
            return (p - pk) * math.sqrt(A / (p + B))
        return 2 * ck / (g - 1) * ((p / pk) ** ((g - 1) / (2 * g)) - 1)

    p = 0.3
    for _ in range(100):
        F = f(p, rl, pl, cl) + f(p, rr, pr, cr)
        dp = 1e-7
        dF = (f(p + dp, rl, pl, cl) + f(p + dp, rr, pr, cr) - F) / dp
        p -= F / dF
    u = 0.5 * (f(p, rr, pr, cr) - f(p, rl, pl, cl))
    rstar_l = rl * (p / pl) ** (1 / g)
    rstar_r = rr * ((p / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * p / pr + 1))
    shock = math.sqrt((g + 1) / (2 * g) * p / pr + (g - 1) / (2 * g)) * cr
    cstar = cl * (p / pl) ** ((g - 1) / (2 * g))
    s = (np.asarray(x, dtype=np.float64) - 0.5) / t
    c_fan = 2 / (g + 1) * (cl - (g - 1) / 2 * s)
    fan = rl * np.maximum(c_fan / cl, 0.0) ** (2 / (g - 1))
    return np.select([s < -cl, s < u - cstar, s < u, s < shock], [rl, fan, rstar_l, rstar_r], rr)


def riemann_states(rng):
    """Four quadrant states (rho, u, v, p): rho in U[0.1,2], u,v in U[-1,1], p in U[0.05,2]."""
    q = np.empty((4, 4))
    q[:, 0] = rng.uniform(0.1, 2.0, 4)
    q[:, 1] = rng.uniform(-1.0, 1.0, 4)
    q[:, 2] = rng.uniform(-1.0, 1.0, 4)
    q[:, 3] = rng.uniform(0.05, 2.0, 4)
    return q


def riemann2d(n, states, cfl=0.45, precision=0):
    """2D four-quadrant Riemann problem on [0,1]^2 split at (0.5, 0.5), outflow boundaries.
    states[q] = (rho, u, v, p) for quadrants q = 0 (x>.5,y>.5), 1 (x<.5,y>.5), 2 (x<.5,y<.5),
    3 (x>.5,y<.5)."""
    b = make_block((n, n, 0), (1.0, 1.0, 1.0), [OUTFLOW] * 6, cfl=cfl)
    s = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=precision)
    X, Y, _ = cell_centres(b)
    quad = np.where(X > 0.5, np.where(Y > 0.5, 0, 3), np.where(Y > 0.5, 1, 2))
    st = np.asarray(states)[quad]
    U = conserved_ideal(st[..., 0], st[..., 1], st[..., 2], np.zeros_like(X), st[..., 3])
    return b, s, empty_thermal(), U, None


def riemann1d(n, left, right, cfl=0.5, precision=0):
    """1D two-state Riemann problem on [0,1] split at x = 0.5, transmissive ends (the Sod layout
    with arbitrary states): left/right = (rho, u, p)."""
    b = make_block((n, 0, 0), (1.0, 1.0, 1.0), [OUTFLOW] * 6, cfl=cfl)
    s = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=precision)
    X, _, _ = cell_centres(b)
    lft = X < 0.5
    rho = np.where(lft, left[0], right[0])
    u = np.where(lft, left[1], right[1])
    p = np.where(lft, left[2], right[2])
    z = np.zeros_like(rho)
    U = conserved_ideal(rho, u, z, z, p)
    return b, s, empty_thermal(), U, None


def ensemble_sizes(count=256, seed=0, lo=7.0, hi=10.0):
    """Cells per side N = round(2^U[lo,hi]) for each ensemble member, seeded."""
    rng = np.random.default_rng(seed)
    return np.rint(2.0 ** rng.uniform(lo, hi, count)).astype(int), rng


def riemann_ensemble(count=256, seed=0, lo=7.0, hi=10.0, precision=0):
    """Batched ensemble of independent 2D four-quadrant Riemann problems: N per side
    round(2^U[lo,hi]), quadrant states as riemann_states, CFL 0.45, outflow. Returns the scheme
    and a list of (block, U)."""
    sizes, rng = ensemble_sizes(count, seed, lo, hi)
    members = []
    for n in sizes:
        b, s, _, U, _ = riemann2d(int(n), riemann_states(rng), precision=precision)
        members.append((b, U))
    return make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=precision), members


# ---------------------------------------------------------------------------------------------
# multi-component mixing layer
# ---------------------------------------------------------------------------------------------
MIXING_SPECIES = ["H2", "O2", "N2", "H2O", "AR"]


def _hash_uniform(seed, i, j, k):
    """Counter-based uniform in [-1, 1) from (seed, i, j, k): splitmix64 of the packed counter, so
    the perturbation is identical wherever it is generated."""
    with np.errstate(over="ignore"):
        x = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)
             + (i.astype(np.uint64) << np.uint64(42)) + (j.astype(np.uint64) << np.uint64(21))
             + k.astype(np.uint64))
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return (x >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def species_cp_h(thermal, n, T, nasa=False):
    """Cp_i and h_i of species n (J/kg/K, J/kg) for T >= 200 K from the NASA-9 (nasa=True) or
    JANAF / NASA-7 table, the polynomials of the reference's Thermo_device.h:10-102."""
    a = np.array(thermal.Hia[n * 21:(n + 1) * 21]).reshape(7, 3)
    Ri = thermal.Ri[n]
    if not nasa:
        c = np.where((T > 1000.0)[..., None], a[:, 0], a[:, 1])
        cp = Ri * (c[..., 0] + (c[..., 1] + (c[..., 2] + (c[..., 3] + c[..., 4] * T) * T) * T) * T)
        h = Ri * (T * (c[..., 0] + T * (c[..., 1] * 0.5 + T * (c[..., 2] / 3.0 + T * (c[..., 3] * 0.25 + c[..., 4] * T * 0.2)))) + c[..., 5])
        return cp, h
    rg = np.where(T >= 6000.0, 2, np.where(T >= 1000.0, 1, 0))
    c = a[:, rg]                       # (7, ...) coefficients of the range of each cell
    b0 = np.array(thermal.Hib[n * 6:(n + 1) * 6]).reshape(2, 3)[0][rg]
    _T = 1.0 / T
    cp = Ri * ((c[0] * _T + c[1]) * _T + c[2] + (c[3] + (c[4] + (c[5] + c[6] * T) * T) * T) * T)
    h = Ri * (-c[0] / T + c[1] * np.log(T) + (c[2] + (0.5 * c[3] + (c[4] / 3.0 + (0.25 * c[5] + 0.2 * c[6] * T) * T) * T) * T) * T + b0)
    return cp, h


def mixing_layer(shape=(512, 256, 256), thermal=None, length=0.01, seed=1234, precision=0, order=7,
                 noise=0.01, ybc=OUTFLOW, thermo_kind=0):
    """3D inert temporal mixing layer of 5 species (H2, O2, N2, H2O, AR), NASA-7 thermo.

    Domain [0, L] x [0, L*ny/nx] x [0, L*nz/nx]. Upper stream (y > mid): Y_O2 = 0.233,
    Y_N2 = 0.767 at 1200 K, Mach +0.6; lower stream: Y_H2 = 0.05, Y_N2 = 0.95 at 300 K,
    Mach -0.6; tanh blend of thickness 0.01 L; p = 1 atm; velocity perturbed by `noise` times
    the local speed with a counter-based hash of (seed, i, j, k). Periodic in x and z; in y
    `ybc` (outflow by default; with PERIODIC the ghost rows start as the periodic images).
    """
    nx, ny, nz = shape
    dom = (length, length * ny / nx, length * nz / nx)
    b = make_block((nx, ny, nz), dom, [PERIODIC, PERIODIC, ybc, ybc, PERIODIC, PERIODIC], cfl=0.5)
    s = make_scheme(cop=True, num_species=5, scheme_order=order, artificial_type=LLF, thermo=thermo_kind,
                    ghost_species=False, precision=precision)
    # the mean state depends on y only: build it on the y column, then broadcast (same values as
    # evaluating every cell)
    jy = np.arange(b.Ymax) - b.Bwidth_Y
    if ybc == PERIODIC:
        # ghost rows hold their periodic images, so that the initial T (the warm start of the
        # clamped temperature Newton iteration) agrees with the state the boundary fill puts there
        jy = np.mod(jy, ny)
    Y = (jy + 0.5) * b.dy
    ymid = 0.5 * dom[1]
    wgt = 0.5 * (1.0 + np.tanh((Y - ymid) / (0.01 * length)))  # 1 upper, 0 lower
    y_up = np.array([0.0, 0.233, 0.767, 0.0, 0.0])
    y_lo = np.array([0.05, 0.0, 0.95, 0.0, 0.0])
    Ys = wgt[..., None] * y_up + (1.0 - wgt[..., None]) * y_lo
    T = 300.0 + wgt * (1200.0 - 300.0)
    p = 101325.0
    Rmix = RU * sum(Ys[..., n] / thermal.Wi[n] for n in range(5))
    rho = p / (Rmix * T)
    cph = [species_cp_h(thermal, n, T, nasa=bool(thermo_kind)) for n in range(5)]
    cp = sum(Ys[..., n] * cph[n][0] for n in range(5))
    h = sum(Ys[..., n] * cph[n][1] for n in range(5))
    gam = cp / (cp - Rmix)
    c = np.sqrt(gam * Rmix * T)
    c_up = float(np.sqrt(gam.max() * Rmix.min() * 1200.0))
    c_lo = float(np.sqrt(gam.min() * Rmix.max() * 300.0))
    u0 = wgt * (0.6 * c_up) + (1.0 - wgt) * (-0.6 * c_lo)
    col = lambda a: a[None, :, None]  # (Zmax, Ymax, Xmax) broadcast of a y column
    kk, jj, ii = np.meshgrid(np.arange(b.Zmax), np.arange(b.Ymax), np.arange(b.Xmax), indexing="ij")
    amp = col(noise * c)
    u = col(u0) + amp * _hash_uniform(seed, ii, jj, kk)
    v = amp * _hash_uniform(seed + 1, ii, jj, kk)
    w = amp * _hash_uniform(seed + 2, ii, jj, kk)
    del kk, jj, ii
    e = h - Rmix * T
    rho3 = np.broadcast_to(col(rho), u.shape)
    Et = rho3 * (col(e) + 0.5 * (u * u + v * v + w * w))
    U = np.empty(u.shape + (9,))
    U[..., 0] = rho3
    U[..., 1] = rho3 * u
    U[..., 2] = rho3 * v
    U[..., 3] = rho3 * w
    U[..., 4] = Et
    for n in range(4):
        U[..., 5 + n] = col(rho * Ys[..., n])
    U = U.reshape(-1, 9)
    T = np.ascontiguousarray(np.broadcast_to(col(T), u.shape))
    return b, s, thermal, U, np.ascontiguousarray(T.reshape(-1))
