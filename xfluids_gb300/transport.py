"""Fitted transport coefficients of a mixture: a restatement of Setup::GetFitCoefficient
(src/read_ini/src/viscfit.cpp:148-196) and what it calls, so that a viscous scheme can be set up
without the reference's C++ Setup.

For each species k: ln(mu_k) and ln(kappa_k), and for each pair (k, j): ln(p D_kj), are fitted by
least squares as cubics in ln(T) over the temperature nodes (JSON "ViscosityFittingTnode",
src/read_ini/settings/read_json.cpp:70). The accurate values at the nodes are the Chapman-Enskog
forms of viscfit.cpp:436-555 with the collision integrals interpolated in the tables of
runtime.dat/collision_integral.dat (viscfit.cpp:347-434) and the Lennard-Jones data of
runtime.dat/transport_data.dat (src/read_ini/src/thermal.cpp:131-166).

Every expression keeps the reference's operation order in Python floats (IEEE double, no
contraction) with the same libm calls (math.log / exp / pow / sqrt), so the coefficients are those
of the reference's host build. For a reduced temperature between the table's last two nodes
(75 < T* < 100) the reference's Omega_interpolated reads one element past T_star (viscfit.cpp:
378-386, ti3 = 37) and one row past each Omega table: the element past T_star is the first member
of the next data member of Setup (Reaction::React_ThirdCoef, a pointer), whose bits read as a
double are zero or subnormal, and the rows past the tables are the members that follow them (the
same happens for a reduced dipole moment in the last interval of delta_star).

fit_transport takes the interpolation nodes inside the tables by default: a quadratic through the
last three nodes of T_star (and of delta_star) for a point in the last interval, the mathematically
intended interpolation. reference_layout=True reproduces the reference's reads past the tables
through the reference's member layout (_Fitter.mem) and with them the reference's fits of H2 and
of its pairs with N2 and O2, whose nodes at 3000 K fall there, bit for bit: a parity switch for the
comparisons with the reference build, not a modelling choice.
"""
from __future__ import annotations

import json
import math
import os


# src/include/global_setup.h:42-54
PI = 3.1415926535897932384626433832795
KB = 1.3806549 * 1.0e-16                      # erg/K
NA = 6.02214129 * 1.0e23
UNIVERSAL_GAS_CONST = 6.02214076e26 * 1.380649e-23  # Avogadro [1/kmol] * Boltzmann [J/K]
TNODE = [273.15, 500.0, 750.0, 1000.0, 1250.0, 1500.0, 1750.0, 2000.0, 2250.0, 2500.0, 2750.0, 3000.0, 5000.0]
ORDER = 4                                    # order_polynominal_fitted
GEO, EPS, DIAM, MUE, ALPHA, ZROT, WI, VIS, SID = range(9)  # Specie_chara (global_setup.h:135-146)


def _tokens(path):
    with open(path, "r", encoding="latin-1") as f:
        return f.read().split()


def read_transport_data(runtime_dir, species):
    """The 6 Lennard-Jones entries of each species (thermal.cpp:131-156): the first whitespace token
    equal to the name, then geo, eps/kB, sigma, dipole moment, polarizability, Zrot(298 K)."""
    tk = _tokens(os.path.join(runtime_dir, "transport_data.dat"))
    out = []
    for name in species:
        row = None
        for n, t in enumerate(tk):
            if t == "*END":
                break
            if t == name:
                row = [float(x) for x in tk[n + 1:n + 7]]
                break
        if row is None:
            raise KeyError(f"species {name} not in transport_data.dat")
        out.append(row)
    return out


def read_collision_integrals(runtime_dir):
    """Setup::ReadOmega_table (viscfit.cpp:347-365): 8 reduced dipole moments, then 37 rows of
    (T*, Omega(1,1) x 8), then 37 x 8 Omega(2,2)."""
    # the stream reads 8 + 37 x 9 + 37 x 8 numbers; text after them (notes) is never read
    tk = [float(x) for x in _tokens(os.path.join(runtime_dir, "collision_integral.dat"))[:8 + 37 * 9 + 37 * 8]]
    p = 0
    delta = tk[p:p + 8]
    p += 8
    tstar, om1 = [], []
    for _ in range(37):
        tstar.append(tk[p])
        om1.append(tk[p + 1:p + 9])
        p += 9
    om2 = [tk[p + 8 * i:p + 8 * i + 8] for i in range(37)]
    return {"delta_star": delta, "T_star": tstar, "omega": [om2, om1]}


def dump_transport_tables(runtime_dir, species, path):
    """Write the species rows and the collision tables to a JSON file (the inputs of fit())."""
    with open(path, "w") as f:
        json.dump({"species": list(species), "lj": read_transport_data(runtime_dir, species),
                   "collision": read_collision_integrals(runtime_dir)}, f, indent=1)


def _quad(x1, x2, x3, f1, f2, f3):
    """GetQuadraticInterCoeff (src/read_ini/mixture.hpp:43-48)."""
    a2 = ((f1 - f2) / (x1 - x2) - (f2 - f3) / (x2 - x3)) / (x1 - x3)
    a1 = (f1 - f2) / (x1 - x2) - a2 * (x1 + x2)
    a0 = f1 - a1 * x1 - a2 * x1 * x1
    return a0, a1, a2


def _zrot(x):
    """ZrotFunc (mixture.hpp:76-80)."""
    return 1.0 + math.sqrt(PI * x) * PI / 2.0 + x * (0.25 * PI * PI + 2.0) + math.pow(PI * x, 1.5)


class _Fitter:
    """The accurate transport properties and the fits, with the reference's member layout of the
    collision tables: Omega_table[2][37][8], then delta_star[8], then T_star[37] in one flat block
    (setupini.h:48-49), so that an index one past delta_star or past a table row reads what the
    reference reads there."""

    def __init__(self, chara, thermal, thermo_kind, coll, reference_layout=False):
        self.reference_layout = reference_layout
        self.chara = chara
        self.Hia = list(thermal.Hia)
        self.Ri = list(thermal.Ri)
        self.nasa = bool(thermo_kind)
        om2, om1 = coll["omega"]
        # Omega_table[0], Omega_table[1], delta_star, T_star, then the 8 bytes after T_star (a
        # pointer member: 0.0 or a subnormal as a double, the same here)
        self.mem = [v for row in om2 for v in row] + [v for row in om1 for v in row] + \
            list(coll["delta_star"]) + list(coll["T_star"]) + [0.0]

    def _tstar(self, i):
        return self.mem[600 + i]

    def _delta(self, j):
        return self.mem[592 + j]

    def _om(self, index, i, j):
        return self.mem[296 * index + 8 * i + j]

    def omega(self, Tstar, deltastar, index):
        """Setup::Omega_interpolated (viscfit.cpp:367-434)."""
        T = self._tstar
        if Tstar > T(0) and Tstar < T(36):
            ii = 1
            while Tstar > T(ii):
                ii += 1
            # ii = 36: the reference reads past T_star (see the module doc); otherwise the last
            # three nodes
            ti = (ii - 1, ii, ii + 1) if (ii < 36 or self.reference_layout) else (34, 35, 36)
        elif Tstar <= T(0):
            ti = (0, 1, 2)
        else:
            ti = (34, 35, 36)
        dl = self._delta
        if deltastar > dl(0) and deltastar < dl(7):
            jj = 1
            while deltastar > dl(jj):
                jj += 1
            tj = (jj - 1, jj, jj + 1) if (jj < 7 or self.reference_layout) else (5, 6, 7)
        elif deltastar <= dl(0):
            tj = (0, 1, 2)
        else:
            tj = (5, 6, 7)
        x1, x2, x3 = T(ti[0]), T(ti[1]), T(ti[2])
        tmp = []
        for j in tj:
            a0, a1, a2 = _quad(x1, x2, x3, self._om(index, ti[0], j), self._om(index, ti[1], j), self._om(index, ti[2], j))
            tmp.append(a0 + a1 * Tstar + a2 * Tstar * Tstar)
        a0, a1, a2 = _quad(dl(tj[0]), dl(tj[1]), dl(tj[2]), tmp[0], tmp[1], tmp[2])
        return a0 + a1 * deltastar + a2 * deltastar * deltastar

    def heat_capacity(self, n, T0):
        """HeatCapacity_NASA / HeatCapacity_JANAF (src/solver_Ini/Thermo_device.h:10-40)."""
        T = max(T0, 200.0)
        Ri, a = self.Ri[n], self.Hia
        _T = 1.0 / T
        if self.nasa:
            rg = 1 if (T >= 1000.0 and T < 6000.0) else (0 if T < 1000.0 else 2)
            c = [a[n * 21 + q * 3 + rg] for q in range(7)]
            return Ri * ((c[0] * _T + c[1]) * _T + c[2] + (c[3] + (c[4] + (c[5] + c[6] * T) * T) * T) * T)
        rg = 0 if T > 1000.0 else 1
        c = [a[n * 21 + q * 3 + rg] for q in range(5)]
        return Ri * (c[0] + (c[1] + (c[2] + (c[3] + c[4] * T) * T) * T) * T)

    def viscosity(self, sp, T):
        """Setup::viscosity (viscfit.cpp:442-449), Pa s."""
        Tstar = T / sp[EPS]
        deltastar = 0.5 * sp[MUE] * sp[MUE] / sp[EPS] / KB / (math.pow(sp[DIAM], 3)) * 1.0e-12
        Omega2 = self.omega(Tstar, deltastar, 0)
        visc = 5 * 1.0e16 * math.sqrt(PI * (sp[WI] * 1e3) / NA * KB * T) / (16 * PI * sp[DIAM] * sp[DIAM] * Omega2)
        return 0.1 * visc

    def conductivity(self, sp, T, PP):
        """Setup::thermal_conductivities (viscfit.cpp:458-498), W/(m K)."""
        Cv_trans = 1.5 * UNIVERSAL_GAS_CONST
        Cpi = self.heat_capacity(int(sp[SID]), T)
        Cv = Cpi * sp[WI] * 1.0e3 - UNIVERSAL_GAS_CONST
        geo = int(sp[GEO])
        if geo == 0:
            Cv_rot, Cv_vib = 0.0, 0.0
        elif geo == 1:
            Cv_rot, Cv_vib = 1.0 * UNIVERSAL_GAS_CONST, Cv - 2.5 * UNIVERSAL_GAS_CONST
        else:
            Cv_rot, Cv_vib = 1.5 * UNIVERSAL_GAS_CONST, Cv - 3.0 * UNIVERSAL_GAS_CONST
        rho = PP * sp[WI] / T / UNIVERSAL_GAS_CONST
        Dkk = self.dkj(sp, sp, T, PP)
        visc = self.viscosity(sp, T)
        f_vib = rho * Dkk / (visc * 10.0)
        Zrot = sp[ZROT] * _zrot(sp[EPS] / 298.0) / _zrot(sp[EPS] / T)
        Aa = 2.5 - f_vib
        Bb = Zrot + 2.0 * (5.0 * Cv_rot / 3.0 / (UNIVERSAL_GAS_CONST) + f_vib) / PI
        f_trans = 2.5 * (1.0 - 2.0 * Cv_rot * Aa / PI / Cv_trans / Bb)
        f_rot = f_vib * (1.0 + 2.0 * Aa / PI / Bb)
        return visc * (f_trans * Cv_trans + f_rot * Cv_rot + f_vib * Cv_vib) / sp[WI] * 1.0e-3

    def dkj(self, sk, sj, T, PP):
        """Setup::Dkj (viscfit.cpp:507-555), cm^2/s."""
        if (sj[MUE] > 0 and sk[MUE] > 0) or (sj[MUE] == 0 and sk[MUE] == 0):
            eps_jk = math.sqrt(sj[EPS] * sk[EPS])
            d_jk = (sj[DIAM] + sk[DIAM]) / 2.0
            mue_sqr = sj[MUE] * sk[MUE]
        else:
            n_, p_ = (sj, sk) if (sk[MUE] > 0 and sj[MUE] == 0) else (sk, sj)
            alpha_n_star = n_[ALPHA] / math.pow(n_[DIAM], 3.0)
            mue_p_star = p_[MUE] / math.pow(p_[EPS] * KB, 0.5) / math.pow(p_[DIAM], 1.5) * 1.0e-6
            ksi = 1.0 + 0.25 * alpha_n_star * mue_p_star * math.sqrt(p_[EPS] / n_[EPS])
            eps_jk = ksi * ksi * math.sqrt(n_[EPS] * p_[EPS])
            d_jk = math.pow(ksi, -1.0 / 6.0) * (sj[DIAM] + sk[DIAM]) / 2.0
            mue_sqr = 0.0
        T_jk_star = T / eps_jk
        delta_jk_star = 0.5 * mue_sqr / d_jk / d_jk / d_jk / eps_jk / KB * 1.0e-12
        W_jk = sk[WI] * sj[WI] / (sk[WI] + sj[WI]) / NA * 1.0e3
        Omega1 = self.omega(T_jk_star, delta_jk_star, 1)
        PPP = PP * 10.0
        return 3.0 * math.sqrt(2.0 * PI * math.pow(T * KB, 3.0) / W_jk) / (16.0 * PPP * PI * d_jk * d_jk * Omega1) * 1.0e16

    def fit(self, sk, sj, indicator, tnode):
        """Setup::Fitting (viscfit.cpp:318-341): least squares of ln(value) over powers of ln(T)."""
        b, AA = [], []
        for T in tnode:
            if indicator == 0:
                b.append(math.log(self.viscosity(sk, T)))
            elif indicator == 1:
                b.append(math.log(self.conductivity(sk, T, 1.0)))
            else:
                b.append(math.log(self.dkj(sk, sj, T, 1.0)))
            AA.append([math.pow(math.log(T), float(jj)) for jj in range(ORDER)])
        return _solve_overdetermined(AA, b)


def _solve_overdetermined(AA, b):
    """Solve_Overdeter_equations (mixture.hpp:89-142): normal equations, Cholesky, two triangular
    solves, in the reference's loop order."""
    nn, mm = ORDER, len(b)
    CC = [[0.0] * nn for _ in range(nn)]
    dd = [0.0] * nn
    for i in range(nn):
        for q in range(mm):
            dd[i] = dd[i] + AA[q][i] * b[q]
        for j in range(nn):
            for k in range(mm):
                CC[i][j] = CC[i][j] + AA[k][i] * AA[k][j]
    CC[0][0] = math.sqrt(CC[0][0])
    for p in range(1, nn):
        CC[p][0] = CC[p][0] / CC[0][0]
    for k in range(1, nn):
        for m in range(k):
            CC[k][k] = CC[k][k] - CC[k][m] * CC[k][m]
        CC[k][k] = math.sqrt(CC[k][k])
        for i in range(k + 1, nn):
            for m in range(k):
                CC[i][k] = CC[i][k] - CC[i][m] * CC[k][m]
            CC[i][k] = CC[i][k] / CC[k][k]
    xx = [0.0] * nn
    xx[0] = dd[0] / CC[0][0]
    for j in range(1, nn):
        for q in range(j):
            dd[j] = dd[j] - CC[j][q] * xx[q]
        xx[j] = dd[j] / CC[j][j]
    dd[nn - 1] = xx[nn - 1] / CC[nn - 1][nn - 1]
    for i in range(nn - 2, -1, -1):
        for p in range(nn - 1, i, -1):
            xx[i] = xx[i] - CC[p][i] * dd[p]
        dd[i] = xx[i] / CC[i][i]
    return list(dd)


def fit_transport(species, thermal, thermo_kind, runtime_dir=None, tables_json=None, inv_spacing=None,
                  yil_limiter=1.0e10, dim_limiter=2.0e-3, tnode=None, reference_layout=False):
    """xfg_transport of a mixture (Setup::GetFitCoefficient, viscfit.cpp:148-196) from the
    Lennard-Jones data and collision tables of runtime.dat (runtime_dir) or of a JSON written by
    dump_transport_tables (tables_json). thermal: the scheme's xfg_thermal (molar masses and the
    heat-capacity tables of thermo_kind, 0 JANAF / 1 NASA-9). inv_spacing: (1/dx, 1/dy, 1/dz) of the
    block for Block::Yil_limiter = max(1/d) * clamp(yil_limiter, 0, 1); dim_limiter: the JSON
    "Dim_limiter" (iniset.cpp:358-359). reference_layout: reproduce the reference's reads past the
    collision tables (module doc); off, the last interval interpolates within the tables."""
    from .thermo import transport_from_arrays
    if tables_json is not None:
        with open(tables_json) as f:
            tab = json.load(f)
        idx = [tab["species"].index(s) for s in species]
        lj = [tab["lj"][i] for i in idx]
        coll = tab["collision"]
    else:
        lj = read_transport_data(runtime_dir, species)
        coll = read_collision_integrals(runtime_dir)
    ns = len(species)
    chara = [list(lj[i]) + [thermal.Wi[i], 0.0, float(i)] for i in range(ns)]
    fz = _Fitter(chara, thermal, thermo_kind, coll, reference_layout=reference_layout)
    tn = TNODE if tnode is None else list(tnode)
    visc, therm = [], []
    dkj = [[None] * ns for _ in range(ns)]
    for k in range(ns):
        visc.append(fz.fit(chara[k], chara[k], 0, tn))
        therm.append(fz.fit(chara[k], chara[k], 1, tn))
        for j in range(ns):
            dkj[k][j] = fz.fit(chara[k], chara[j], 2, tn) if k <= j else dkj[j][k]
    yil = (max(inv_spacing) if inv_spacing else 1.0) * min(max(yil_limiter, 0.0), 1.0)
    dim = min(max(dim_limiter, 0.0), 1.0)
    return transport_from_arrays(ns, visc, therm, [c for row in dkj for c in row], chara, yil, dim)
