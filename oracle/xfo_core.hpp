// xfo_core.hpp - CPU restatement of the XFluids convective right-hand side (test infrastructure).
//
// This is the ORACLE: a plain, serial/OpenMP restatement of the reference algorithm that the CUDA
// path is checked against. It is only used by tests/, __graft_entry__.smoke() and the CPU arms of
// bench.py. The product library never links or calls it.
//
// Every function restates one reference function with the same operation order (parenthesised
// exactly as C++ parses the reference expressions), so that built with -ffp-contract=off it
// reproduces the reference CPU build bit for bit. The reference's compile-time switches become
// fields of Scheme. Two deliberate differences, both bit-neutral for finite values:
//   * eigenvector entries that are structural zeros are skipped in the projections
//     (x + U*0.0 == x) and structural +-1 entries become additions/subtractions (x + U*1.0 == x+U);
//   * per-call invariants the reference recomputes in each helper (MARCO_PREEIGEN) are computed once.
// The scalar type R is a template parameter so that the same code runs on double (oracle) and on
// a counting scalar (algorithmic flop count, xfo_count.hpp).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/xfluids_gb300.h"

namespace xfo {

constexpr int kMaxS = XFG_MAX_SPECIES;
constexpr int kMaxE = XFG_MAX_EQ;

// Physical constants, src/include/global_setup.h:48-54 (Ru in J/mol/K).
constexpr double kAvogadro = 6.02214076e26;
constexpr double kBoltzmann = 1.380649e-23;
constexpr double kUniversalGas = kAvogadro * kBoltzmann;
constexpr double kRu = kUniversalGas * 1.0E-3;
constexpr double kOT = 1.0 / 3.0;    // _OT, global_setup.h:35
constexpr double kSix = 1.0 / 6.0;   // _six, schemes/Utils_schemes.hpp:5

inline double dval(double x) { return x; }

// ---------------------------------------------------------------------------------------------
// Thermodynamics of species n (src/solver_Ini/Thermo_device.h)
// ---------------------------------------------------------------------------------------------
struct ThermoTable {
    int ns;
    int nasa;  // Thermo: 1 NASA-9, 0 JANAF
    const double *Hia, *Hib, *Ri, *Wi, *_Wi;
};

// HeatCapacity_NASA, Thermo_device.h:10-23
template <class R>
R cp_nasa(const ThermoTable &t, R T0, double Ri, int n) {
    using std::fmax;
    R T = fmax(T0, R(200.0));
    R _T = R(1.0) / T;
    // range 1 for [1000, 6000), 0 below, 2 from 6000 K; none (Cp = 0) when T is NaN
    int rg = (T >= R(1000.0) && T < R(6000.0)) ? 1 : (T < R(1000.0) ? 0 : (T >= R(6000.0) ? 2 : -1));
    if (rg < 0) return R(0.0);
    const double *a = t.Hia + n * 21 + rg;
    return Ri * ((a[0] * _T + a[3]) * _T + a[6] + (a[9] + (a[12] + (a[15] + a[18] * T) * T) * T) * T);
}
// HeatCapacity_JANAF, Thermo_device.h:29-40
template <class R>
R cp_janaf(const ThermoTable &t, R T0, double Ri, int n) {
    using std::fmax;
    R T = fmax(T0, R(200.0));
    int rg = (T > R(1000.0)) ? 0 : 1;
    const double *a = t.Hia + n * 21 + rg;
    return Ri * (a[0] + (a[3] + (a[6] + (a[9] + a[12] * T) * T) * T) * T);
}
template <class R>
R heat_capacity(const ThermoTable &t, R T0, double Ri, int n) {
    return t.nasa ? cp_nasa(t, T0, Ri, n) : cp_janaf(t, T0, Ri, n);
}
// get_Enthalpy_NASA, Thermo_device.h:62-80
template <class R>
R h_nasa(const ThermoTable &t, R T0, double Ri, int n) {
    using std::fmax;
    using std::log;
    R TT = T0, T = fmax(T0, R(200.0));
    int rg = (T >= R(1000.0) && T < R(6000.0)) ? 1 : (T < R(1000.0) ? 0 : (T >= R(6000.0) ? 2 : -1));
    R hi = R(0.0);
    if (rg >= 0) {
        const double *a = t.Hia + n * 21 + rg;
        const double b0 = t.Hib[n * 6 + rg];
        hi = Ri * (-a[0] / T + a[3] * log(T) +
                   (a[6] + (0.5 * a[9] + (a[12] * kOT + (0.25 * a[15] + 0.2 * a[18] * T) * T) * T) * T) * T + b0);
    }
    if (TT < R(200.0)) {
        R Cpi = cp_nasa(t, R(200.0), Ri, n);
        hi += Cpi * (TT - R(200.0));
    }
    return hi;
}
// get_Enthalpy_JANAF, Thermo_device.h:86-102
template <class R>
R h_janaf(const ThermoTable &t, R T0, double Ri, int n) {
    using std::fmax;
    R TT = T0, T = fmax(T0, R(200.0));
    int rg = (T > R(1000.0)) ? 0 : 1;
    const double *a = t.Hia + n * 21 + rg;
    R hi = Ri * (T * (a[0] + T * (a[3] * 0.5 + T * (a[6] * kOT + T * (a[9] * 0.25 + a[12] * T * 0.2)))) + a[15]);
    if (TT < R(200.0)) {
        R Cpi = cp_janaf(t, R(200.0), Ri, n);
        hi += Cpi * (TT - R(200.0));
    }
    return hi;
}
template <class R>
R enthalpy(const ThermoTable &t, R T0, double Ri, int n) {
    return t.nasa ? h_nasa(t, T0, Ri, n) : h_janaf(t, T0, Ri, n);
}

// ---------------------------------------------------------------------------------------------
// Mixture functions (src/solver_Ini/Mixing_device.h)
// ---------------------------------------------------------------------------------------------
template <class R>  // get_CopR :49-56
R mix_R(const ThermoTable &t, const R *yi) {
    R s = R(0.0);
    for (int n = 0; n < t.ns; n++) s += yi[n] * t._Wi[n];
    return s * kRu;
}
template <class R>  // get_CopCp :61-68
R mix_Cp(const ThermoTable &t, const R *yi, R T) {
    R s = R(0.0);
    for (int n = 0; n < t.ns; n++) s += yi[n] * heat_capacity(t, T, t.Ri[n], n);
    return s;
}
template <class R>  // get_CopGamma(thermal, yi, Cp, T) :114-126 (guarded form used by GetStates)
R mix_gamma_guarded(const ThermoTable &t, const R *yi, R Cp) {
    R w = R(0.0);
    for (int n = 0; n < t.ns; n++) w += yi[n] * t._Wi[n];
    R CopW = R(1.0) / w;  // get_CopW :91-97
    R g = Cp / (Cp - kRu / CopW);
    if (g > R(1.0)) return g;
    return R(-1.0);
}
template <class R>  // get_CopGamma(thermal, yi, T) :102-109 = Cp / get_CopCv (:73-86)
R mix_gamma_cpcv(const ThermoTable &t, const R *yi, R T, R Cp) {
    // Cp = get_CopCp(yi, T); get_CopCv recomputes the same sum and subtracts Ru * sum(yi/Wi).
    R w = R(0.0);
    for (int n = 0; n < t.ns; n++) w += yi[n] * t._Wi[n];
    R Cv = Cp - kRu * w;
    return Cp / Cv;
}
template <class R>  // get_Coph :131-140
R mix_h(const ThermoTable &t, const R *yi, R T) {
    R h = R(0.0);
    for (int n = 0; n < t.ns; n++) h += enthalpy(t, T, t.Ri[n], n) * yi[n];
    return h;
}
// get_T :171-193 with sub_FuncT :159-166. Newton on h(T) - R T - e = 0, warm-started from T0.
template <class R>
R newton_T(const ThermoTable &t, const R *yi, R e, R T0) {
    using std::fabs;
    using std::fmax;
    using std::fmin;
    R T = T0;
    for (int it = 1; it < 101; it++) {
        R h = mix_h(t, yi, T);
        R Rm = mix_R(t, yi);
        R Cp = mix_Cp(t, yi, T);
        R f = h - Rm * T - e;
        R df_ = Cp - Rm;
        R df = fmin(f / (df_ + R(1.0e-30)), R(1e-3) * T);
        df = fmax(df, -R(1e-2) * T);
        T = T - df;
        if (fabs(df) <= R(1.0e-6)) break;
    }
    return T;
}

// ---------------------------------------------------------------------------------------------
// Configuration
// ---------------------------------------------------------------------------------------------
struct Config {
    xfg_block bl;
    xfg_scheme sc;
    xfg_thermal th;
    xfg_transport tr;  // viscous schemes
    int E() const { return sc.cop ? sc.num_species + 4 : 5; }
    int NS() const { return sc.num_species; }
    int NCOP() const { return sc.cop ? sc.num_species - 1 : 0; }
    size_t ncell() const { return (size_t)bl.Xmax * bl.Ymax * bl.Zmax; }
    ThermoTable table() const { return ThermoTable{th.num_species, sc.thermo, th.Hia, th.Hib, th.Ri, th.Wi, th._Wi}; }
};

// Arrays of one fluid, in the reference's layouts (AoS U, SoA primitives, AoS y).
template <class R>
struct Fields {
    std::vector<R> U, U1, LU;
    std::vector<R> rho, p, u, v, w, c, gamma, e, H, T, Cp, Rm, y;
    std::vector<R> FluxF, FluxG, FluxH, Fw[3];
    std::vector<R> eig[3];        // eigen_local_{x,y,z}, AoS Emax
    R eigen_block[3][kMaxE];      // GLF maxima
    R uvw_c_max[3];
    std::vector<R> Vde, mu, kappa, Dkm, hi;  // viscous: 9 velocity derivatives, transport, enthalpies
    void alloc(const Config &cf) {
        size_t n = cf.ncell(), E = cf.E();
        for (std::vector<R> *a : {&U, &U1, &LU, &FluxF, &FluxG, &FluxH, &Fw[0], &Fw[1], &Fw[2], &eig[0], &eig[1], &eig[2]})
            a->assign(n * E, R(0.0));
        for (std::vector<R> *a : {&rho, &p, &u, &v, &w, &this->c, &gamma, &e, &H, &T, &Cp, &Rm}) a->assign(n, R(0.0));
        y.assign(n * cf.NS(), R(0.0));
        if (cf.sc.viscous) {
            Vde.assign(9 * n, R(0.0)), mu.assign(n, R(0.0)), kappa.assign(n, R(0.0));
            Dkm.assign(n * cf.NS(), R(0.0)), hi.assign(n * cf.NS(), R(0.0));
        }
        for (int d = 0; d < 3; d++)
            for (int k = 0; k < kMaxE; k++) eigen_block[d][k] = R(0.0);
        for (int d = 0; d < 3; d++) uvw_c_max[d] = R(0.0);
    }
};

// ---------------------------------------------------------------------------------------------
// Boundary conditions, src/solver_BCs/BCs_kernels.hpp:9-258 driven as BCs_block.cpp:4-218:
// X faces over all (j,k), then Y faces over all (i,k), then Z faces over all (i,j).
// ---------------------------------------------------------------------------------------------
template <class R>
void bc_cell(const Config &cf, R *U, int d, int BC, int i, int j, int k, int mirror_offset, int index_inner, int sign) {
    const xfg_block &b = cf.bl;
    const int E = cf.E(), NCOP = cf.NCOP();
    const int Xmax = b.Xmax, Ymax = b.Ymax;
    const int inner = d == 0 ? b.X_inner : (d == 1 ? b.Y_inner : b.Z_inner);
    const int bw = d == 0 ? b.Bwidth_X : (d == 1 ? b.Bwidth_Y : b.Bwidth_Z);
    int c = d == 0 ? i : (d == 1 ? j : k);  // coordinate along the face normal
    auto at = [&](int cc) -> size_t {
        int ii = d == 0 ? cc : i, jj = d == 1 ? cc : j, kk = d == 2 ? cc : k;
        return (size_t)Xmax * Ymax * kk + (size_t)Xmax * jj + ii;
    };
    size_t id = at(c);
    int src;
    int vel = 1 + d;
    switch (BC) {
    case XFG_SYMMETRY: {
        src = 2 * (bw + mirror_offset) - 1 - c;
        size_t t = at(src);
        for (int n = 0; n < E; n++) U[E * id + n] = U[E * t + n];
        U[E * id + vel] = -U[E * t + vel];
    } break;
    case XFG_PERIODIC: {
        size_t t = at(c + sign * inner);
        for (int n = 0; n < E; n++) U[E * id + n] = U[E * t + n];
    } break;
    case XFG_OUTFLOW: {
        size_t t = at(index_inner);
        for (int n = 0; n < E; n++) U[E * id + n] = U[E * t + n];
    } break;
    case XFG_NSLIPWALL:
    case XFG_VISCWALL:
    case XFG_SLIPWALL: {
        // the Y and Z kernels mirror only nslipWall; viscWall and slipWall are no-ops there
        // (BCs_kernels.hpp FluidBCKernelY/Z), the X kernel mirrors all three walls
        if (d != 0 && BC != XFG_NSLIPWALL) break;
        src = 2 * (bw + mirror_offset) - 1 - c;
        size_t t = at(src);
        U[E * id + 0] = U[E * t + 0];
        U[E * id + 1] = -U[E * t + 1];
        U[E * id + 2] = -U[E * t + 2];
        U[E * id + 3] = -U[E * t + 3];
        U[E * id + 4] = U[E * t + 4];
        for (int n = E - NCOP; n < E; n++) U[E * id + n] = U[E * t + n];
    } break;
    default:  // Inflow, innerBlock: untouched
        break;
    }
}

template <class R>
void boundary(const Config &cf, R *U) {
    const xfg_block &b = cf.bl;
    if (b.DimX)
        for (int k = 0; k < b.Zmax; k++)
            for (int j = 0; j < b.Ymax; j++)
                for (int g = 0; g < b.Bwidth_X; g++) {
                    bc_cell(cf, U, 0, b.Boundarys[0], g, j, k, 0, b.Bwidth_X, 1);
                    bc_cell(cf, U, 0, b.Boundarys[1], g + b.Xmax - b.Bwidth_X, j, k, b.X_inner, b.Xmax - b.Bwidth_X - 1, -1);
                }
    if (b.DimY)
        for (int k = 0; k < b.Zmax; k++)
            for (int g = 0; g < b.Bwidth_Y; g++)
                for (int i = 0; i < b.Xmax; i++) {
                    bc_cell(cf, U, 1, b.Boundarys[2], i, g, k, 0, b.Bwidth_Y, 1);
                    bc_cell(cf, U, 1, b.Boundarys[3], i, g + b.Ymax - b.Bwidth_Y, k, b.Y_inner, b.Ymax - b.Bwidth_Y - 1, -1);
                }
    if (b.DimZ)
        for (int g = 0; g < b.Bwidth_Z; g++)
            for (int j = 0; j < b.Ymax; j++)
                for (int i = 0; i < b.Xmax; i++) {
                    bc_cell(cf, U, 2, b.Boundarys[4], i, j, g, 0, b.Bwidth_Z, 1);
                    bc_cell(cf, U, 2, b.Boundarys[5], i, j, g + b.Zmax - b.Bwidth_Z, b.Z_inner, b.Zmax - b.Bwidth_Z - 1, -1);
                }
}

// ---------------------------------------------------------------------------------------------
// Primitive recovery (src/solver_UpdateStates/Update_device.hpp)
// ---------------------------------------------------------------------------------------------
// Getrhoyi :7-29
template <class R>
void get_rho_yi(const Config &cf, R *U, R &rho, R *yi) {
    rho = U[0];
    R rho1 = R(1.0) / rho;
    if (!cf.sc.cop) return;
    const int NCOP = cf.NCOP(), E = cf.E();
    if (cf.sc.ghost_species) {
        yi[NCOP] = R(0.0);
        R sum = R(0.0);
        for (int s = 0; s < NCOP; s++) yi[s] = U[s + 5] * rho1, sum += yi[s];
        sum = R(1.0) / sum;
        for (int s = 0; s < NCOP; s++) yi[s] *= sum, U[s + 5] = rho * yi[s];
    } else {
        yi[NCOP] = R(1.0);
        for (int s = 5; s < E; s++) yi[s - 5] = U[s] * rho1, yi[NCOP] += -yi[s - 5];
    }
}

// GetStates :33-54 and GetPhysFlux :81-110
template <class R>
void get_states(const Config &cf, const ThermoTable &tt, const R *U, R rho, R &u, R &v, R &w, R &p, R &H, R &c,
                R &gamma, R &T, R &e, R &Cp, R &Rm, const R *yi) {
    using std::sqrt;
    R rho1 = R(1.0) / rho;
    u = U[1] * rho1, v = U[2] * rho1, w = U[3] * rho1;
    R tme = U[4] * rho1 - R(0.5) * (u * u + v * v + w * w);
    if (cf.sc.cop) {
        R R_ = mix_R(tt, yi);
        T = newton_T(tt, yi, tme, T);
        p = rho * R_ * T, Rm = R_;
        Cp = mix_Cp(tt, yi, T);
        gamma = mix_gamma_guarded(tt, yi, Cp);
    } else {
        gamma = R(cf.sc.ncop_gamma);
        p = (cf.sc.ncop_gamma - 1.0) * rho * tme;
    }
    H = (U[4] + p) * rho1;
    c = sqrt(gamma * p * rho1);
    e = tme;
}

template <class R>
void phys_flux(const Config &cf, const R *U, const R *yi, R *F, R *G, R *Hf, R u, R v, R w, R p) {
    F[0] = U[1]; F[1] = U[1] * u + p; F[2] = U[1] * v; F[3] = U[1] * w; F[4] = (U[4] + p) * u;
    G[0] = U[2]; G[1] = U[2] * u; G[2] = U[2] * v + p; G[3] = U[2] * w; G[4] = (U[4] + p) * v;
    Hf[0] = U[3]; Hf[1] = U[3] * u; Hf[2] = U[3] * v; Hf[3] = U[3] * w + p; Hf[4] = (U[4] + p) * w;
    if (cf.sc.cop)
        for (int n = 5; n < cf.E(); n++) F[n] = U[1] * yi[n - 5], G[n] = U[2] * yi[n - 5], Hf[n] = U[3] * yi[n - 5];
}

// UpdateFluidStateFlux (UpdateStates_block.cpp:7-191): Updaterhoyi on all cells, then
// UpdateFuidStatesKernel on all cells. Returns 0.
template <class R>
void update_states(const Config &cf, Fields<R> &f, std::vector<R> &UI) {
    const ThermoTable tt = cf.table();
    const long n = (long)cf.ncell();
    const int E = cf.E(), NS = cf.NS();
#pragma omp parallel for schedule(static)
    for (long id = 0; id < n; id++) get_rho_yi(cf, &UI[E * id], f.rho[id], &f.y[NS * id]);
#pragma omp parallel for schedule(static)
    for (long id = 0; id < n; id++) {
        const R *U = &UI[E * id];
        get_states(cf, tt, U, f.rho[id], f.u[id], f.v[id], f.w[id], f.p[id], f.H[id], f.c[id], f.gamma[id], f.T[id],
                   f.e[id], f.Cp[id], f.Rm[id], &f.y[NS * id]);
        phys_flux(cf, U, &f.y[NS * id], &f.FluxF[E * id], &f.FluxG[E * id], &f.FluxH[E * id], f.u[id], f.v[id], f.w[id],
                  f.p[id]);
    }
}

// ---------------------------------------------------------------------------------------------
// Eigensystem (src/solver_Reconstruction/FDM_Method/positive-definite_eigen)
// ---------------------------------------------------------------------------------------------
// An eigenvector row/column entry: structural zero, +1, -1 or a general value.
enum Kind : uint8_t { KZ = 0, KP1 = 1, KM1 = 2, KG = 3 };
template <class R>
struct Vec {
    R v[kMaxE];
    uint8_t k[kMaxE];
    void zero(int E) { for (int n = 0; n < E; n++) v[n] = R(0.0), k[n] = KZ; }
    void set(int n, R x) { v[n] = x, k[n] = KG; }
    void one(int n) { v[n] = R(1.0), k[n] = KP1; }
    void mone(int n) { v[n] = R(-1.0), k[n] = KM1; }
};
// sum_n a[n] * vec[n], accumulated in ascending n from 0.0 as the reference loops do.
template <class R>
R dot(const Vec<R> &l, const R *a, int E) {
    R acc = R(0.0);
    bool first = true;
    for (int n = 0; n < E; n++) {
        switch (l.k[n]) {
        case KZ: break;
        case KP1: acc = first ? a[n] : acc + a[n]; first = false; break;
        case KM1: acc = first ? -a[n] : acc - a[n]; first = false; break;
        default: acc = first ? a[n] * l.v[n] : acc + a[n] * l.v[n]; first = false; break;
        }
    }
    return acc;
}

// Roe-averaged face state and the quantities MARCO_PREEIGEN derives from it.
template <class R>
struct Face {
    R D, D1, _u, _v, _w, _H, _P, _rho;
    R c2, b1, b3, Gamma0;
    R z[kMaxS], _yi[kMaxS];
    R q2, _c, b2, _c1;
};

// ReconstructSoundSpeed + SoundSpeedMultiSpecies, Utils_device.hpp:42-79, :102-140.
template <class R>
R cop_sound_speed(const Config &cf, const ThermoTable &tt, const Fields<R> &f, size_t id_l, size_t id_r, Face<R> &F) {
    const int NS = cf.NS(), NCOP = cf.NCOP();
    const R *yl = &f.y[NS * id_l], *yr = &f.y[NS * id_r];
    const R D = F.D, D1 = F.D1;
    auto roe = [&](R a, R b) { return (a + D * b) * D1; };  // get_RoeAverage, Recon_device.hpp:14-17
    R hl[kMaxS], hr[kMaxS], dpdrhoi[kMaxS], drhoi[kMaxS];
    const R Tl = f.T[id_l], Tr = f.T[id_r];
    for (int n = 0; n < NS; n++) {
        hl[n] = enthalpy(tt, Tl, tt.Ri[n], n);
        hr[n] = enthalpy(tt, Tr, tt.Ri[n], n);
        F._yi[n] = (yl[n] + D * yr[n]) * D1;
    }
    R Cpl = mix_Cp(tt, yl, Tl), Cpr = mix_Cp(tt, yr, Tr);
    R gl = mix_gamma_cpcv(tt, yl, Tl, Cpl), gr = mix_gamma_cpcv(tt, yr, Tr, Cpr);
    F.Gamma0 = roe(gl, gr);
    const R ul = f.u[id_l], vl = f.v[id_l], wl = f.w[id_l], ur = f.u[id_r], vr = f.v[id_r], wr = f.w[id_r];
    R q2l = ul * ul + vl * vl + wl * wl, q2r = ur * ur + vr * vr + wr * wr;
    R Rl = mix_R(tt, yl), Rr = mix_R(tt, yr);
    const R rl = f.rho[id_l], rr = f.rho[id_r], pl = f.p[id_l], pr = f.p[id_r];
    R el = f.H[id_l] - R(0.5) * q2l - pl / rl, er = f.H[id_r] - R(0.5) * q2r - pr / rr;
    const double RN = tt.Ri[NCOP];
    auto dpdrho = [&](R hN, R q2, R Cp, R Rm, R T, R g) {  // get_DpDrho :14-19
        R RNT = RN * T;
        return (g - R(1.0)) * (R(0.5) * q2 - hN + Cp * RNT / Rm);
    };
    auto dpdrhoi_of = [&](R hin, double Rin, R hiN, R T, R Cp, R Rm, R g) {  // get_DpDrhoi :29-35
        R hN_minus_hi = -hin + hiN;
        R Ri_minus_RN = R(Rin - RN);
        return (g - R(1.0)) * (hN_minus_hi + Cp * Ri_minus_RN * T / Rm);
    };
    R _dpdrho = roe(dpdrho(hl[NCOP], q2l, Cpl, Rl, Tl, gl), dpdrho(hr[NCOP], q2r, Cpr, Rr, Tr, gr));
    for (int n = 0; n < NCOP; n++) {
        dpdrhoi[n] = roe(dpdrhoi_of(hl[n], tt.Ri[n], hl[NCOP], Tl, Cpl, Rl, gl), dpdrhoi_of(hr[n], tt.Ri[n], hr[NCOP], Tr, Cpr, Rr, gr));
        drhoi[n] = rr * yr[n] - rl * yl[n];
    }
    R _prho = roe(pl / rl, pr / rr) +
              R(0.5) * D * D1 * D1 * ((ur - ul) * (ur - ul) + (vr - vl) * (vr - vl) + (wr - wl) * (wr - wl));
    R _dpdE = roe(gl - R(1.0), gr - R(1.0));
    R _dpde = roe((gl - R(1.0)) * rl, (gr - R(1.0)) * rr);
    // SoundSpeedMultiSpecies
    R dp = pr - pl, drho = rr - rl, de = er - el;
    R Sum_dpdrhoi = R(0.0), Sum_dpdrhoi2 = R(0.0), Sum_Yidpdrhoi = R(0.0);
    for (int n = 0; n < NCOP; n++) {
        Sum_dpdrhoi += dpdrhoi[n] * drhoi[n];
        Sum_dpdrhoi2 += dpdrhoi[n] * drhoi[n] * dpdrhoi[n] * drhoi[n];
    }
    R temp1 = dp - (_dpdrho * drho + _dpde * de + Sum_dpdrhoi);
    R temp = temp1 / (_dpdrho * _dpdrho * drho * drho + _dpde * de * _dpde * de + Sum_dpdrhoi2 + R(1e-19));
    for (int n = 0; n < NCOP; n++) Sum_Yidpdrhoi += F._yi[n] * dpdrhoi[n];
    R _dpdE_new = _dpdE + _dpdE * _dpdE * de * F._rho * temp;
    R _dpdrho_new = _dpdrho + _dpdrho * _dpdrho * drho * temp;
    R dpdrhoi_new[kMaxS];
    for (int n = 0; n < NCOP; n++) dpdrhoi_new[n] = dpdrhoi[n] + dpdrhoi[n] * dpdrhoi[n] * drhoi[n] * temp;
    R csqr = _dpdrho_new + _dpdE_new * _prho + Sum_Yidpdrhoi;
    F.b1 = _dpdE_new / csqr;
    F.b3 = R(0.0);
    for (int n = 0; n < NCOP; n++) {
        F.z[n] = -dpdrhoi_new[n] / _dpdE_new;
        F.b3 += F._yi[n] * F.z[n];
    }
    F.b3 *= F.b1;
    // c2 <= 0 fallback (sycl::step(c2, 0) is 1 when c2 <= 0)
    R c2w = (R(0.0) < csqr) ? R(0.0) : R(1.0);
    R c2 = F.Gamma0 * F._P * F._rho * c2w + (R(1.0) - c2w) * csqr;
    return c2;
}

// MARCO_ROE (global_marco.h:26-37) + MARCO_NOCOPC2 / MARCO_COPC2 + MARCO_PREEIGEN.
template <class R>
void face_state(const Config &cf, const ThermoTable &tt, const Fields<R> &f, size_t id_l, size_t id_r, Face<R> &F) {
    using std::sqrt;
    F.D = sqrt(f.rho[id_r] / f.rho[id_l]);
    F.D1 = R(1.0) / (F.D + R(1.0));
    F._u = (f.u[id_l] + F.D * f.u[id_r]) * F.D1;
    F._v = (f.v[id_l] + F.D * f.v[id_r]) * F.D1;
    F._w = (f.w[id_l] + F.D * f.w[id_r]) * F.D1;
    F._H = (f.H[id_l] + F.D * f.H[id_r]) * F.D1;
    F._P = (f.p[id_l] + F.D * f.p[id_r]) * F.D1;
    F._rho = sqrt(f.rho[id_r] * f.rho[id_l]);
    if (cf.sc.cop) {
        F.c2 = cop_sound_speed(cf, tt, f, id_l, id_r, F);
    } else {
        F.Gamma0 = R(cf.sc.ncop_gamma);
        F.c2 = F.Gamma0 * F._P / F._rho;
        F.b1 = (F.Gamma0 - R(1.0)) / F.c2;
        F.b3 = R(0.0);
    }
    F.q2 = F._u * F._u + F._v * F._v + F._w * F._w;
    F._c = sqrt(F.c2);
    F.b2 = R(1.0) + F.b1 * F.q2 - F.b1 * F._H;
    F._c1 = R(1.0) / F._c;
}

// RoeAverageLeft_{x,y,z} (Eigen_matrix.hpp:7-84, :157-234, :307-384): row n of L and |lambda_n|.
// d = 0,1,2 for x,y,z. Velocity components are permuted so that un is normal, ut1/ut2 follow the
// reference's row layout for that direction.
template <class R>
void left_row(const Config &cf, int d, int n, const Face<R> &F, Vec<R> &l, R &ev) {
    using std::fabs;
    const int E = cf.E(), NCOP = cf.NCOP();
    const R b1 = F.b1, b2 = F.b2, b3 = F.b3, _c1 = F._c1, _c = F._c;
    const R vel[3] = {F._u, F._v, F._w};
    const R un = vel[d];
    l.zero(E);
    const R hb1 = R(0.5) * b1;
    if (n == 0 || n == E - 1) {
        const R un_c = un * _c1;
        const R s = (n == 0) ? R(1.0) : R(-1.0);
        // n = 0: 0.5*(b2 + un_c + b3), -0.5*(b1*u_m [+ _c1 if m == d]);
        // n = E-1: 0.5*(b2 - un_c + b3), 0.5*(-b1*u_m [+ _c1 if m == d]).
        if (n == 0) l.set(0, R(0.5) * (b2 + un_c + b3));
        else l.set(0, R(0.5) * (b2 - un_c + b3));
        for (int m = 0; m < 3; m++) {
            if (n == 0) l.set(1 + m, m == d ? -R(0.5) * (b1 * vel[m] + _c1) : -R(0.5) * (b1 * vel[m]));
            else l.set(1 + m, m == d ? R(0.5) * (-b1 * vel[m] + _c1) : R(0.5) * (-b1 * vel[m]));
        }
        l.set(4, hb1);
        for (int m = 0; m < NCOP; m++) l.set(m + E - NCOP, -R(0.5) * b1 * F.z[m]);
        ev = (n == 0) ? fabs(un - _c) : fabs(un + _c);
        (void)s;
        return;
    }
    ev = fabs(un);
    // rows 1..3: one of them is the entropy-like row (the one whose index is d+1), the others the
    // shear rows, in the order the reference lays them out per direction.
    if (n >= 1 && n <= 3) {
        const int dn = d + 1;  // row with (1-b2-b3)/b1, u, v, w, -1
        if (n == dn) {
            l.set(0, (R(1.0) - b2 - b3) / b1);
            l.set(1, F._u); l.set(2, F._v); l.set(3, F._w);
            l.mone(4);
            for (int m = 0; m < NCOP; m++) l.set(m + E - NCOP, F.z[m]);
            return;
        }
        // shear rows: x: n=2 -> (v, 0, -1, 0, 0), n=3 -> (-w, 0, 0, 1, 0)
        //             y: n=1 -> (-u, 1, 0, 0, 0), n=3 -> (w, 0, 0, -1, 0)
        //             z: n=1 -> (u, -1, 0, 0, 0), n=2 -> (-v, 0, 1, 0, 0)
        if (d == 0) {
            if (n == 2) { l.set(0, F._v); l.mone(2); }
            else { l.set(0, -F._w); l.one(3); }
        } else if (d == 1) {
            if (n == 1) { l.set(0, -F._u); l.one(1); }
            else { l.set(0, F._w); l.mone(3); }
        } else {
            if (n == 1) { l.set(0, F._u); l.mone(1); }
            else { l.set(0, -F._v); l.one(2); }
        }
        return;
    }
    // species rows n = 4 .. E-2
    const int s = n + cf.NS() - E;
    l.set(0, -F._yi[s]);
    l.one(5 + s);
}

// RoeAverageRight_{x,y,z} (Eigen_matrix.hpp:86-155, :236-305, :386-455): column n of R.
template <class R>
void right_col(const Config &cf, int d, int n, const Face<R> &F, Vec<R> &r) {
    const int E = cf.E(), NCOP = cf.NCOP();
    const R b1 = F.b1, _c = F._c, _H = F._H;
    const R vel[3] = {F._u, F._v, F._w};
    const R un = vel[d];
    r.zero(E);
    if (n == 0 || n == E - 1) {
        r.one(0);
        for (int m = 0; m < 3; m++) {
            if (m == d) r.set(1 + m, n == 0 ? vel[m] - _c : vel[m] + _c);
            else r.set(1 + m, vel[m]);
        }
        r.set(4, n == 0 ? _H - un * _c : _H + un * _c);
        for (int m = 0; m < NCOP; m++) r.set(m + E - NCOP, F._yi[m]);
        return;
    }
    if (n >= 1 && n <= 3) {
        const int dn = d + 1;
        if (n == dn) {
            r.set(0, b1);
            r.set(1, F._u * b1); r.set(2, F._v * b1); r.set(3, F._w * b1);
            if (d == 2) { r.set(1, b1 * F._u); r.set(2, b1 * F._v); r.set(3, b1 * F._w); }
            r.set(4, _H * b1 - R(1.0));
            for (int m = 0; m < NCOP; m++) r.set(m + E - NCOP, b1 * F._yi[m]);
            return;
        }
        // x: n=2 -> (0,0,-1,0,-v), n=3 -> (0,0,0,1,w)
        // y: n=1 -> (0,1,0,0,u),   n=3 -> (0,0,0,-1,-w)
        // z: n=1 -> (0,-1,0,0,-u), n=2 -> (0,0,1,0,v)
        if (d == 0) {
            if (n == 2) { r.mone(2); r.set(4, -F._v); }
            else { r.one(3); r.set(4, F._w); }
        } else if (d == 1) {
            if (n == 1) { r.one(1); r.set(4, F._u); }
            else { r.mone(3); r.set(4, -F._w); }
        } else {
            if (n == 1) { r.mone(1); r.set(4, -F._u); }
            else { r.one(2); r.set(4, F._v); }
        }
        return;
    }
    const int s = n + cf.NS() - E;
    r.set(4, F.z[s]);
    r.one(5 + s);
}

// ---------------------------------------------------------------------------------------------
// WENO schemes (src/solver_Reconstruction/schemes)
// ---------------------------------------------------------------------------------------------
// weno5old_BODY, WENO5s_schemes.hpp:12-69 (double-precision branch)
template <class R>
R weno5_body(R v1, R v2, R v3, R v4, R v5) {
    R a1, a2, a3;
    const R dtwo = R(2.0), dtre = R(3.0);
    a1 = v1 - dtwo * v2 + v3;
    R s1 = R(13.0) * a1 * a1;
    a1 = v1 - R(4.0) * v2 + dtre * v3;
    s1 += dtre * a1 * a1;
    a1 = v2 - dtwo * v3 + v4;
    R s2 = R(13.0) * a1 * a1;
    a1 = v2 - v4;
    s2 += dtre * a1 * a1;
    a1 = v3 - dtwo * v4 + v5;
    R s3 = R(13.0) * a1 * a1;
    a1 = dtre * v3 - R(4.0) * v4 + v5;
    s3 += dtre * a1 * a1;
    const R tol = R(1.0E-6);
    s1 += tol, s2 += tol, s3 += tol;
    a1 = R(0.1) * s2 * s2 * s3 * s3;
    a2 = R(0.6) * s1 * s1 * s3 * s3;
    a3 = R(0.3) * s1 * s1 * s2 * s2;
    R tw1 = R(1.0) / (a1 + a2 + a3);
    a1 = a1 * tw1, a2 = a2 * tw1, a3 = a3 * tw1;
    s1 = a1 * (dtwo * v1 - R(7.0) * v2 + R(11.0) * v3);
    s2 = a2 * (-v2 + R(5.0) * v3 + dtwo * v4);
    s3 = a3 * (dtwo * v3 + R(5.0) * v4 - v5);
    return (s1 + s2 + s3);
}
// weno5old_GPU :71-95; f and m point at index 3 of the 8-point stencil arrays.
template <class R>
R weno5(const R *f, const R *m) {
    R temf = weno5_body(f[-2], f[-1], f[0], f[1], f[2]);
    R temm = weno5_body(m[3], m[2], m[1], m[0], m[-1]);
    return (temf + temm) * R(kSix);
}
// weno7_P / weno7_M body, WENO7s_schemes.hpp:8-67 (v1..v7 in upwind order)
template <class R>
R weno7_body(R v1, R v2, R v3, R v4, R v5, R v6, R v7) {
    const R ep = R(1.0e-7);
    const R C0 = R(1.0 / 35.0), C1 = R(12.0 / 35.0), C2 = R(18.0 / 35.0), C3 = R(4.0 / 35.0);
    R S10 = R(-2.0 / 6.0) * v1 + R(9.0 / 6.0) * v2 - R(18.0 / 6.0) * v3 + R(11.0 / 6.0) * v4;
    R S11 = R(1.0 / 6.0) * v2 - R(6.0 / 6.0) * v3 + R(3.0 / 6.0) * v4 + R(2.0 / 6.0) * v5;
    R S12 = R(-2.0 / 6.0) * v3 - R(3.0 / 6.0) * v4 + R(6.0 / 6.0) * v5 - R(1.0 / 6.0) * v6;
    R S13 = R(-11.0 / 6.0) * v4 + R(18.0 / 6.0) * v5 - R(9.0 / 6.0) * v6 + R(2.0 / 6.0) * v7;
    R S20 = -v1 + R(4.0) * v2 - R(5.0) * v3 + R(2.0) * v4;
    R S21 = v3 - R(2.0) * v4 + v5;
    R S22 = v4 - R(2.0) * v5 + v6;
    R S23 = R(2.0) * v4 - R(5.0) * v5 + R(4.0) * v6 - R(1.0) * v7;
    R S30 = -v1 + R(3.0) * v2 - R(3.0) * v3 + v4;
    R S31 = -v2 + R(3.0) * v3 - R(3.0) * v4 + v5;
    R S32 = -v3 + R(3.0) * v4 - R(3.0) * v5 + v6;
    R S33 = -v4 + R(3.0) * v5 - R(3.0) * v6 + v7;
    const R k13 = R(13.0 / 12.0), k1043 = R(1043.0 / 960.0), k112 = R(1.0 / 12.0);
    R S0 = S10 * S10 + k13 * S20 * S20 + k1043 * S30 * S30 + k112 * S10 * S30;
    R S1 = S11 * S11 + k13 * S21 * S21 + k1043 * S31 * S31 + k112 * S11 * S31;
    R S2 = S12 * S12 + k13 * S22 * S22 + k1043 * S32 * S32 + k112 * S12 * S32;
    R S3 = S13 * S13 + k13 * S23 * S23 + k1043 * S33 * S33 + k112 * S13 * S33;
    R a0 = C0 / ((ep + S0) * (ep + S0));
    R a1 = C1 / ((ep + S1) * (ep + S1));
    R a2 = C2 / ((ep + S2) * (ep + S2));
    R a3 = C3 / ((ep + S3) * (ep + S3));
    R sum = a0 + a1 + a2 + a3;
    R W0 = a0 / sum, W1 = a1 / sum, W2 = a2 / sum, W3 = a3 / sum;
    R q0 = R(-3.0 / 12.0) * v1 + R(13.0 / 12.0) * v2 - R(23.0 / 12.0) * v3 + R(25.0 / 12.0) * v4;
    R q1 = R(1.0 / 12.0) * v2 - R(5.0 / 12.0) * v3 + R(13.0 / 12.0) * v4 + R(3.0 / 12.0) * v5;
    R q2 = R(-1.0 / 12.0) * v3 + R(7.0 / 12.0) * v4 + R(7.0 / 12.0) * v5 - R(1.0 / 12.0) * v6;
    R q3 = R(3.0 / 12.0) * v4 + R(13.0 / 12.0) * v5 - R(5.0 / 12.0) * v6 + R(1.0 / 12.0) * v7;
    return W0 * q0 + W1 * q1 + W2 * q2 + W3 * q3;
}
// weno7_P(&pp[3]) + weno7_M(&mm[3]), WENO7s_schemes.hpp:8-128
template <class R>
R weno7(const R *f, const R *m) {
    R tp = weno7_body(f[-3], f[-2], f[-1], f[0], f[1], f[2], f[3]);
    R tm = weno7_body(m[4], m[3], m[2], m[1], m[0], m[-1], m[-2]);
    return tp + tm;
}

// WENOCU6_BODYGPU, WENO6s_schemes.hpp:5-55: the three WENO5 indicators, a sixth-order global
// indicator s6 from the tau_6k differences, the CU6 weights 20 + |s6 - s55| / (s_k + eps) with
// linear weights (0.05, 0.45, 0.45, 0.05) and the four candidates; v1..v6 in upwind order.
template <class R>
R wenocu6_body(R v1, R v2, R v3, R v4, R v5, R v6, R eps) {
    using std::fabs;
    R s11 = v1 - R(2.0) * v2 + v3;
    R s12 = v1 - R(4.0) * v2 + R(3.0) * v3;
    R s1 = R(13.0) * s11 * s11 + R(3.0) * s12 * s12;
    R s21 = v2 - R(2.0) * v3 + v4;
    R s22 = v2 - v4;
    R s2 = R(13.0) * s21 * s21 + R(3.0) * s22 * s22;
    R s31 = v3 - R(2.0) * v4 + v5;
    R s32 = R(3.0) * v3 - R(4.0) * v4 + v5;
    R s3 = R(13.0) * s31 * s31 + R(3.0) * s32 * s32;
    R tau61 = (R(259.0) * v6 - R(1895.0) * v5 + R(6670.0) * v4 - R(2590.0) * v3 - R(2785.0) * v2 + R(341.0) * v1) *
              R(1.0 / 5760.0);
    R tau62 = -(v5 - R(12.0) * v4 + R(22.0) * v3 - R(12.0) * v2 + v1) * R(1.0 / 16.0);
    R tau63 = -(R(7.0) * v6 - R(47.0) * v5 + R(94.0) * v4 - R(70.0) * v3 + R(11.0) * v2 + R(5.0) * v1) * R(1.0 / 144.0);
    R tau64 = (v5 - R(4.0) * v4 + R(6.0) * v3 - R(4.0) * v2 + v1) * R(1.0 / 24.0);
    R tau65 = -(-v6 + R(5.0) * v5 - R(10.0) * v4 + R(10.0) * v3 - R(5.0) * v2 + v1) * R(1.0 / 120.0);
    const R a1a1 = R(1.0), a2a2 = R(13.0 / 3.0), a1a3 = R(0.5), a3a3 = R(3129.0 / 80.0), a2a4 = R(4.2);
    const R a1a5 = R(0.125), a4a4 = R(87617.0 / 140.0), a3a5 = R(14127.0 / 224.0), a5a5 = R(252337135.0 / 16128.0);
    R s6 = (tau61 * tau61 * a1a1 + tau62 * tau62 * a2a2 + tau61 * tau63 * a1a3 + tau63 * tau63 * a3a3 +
            tau62 * tau64 * a2a4 + tau61 * tau65 * a1a5 + tau64 * tau64 * a4a4 + tau63 * tau65 * a3a5 +
            tau65 * tau65 * a5a5) * R(12.0);
    R s55 = (s1 + s3 + R(4.0) * s2) * R(kSix);
    R s5 = fabs(s6 - s55);
    R r0 = R(20.0);
    R r1 = r0 + s5 / (s1 + eps);
    R r2 = r0 + s5 / (s2 + eps);
    R r3 = r0 + s5 / (s3 + eps);
    R r4 = r0 + s5 / (s6 + eps);
    R a1 = R(0.05) * r1, a2 = R(0.45) * r2, a3 = R(0.45) * r3, a4 = R(0.05) * r4;
    R tw1 = R(1.0) / (a1 + a2 + a3 + a4);
    R w1 = a1 * tw1, w2 = a2 * tw1, w3 = a3 * tw1, w4 = a4 * tw1;
    R temp = R(0.0);
    temp += w1 * (R(2.0) * v1 - R(7.0) * v2 + R(11.0) * v3);
    temp += w2 * (-v2 + R(5.0) * v3 + R(2.0) * v4);
    temp += w3 * (R(2.0) * v3 + R(5.0) * v4 - v5);
    temp += w4 * (R(11.0) * v4 - R(7.0) * v5 + R(2.0) * v6);
    return temp;
}
// WENOCU6_GPU, WENO6s_schemes.hpp:58-84: epsilon = 1e-8 dl^2 with dl the cell size along the sweep
template <class R>
R wenocu6(const R *f, const R *m, R dl) {
    const R eps = R(1.e-8) * dl * dl;
    R temf = wenocu6_body(f[-2], f[-1], f[0], f[1], f[2], f[3], eps);
    R temm = wenocu6_body(m[3], m[2], m[1], m[0], m[-1], m[-2], eps);
    return (temf + temm) * R(kSix);
}

// ---------------------------------------------------------------------------------------------
// Convective flux at face (i+1/2) in direction d:
// ReconstructFlux{X,Y,Z}, Reconstruction_kernels.hpp:8-199 with MARCO_FLUXWALL_WENO5 / _WENO7
// (Eigen_callback.h:127-230).
// ---------------------------------------------------------------------------------------------
template <class R>
void face_flux(const Config &cf, const ThermoTable &tt, const Fields<R> &f, const std::vector<R> &UI, int d, int i, int j,
               int k, R *Fwall_out) {
    using std::fabs;
    using std::fmax;
    const xfg_block &b = cf.bl;
    const int E = cf.E();
    const size_t Xmax = b.Xmax, Ymax = b.Ymax;
    const size_t stride = d == 0 ? 1 : (d == 1 ? Xmax : Xmax * Ymax);
    const size_t id_l = Xmax * Ymax * k + Xmax * j + i;
    const size_t id_r = id_l + stride;
    const std::vector<R> &Fl = d == 0 ? f.FluxF : (d == 1 ? f.FluxG : f.FluxH);
    const std::vector<R> &eig = f.eig[d];
    Face<R> F;
    face_state(cf, tt, f, id_l, id_r, F);
    const int order = cf.sc.scheme_order;
    const int at = cf.sc.artificial_type;
    R out[kMaxE];
    for (int n = 0; n < E; n++) out[n] = R(0.0);
    R acc[kMaxE];
    bool first[kMaxE];
    for (int n = 0; n < E; n++) first[n] = true;
    for (int n = 0; n < E; n++) {
        Vec<R> l;
        R ev;
        left_row(cf, d, n, F, l, ev);
        R av;
        if (order == 7) {
            R elm = ev;
            R ll = eig[E * id_l + n], lr = eig[E * id_r + n];
            if (ll * lr < R(0.0))
                for (int m = -3; m < 5; m++) elm = fmax(elm, fabs(eig[E * (id_l + (long)m * (long)stride) + n]));
            av = at == XFG_ROE ? ev : (at == XFG_LLF ? elm : f.eigen_block[d][n]);
        } else {
            R elm = R(0.0);
            for (int m = -2; m < 4; m++) elm = fmax(elm, fabs(eig[E * (id_l + (long)m * (long)stride) + n]));
            av = at == XFG_ROE ? ev : (at == XFG_LLF ? elm : f.eigen_block[d][n]);
        }
        // project U and F at points m = -3..4 (index m+3); WENO5 and WENO-CU6 read m = -2..3 only
        R pp[8], mm[8];
        const int m0 = order == 7 ? -3 : -2, m1 = order == 7 ? 4 : 3;
        for (int m = m0; m <= m1; m++) {
            size_t idm = id_l + (long)m * (long)stride;
            R uf = dot(l, &UI[E * idm], E);
            R ff = dot(l, &Fl[E * idm], E);
            pp[m + 3] = R(0.5) * (ff + av * uf);
            mm[m + 3] = R(0.5) * (ff - av * uf);
        }
        const R dl = R(d == 0 ? b.dx : (d == 1 ? b.dy : b.dz));
        R f_flux = order == 7 ? weno7(&pp[3], &mm[3]) : (order == 6 ? wenocu6(&pp[3], &mm[3], dl) : weno5(&pp[3], &mm[3]));
        Vec<R> r;
        right_col(cf, d, n, F, r);
        // _p[n][n1] = f_flux * r[n1]; Fwall[n1] = sum_n _p[n][n1]
        for (int n1 = 0; n1 < E; n1++) {
            R t;
            switch (r.k[n1]) {
            case KZ: continue;
            case KP1: t = f_flux; break;
            case KM1: t = -f_flux; break;
            default: t = f_flux * r.v[n1]; break;
            }
            acc[n1] = first[n1] ? t : acc[n1] + t;
            first[n1] = false;
        }
    }
    for (int n = 0; n < E; n++) Fwall_out[n] = first[n] ? R(0.0) : acc[n];
    (void)out;
}

// max over cells id in [0, n) of term(id), starting from init: the reference's SYCL max
// reductions, over the threads (fmax is order-independent, so the result does not depend on them).
template <class R, class T>
R max_over_cells(long n, R init, T term) {
    using std::fmax;
    R mx = init;
#pragma omp parallel
    {
        R loc = init;
#pragma omp for schedule(static) nowait
        for (long id = 0; id < n; id++) loc = fmax(loc, term(id));
#pragma omp critical(xfo_max_over_cells)
        mx = fmax(mx, loc);
    }
    return mx;
}

// GetLocalEigen, Eigen_value.hpp:5-36, for direction d on all cells.
template <class R>
void local_eigen(const Config &cf, Fields<R> &f, int d) {
    const long n = (long)cf.ncell();
    const int E = cf.E();
    std::vector<R> &eig = f.eig[d];
#pragma omp parallel for schedule(static)
    for (long id = 0; id < n; id++) {
        if (cf.sc.scheme_order == 7) {
            for (int m = 0; m < E; m++) eig[E * id + m] = R(0.0);
            continue;
        }
        const R AA = R(d == 0 ? 1.0 : 0.0), BB = R(d == 1 ? 1.0 : 0.0), CC = R(d == 2 ? 1.0 : 0.0);
        // uu = AA*u + BB*v + CC*w, evaluated exactly (the zero terms contribute +0.0)
        R uu = d == 0 ? f.u[id] : (d == 1 ? f.v[id] : f.w[id]);
        (void)AA, (void)BB, (void)CC;
        R uuPc = uu + f.c[id], uuMc = uu - f.c[id];
        eig[E * id + 0] = uuMc;
        for (int m = 1; m < E - 1; m++) eig[E * id + m] = uu;
        eig[E * id + E - 1] = uuPc;
    }
}

// GetLU, ConVenction_block.hpp:10-617 (inviscid, no positivity preserving), in its three phases:
// local eigenvalues + global LF maxima, face fluxes per direction, flux divergence.
template <class R>
void lu_eigen(const Config &cf, Fields<R> &f) {
    using std::fabs;
    using std::fmax;
    const xfg_block &b = cf.bl;
    const int E = cf.E();
    const int dims[3] = {b.DimX, b.DimY, b.DimZ};
    const long ncell = (long)cf.ncell();
    for (int d = 0; d < 3; d++) {
        if (!dims[d]) continue;
        local_eigen(cf, f, d);
        // ConVenction_block.hpp:115-215: the SYCL max reduction folds in the previous value of
        // eigen_block (zeroed once at allocation, src/Fluids.cpp:421-429), so the GLF maxima are
        // running maxima over every GetLU call of the run
        const std::vector<R> &eg = f.eig[d];
        for (int n = 0; n < E; n++)
            f.eigen_block[d][n] = max_over_cells(ncell, f.eigen_block[d][n], [&](long id) { return fabs(eg[E * id + n]); });
    }
}

// ReconstructFlux{X,Y,Z} launch ranges, ConVenction_block.hpp:217-320: faces i+1/2 for
// i in [Bwidth-1, inner+Bwidth) along d, inner cells along the other directions.
template <class R>
void lu_faces(const Config &cf, Fields<R> &f, const std::vector<R> &UI, int d) {
    const xfg_block &b = cf.bl;
    const ThermoTable tt = cf.table();
    const int E = cf.E();
    const int i0 = b.Bwidth_X - (d == 0 ? 1 : 0), j0 = b.Bwidth_Y - (d == 1 ? 1 : 0), k0 = b.Bwidth_Z - (d == 2 ? 1 : 0);
    const int i1 = b.X_inner + b.Bwidth_X, j1 = b.Y_inner + b.Bwidth_Y, k1 = b.Z_inner + b.Bwidth_Z;
    std::vector<R> &Fw = f.Fw[d];
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = k0; k < k1; k++)
        for (int j = j0; j < j1; j++)
            for (int i = i0; i < i1; i++) {
                size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                face_flux(cf, tt, f, UI, d, i, j, k, &Fw[E * id]);
            }
}

// UpdateFluidLU, Reconstruction_kernels.hpp:201-234, inner cells.
template <class R>
void lu_divergence(const Config &cf, Fields<R> &f) {
    const xfg_block &b = cf.bl;
    const int E = cf.E();
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = b.Bwidth_Z; k < b.Z_inner + b.Bwidth_Z; k++)
        for (int j = b.Bwidth_Y; j < b.Y_inner + b.Bwidth_Y; j++)
            for (int i = b.Bwidth_X; i < b.X_inner + b.Bwidth_X; i++) {
                size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                size_t im = id - 1, jm = id - b.Xmax, km = id - (size_t)b.Xmax * b.Ymax;
                for (int n = 0; n < E; n++) {
                    R LU0 = R(0.0);
                    bool first = true;  // 0.0 + t == t
                    if (b.DimX) { R t = (f.Fw[0][E * im + n] - f.Fw[0][E * id + n]) * b._dx; LU0 = t; first = false; }
                    if (b.DimY) { R t = (f.Fw[1][E * jm + n] - f.Fw[1][E * id + n]) * b._dy; LU0 = first ? t : LU0 + t; first = false; }
                    if (b.DimZ) { R t = (f.Fw[2][E * km + n] - f.Fw[2][E * id + n]) * b._dz; LU0 = first ? t : LU0 + t; first = false; }
                    f.LU[E * id + n] = LU0;
                }
            }
}

// PositivityPreservingKernel, FDM_Method/positive-definite_eigen/PositivityPreserving_kernels.hpp:5-76,
// launched per direction over the inner cells after all face sweeps (ConVenction_block.hpp:328-410):
// the face i+1/2 of inner cell i is blended toward the Lax-Friedrichs flux with
// lambda_0 = uvw_c_max[d] (the maxima of the last GetDt) and lambda = CFL / lambda_0, first for
// the density floor min(rho, 1e-13) of both neighbours, then (mixtures) for each mass fraction
// with floor 0. The theta of each species blends the already blended face flux, while the
// predicted states of the species test keep the density-corrected FF.
template <class R>
inline R pp_min(R a, R b) { return (b < a) ? b : a; }  // sycl::min of the shim
template <class R>
inline R pp_max(R a, R b) { return (a < b) ? b : a; }  // sycl::max of the shim
template <class R>
void pp_limit(const Config &cf, Fields<R> &f, const std::vector<R> &UI, int d) {
    const xfg_block &b = cf.bl;
    const int E = cf.E(), NCOP = cf.NCOP();
    const size_t stride = d == 0 ? 1 : (d == 1 ? (size_t)b.Xmax : (size_t)b.Xmax * b.Ymax);
    const std::vector<R> &Fl = d == 0 ? f.FluxF : (d == 1 ? f.FluxG : f.FluxH);
    std::vector<R> &Fw = f.Fw[d];
    const R lambda_0 = f.uvw_c_max[d];
    const R lambda = R(b.CFLnumber) / lambda_0;
    const R eps_rho = R(1.0e-13), eps_y = R(0.0);
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = b.Bwidth_Z; k < b.Z_inner + b.Bwidth_Z; k++)
        for (int j = b.Bwidth_Y; j < b.Y_inner + b.Bwidth_Y; j++)
            for (int i = b.Bwidth_X; i < b.X_inner + b.Bwidth_X; i++) {
                const size_t id_l = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i, id_r = id_l + stride;
                const R *UU = &UI[E * id_l], *UP = &UI[E * id_r];
                const R *Fll = &Fl[E * id_l], *Flr = &Fl[E * id_r];
                R *Fwall = &Fw[E * id_l];
                R F_LF[kMaxE], FF_LF[kMaxE], FF[kMaxE];
                for (int n = 0; n < E; n++) {
                    F_LF[n] = R(0.5) * (Fll[n] + Flr[n] + lambda_0 * (UU[n] - UP[n]));
                    FF_LF[n] = R(2.0) * lambda * F_LF[n];
                    FF[n] = R(2.0) * lambda * Fwall[n];
                }
                R theta_u = R(1.0), theta_p = R(1.0);
                R rho_min = pp_min(UU[0], eps_rho);
                if (UU[0] - FF[0] < rho_min) theta_u = (UU[0] - FF_LF[0] - rho_min) / (FF[0] - FF_LF[0]);
                rho_min = pp_min(UP[0], eps_rho);
                if (UP[0] + FF[0] < rho_min) theta_p = (UP[0] + FF_LF[0] - rho_min) / (FF_LF[0] - FF[0]);
                R theta = pp_min(theta_u, theta_p);
                for (int n = 0; n < E; n++) {
                    FF[n] = (R(1.0) - theta) * FF_LF[n] + theta * FF[n];
                    Fwall[n] = (R(1.0) - theta) * F_LF[n] + theta * Fwall[n];
                }
                if (NCOP > 0) {
                    const R _rhoq = R(1.0) / (UU[0] - FF[0]), _rhou = R(1.0) / (UU[0] - FF_LF[0]);
                    const R _rhoqp = R(1.0) / (UP[0] + FF[0]), _rhoup = R(1.0) / (UP[0] + FF_LF[0]);
                    for (int n = 0; n < NCOP; n++) {
                        const int tid = n + 5;
                        const R yq = (UU[tid] - FF[tid]) * _rhoq, yu = (UU[tid] - FF_LF[tid]) * _rhou;
                        const R yqp = (UP[tid] + FF[tid]) * _rhoqp, yup = (UP[tid] + FF_LF[tid]) * _rhoup;
                        theta_u = R(1.0), theta_p = R(1.0);
                        if (yq < eps_y) {
                            const R yi_min = pp_min(yu, eps_y);
                            theta_u = (yu - yi_min + R(1.0e-40)) / (yu - yq + R(1.0e-40));
                        }
                        if (yqp < eps_y) {
                            const R yi_min = pp_min(yup, eps_y);
                            theta_p = (yup - yi_min + R(1.0e-40)) / (yup - yqp + R(1.0e-40));
                        }
                        theta = pp_min(theta_u, theta_p);
                        for (int nn = 0; nn < E; nn++) Fwall[nn] = (R(1.0) - theta) * F_LF[nn] + theta * Fwall[nn];
                    }
                }
            }
}

// ---------------------------------------------------------------------------------------------
// Viscous, heat-conduction and diffusion fluxes (Visc / Visc_Heat / Visc_Diffu), fourth order:
// GetCellCenterDerivative (viscosity/Visc_block.hpp:7-84), Gettransport_coeff_aver
// (Visc_kernels.hpp:226-245, Visc_device.h), the diffusion limiter reduction and
// GetWallViscousFlux{X,Y,Z} (Fourth_Order/Visc_Order_kernels.hpp, Flux_discrete.h), launched by
// ConVenction_block.hpp:419-566 after the face sweeps (and the positivity limiter).
// ---------------------------------------------------------------------------------------------
enum { DUCX, DVCX, DWCX, DUCY, DVCY, DWCY, DUCZ, DVCZ, DWCZ };
constexpr double kTwle = 1.0 / 12.0, kTwfr = 1.0 / 24.0, kSxtn = 1.0 / 16.0;

// Viscosity / Thermal_conductivity / the numerator of GetDkj (Visc_device.h:8-100): exp of the
// fitted cubic in ln T (Horner from the highest power)
template <class R>
R fit_exp(const double *c, R T) {
    using std::exp;
    using std::log;
    R v = R(c[XFG_FIT_ORDER - 1]);
    for (int i = XFG_FIT_ORDER - 2; i >= 0; i--) v = v * log(T) + R(c[i]);
    return exp(v);
}
// PHI (Visc_device.h:30-38), the Wilke mixing factor of species k with j
template <class R>
R wilke_phi(const xfg_transport &tr, int k, int j, R T) {
    using std::pow;
    using std::sqrt;
    const double *sk = &tr.species_chara[k * XFG_SPCH], *sj = &tr.species_chara[j * XFG_SPCH];
    const int ik = (int)sk[8], ij = (int)sj[8];
    R phi = R(pow(sj[6] / sk[6], 0.25)) *
            pow(fit_exp(&tr.visc[ik * XFG_FIT_ORDER], T) / fit_exp(&tr.visc[ij * XFG_FIT_ORDER], T), R(0.5));
    phi = (phi + R(1.0)) * (phi + R(1.0)) * R(0.5) / R(sqrt(2.0));
    phi = phi * R(pow(1.0 + sk[6] / sj[6], -0.5));
    return phi;
}

// GetInnerCellCenterDerivativeKernel (Fourth_Order/Visc_Order_kernels.hpp:16-72) on the cells
// [B-2, inner+B+2) of each active direction, then CenterDerivativeBCKernel{X,Y,Z}
// (Visc_kernels.hpp:7-204) on the ghost layers in that order. Derivatives along an absent
// direction are zero (the reference multiplies a read outside the array by DimZ_t = 0).
template <class R>
void velocity_derivatives(const Config &cf, Fields<R> &f) {
    const xfg_block &b = cf.bl;
    const int dims[3] = {b.DimX, b.DimY, b.DimZ};
    const int r0[3] = {b.DimX ? b.Bwidth_X - 2 : 0, b.DimY ? b.Bwidth_Y - 2 : 0, b.DimZ ? b.Bwidth_Z - 2 : 0};
    const int r1[3] = {b.DimX ? b.X_inner + b.Bwidth_X + 2 : 1, b.DimY ? b.Y_inner + b.Bwidth_Y + 2 : 1,
                       b.DimZ ? b.Z_inner + b.Bwidth_Z + 2 : 1};
    const size_t n = cf.ncell(), st[3] = {1, (size_t)b.Xmax, (size_t)b.Xmax * b.Ymax};
    const R inv[3] = {R(b._dx), R(b._dy), R(b._dz)};
    const R dt[3] = {R(b.DimX), R(b.DimY), R(b.DimZ)};
    const std::vector<R> *vel[3] = {&f.u, &f.v, &f.w};
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = r0[2]; k < r1[2]; k++)
        for (int j = r0[1]; j < r1[1]; j++)
            for (int i = r0[0]; i < r1[0]; i++) {
                const size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                for (int d = 0; d < 3; d++)      // derivative direction
                    for (int c = 0; c < 3; c++) {  // velocity component
                        R val = R(0.0);
                        if (dims[d]) {
                            const std::vector<R> &q = *vel[c];
                            val = (R(8.0) * (q[id + st[d]] - q[id - st[d]]) - (q[id + 2 * st[d]] - q[id - 2 * st[d]])) *
                                  inv[d] * R(kTwle) * dt[d];
                            if (c != d) val = val * dt[c];
                        } else {
                            val = R(0.0) * dt[d];
                        }
                        f.Vde[(3 * d + c) * n + id] = val;
                    }
            }
    // ghost layers: the four components each direction's flux reads
    static const int comps[3][4] = {{DUCY, DUCZ, DVCY, DWCZ}, {DVCX, DVCZ, DUCX, DWCZ}, {DWCX, DWCY, DUCX, DVCY}};
    const int ext[3] = {b.Xmax, b.Ymax, b.Zmax}, inner[3] = {b.X_inner, b.Y_inner, b.Z_inner};
    const int bw[3] = {b.Bwidth_X, b.Bwidth_Y, b.Bwidth_Z};
    for (int d = 0; d < 3; d++) {
        if (!dims[d]) continue;
        const int ta = d == 0 ? b.Ymax : b.Xmax, tb = d == 2 ? b.Ymax : b.Zmax;
        for (int side = 0; side < 2; side++) {
            const int BC = b.Boundarys[2 * d + side];
            const int mirror_offset = side == 0 ? 0 : inner[d];
            const int index_inner = side == 0 ? bw[d] : ext[d] - bw[d] - 1;
            const int sign = side == 0 ? 1 : -1;
            for (int q = 0; q < tb; q++)
                for (int p = 0; p < ta; p++)
                    for (int g = 0; g < bw[d]; g++) {
                        const int cn = side == 0 ? g : g + ext[d] - bw[d];
                        auto cell = [&](int c) {
                            const int i = d == 0 ? c : p, j = d == 0 ? p : (d == 1 ? c : q), k = d == 2 ? c : q;
                            return (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                        };
                        const size_t id = cell(cn);
                        long src = -1;
                        R sgn = R(1.0);
                        switch (BC) {
                        case XFG_SYMMETRY: src = (long)cell(2 * (bw[d] + mirror_offset) - 1 - cn); break;
                        case XFG_PERIODIC: src = (long)cell(cn + sign * inner[d]); break;
                        case XFG_OUTFLOW: src = (long)cell(index_inner); break;
                        case XFG_NSLIPWALL:
                            // the mirror of X and Y; the reference's Z case indexes k - offset
                            // (Visc_kernels.hpp:183), outside the array
                            src = (long)cell(2 * (bw[d] + mirror_offset) - 1 - cn), sgn = R(-1.0);
                            break;
                        case XFG_INFLOW:
                            for (int m = 0; m < 4; m++) f.Vde[comps[d][m] * n + id] = R(0.0);
                            break;
                        default: break;  // viscWall, slipWall, innerBlock: unchanged
                        }
                        if (src >= 0)
                            for (int m = 0; m < 4; m++)
                                f.Vde[comps[d][m] * n + id] = sgn == R(1.0) ? f.Vde[comps[d][m] * n + src]
                                                                             : -f.Vde[comps[d][m] * n + src];
                    }
        }
    }
}

// Gettransport_coeff_aver (Visc_kernels.hpp:226-245) with Get_transport_coeff_aver
// (Visc_device.h:106-177) on every cell: mole fractions (get_xi), Wilke-averaged viscosity and
// thermal conductivity, species enthalpies and mixture-averaged diffusion coefficients.
template <class R>
void transport(const Config &cf, Fields<R> &f) {
    using std::ceil;
    const xfg_transport &tr = cf.tr;
    const ThermoTable tt = cf.table();
    const int NS = cf.NS();
    const bool heat = cf.sc.viscous & 2, diffu = cf.sc.viscous & 4;
    const long n = (long)cf.ncell();
#pragma omp parallel for schedule(static)
    for (long id = 0; id < n; id++) {
        const R T = f.T[id], rho = f.rho[id], p = f.p[id];
        R X[kMaxE];
        R C_total = R(0.0);
        for (int i = 0; i < NS; i++) {
            X[i] = f.y[NS * id + i] * R(cf.th._Wi[i]) * R(1e-3) * rho;
            C_total = C_total + X[i];
        }
        const R _C = R(1.0) / C_total;
        for (int i = 0; i < NS; i++) X[i] = X[i] * _C;
        if (diffu)
            for (int k = 0; k < NS; k++) f.hi[NS * id + k] = enthalpy(tt, T, tt.Ri[k], k);
        R mu = R(0.0), kap = R(0.0);
        for (int k = 0; k < NS; k++) {
            R den = R(0.0);
            for (int i = 0; i < NS; i++) den = den + X[i] * wilke_phi(tr, k, i, T);
            const R _den = R(1.0) / den;
            const int ik = (int)tr.species_chara[k * XFG_SPCH + 8];
            mu = mu + X[k] * fit_exp(&tr.visc[ik * XFG_FIT_ORDER], T) * _den;
            if (heat) kap = kap + X[k] * fit_exp(&tr.therm[ik * XFG_FIT_ORDER], T) * _den;
        }
        f.mu[id] = mu;
        if (heat) f.kappa[id] = kap;
        if (diffu) {
            auto dkj = [&](int a, int c) {  // GetDkj: fit / p
                const int ia = (int)tr.species_chara[a * XFG_SPCH + 8], ic = (int)tr.species_chara[c * XFG_SPCH + 8];
                return fit_exp(&tr.dkj[(ia * NS + ic) * XFG_FIT_ORDER], T) / p;
            };
            for (int k = 0; k < NS; k++) {
                R Dk;
                if (NS > 1) {
                    R t1 = R(0.0), t2 = R(1.0e-20);
                    for (int i = 0; i < NS; i++)
                        if (i != k) {
                            t1 += (X[i] + R(1.0e-40)) * R(cf.th.Wi[i]);
                            t2 += (X[i] + R(1.0e-40)) / (dkj(i, k) + R(1.0e-40));
                        }
                    if (!(R(0.0) < ceil(t1))) Dk = dkj(k, k);  // sycl::step(ceil(t1), 0) == 1
                    else Dk = t1 / t2 / rho * C_total;
                } else {
                    Dk = dkj(0, 0);
                }
                Dk *= R(1.0e-1);
                f.Dkm[NS * id + k] = Dk < R(1.0e-10) ? R(1.0e-10) : Dk;  // sycl::max(Dk, 1e-10)
            }
        }
    }
}

// GetWallViscousFlux{X,Y,Z} (Fourth_Order/Visc_Order_kernels.hpp:74-342 with Flux_discrete.h) on
// the faces i+1/2, i in [B-1, inner+B) along d: F_wall_v subtracted from the face flux.
template <class R>
void viscous_faces(const Config &cf, Fields<R> &f, int d, const R *yil_lim, const R *diffu_lim) {
    const xfg_block &b = cf.bl;
    const int E = cf.E(), NS = cf.NS();
    const bool heat = cf.sc.viscous & 2, diffu = cf.sc.viscous & 4;
    const size_t n = cf.ncell();
    const size_t st = d == 0 ? 1 : (d == 1 ? (size_t)b.Xmax : (size_t)b.Xmax * b.Ymax);
    const R _dl = R(d == 0 ? b._dx : (d == 1 ? b._dy : b._dz));
    const R dt[3] = {R(b.DimX), R(b.DimY), R(b.DimZ)};
    const int i0 = b.Bwidth_X - (d == 0 ? 1 : 0), j0 = b.Bwidth_Y - (d == 1 ? 1 : 0), k0 = b.Bwidth_Z - (d == 2 ? 1 : 0);
    const int i1 = b.X_inner + b.Bwidth_X, j1 = b.Y_inner + b.Bwidth_Y, k1 = b.Z_inner + b.Bwidth_Z;
    std::vector<R> &Fw = f.Fw[d];
    const std::vector<R> *vel[3] = {&f.u, &f.v, &f.w};
    // cross derivatives: in the momentum flux along c (c != d) the derivative of u_d along c; in the
    // normal momentum flux the divergence terms of the other two directions
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = k0; k < k1; k++)
        for (int j = j0; j < j1; j++)
            for (int i = i0; i < i1; i++) {
                const size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                const size_t m1 = id - st, p1 = id + st, p2 = id + 2 * st;
                auto half = [&](const std::vector<R> &a, size_t off = 0) {  // 4th-order face average
                    return (R(9.0) * (a[off + p1] + a[off + id]) - (a[off + p2] + a[off + m1])) * R(kSxtn);
                };
                auto grad = [&](const std::vector<R> &a, size_t off = 0) {  // 4th-order face gradient
                    return (R(27.0) * (a[off + p1] - a[off + id]) - (a[off + p2] - a[off + m1])) * _dl * R(kTwfr);
                };
                const R mue = half(f.mu);
                const R lamada = -R(2.0) * R(kOT) * mue;
                auto b27 = [&](const std::vector<R> &a) { return R(27.0) * (a[p1] - a[id]) - (a[p2] - a[m1]); };
                auto vd = [&](int c, size_t q) { return f.Vde[(size_t)c * n + q]; };
                R fv[3], hv[3];
                for (int c = 0; c < 3; c++) {
                    if (c == d) {
                        // (2 mue + lambda) du_d/dx_d + lambda (the two other diagonal derivatives)
                        const int oa = c == 0 ? DVCY : DUCX, ob = c == 2 ? DVCY : DWCZ;
                        fv[c] = (R(2.0) * mue + lamada) * b27(*vel[c]) * _dl * R(kTwfr);
                        fv[c] += lamada *
                                 (R(9.0) * (vd(oa, p1) + vd(oa, id)) - (vd(oa, p2) + vd(oa, m1)) +
                                  R(9.0) * (vd(ob, p1) + vd(ob, id)) - (vd(ob, p2) + vd(ob, m1))) *
                                 R(kSxtn);
                        hv[c] = half(*vel[c]);
                    } else {
                        // mue (du_c/dx_d + du_d/dx_c), the second from the cell-centre derivatives
                        const int cr = 3 * c + d;  // derivative of u_d along x_c
                        fv[c] = mue * b27(*vel[c]) * _dl * R(kTwfr) * dt[c];
                        fv[c] += mue * (R(9.0) * (vd(cr, p1) + vd(cr, id)) - (vd(cr, p2) + vd(cr, m1))) * R(kSxtn) * dt[c];
                        hv[c] = half(*vel[c]) * dt[c];
                    }
                }
                R F[kMaxE];
                F[0] = R(0.0), F[1] = fv[0], F[2] = fv[1], F[3] = fv[2];
                F[4] = fv[0] * hv[0] + fv[1] * hv[1] + fv[2] * hv[2];
                if (heat) {
                    R kk = half(f.kappa);
                    kk *= grad(f.T);
                    F[4] += kk;
                }
                if (diffu) {
                    const R rho_wall = half(f.rho);
                    R CorrectTerm = R(0.0), Dim_Yil = R(1.0e-20);
                    R Yi_wall[kMaxE];
                    for (int l = 0; l < NS; l++) {
                        auto yl = [&](size_t c) { return f.y[NS * c + l]; };
                        auto hl = [&](size_t c) { return f.hi[NS * c + l]; };
                        auto dl = [&](size_t c) { return f.Dkm[NS * c + l]; };
                        const R hi_wall = (R(9.0) * (hl(p1) + hl(id)) - (hl(p2) + hl(m1))) * R(kSxtn);
                        const R Dim_wall = (R(9.0) * (dl(p1) + dl(id)) - (dl(p2) + dl(m1))) * R(kSxtn);
                        R Yil = (R(27.0) * (yl(p1) - yl(id)) - (yl(p2) - yl(m1))) * _dl * R(kTwfr);
                        Yil = pp_min(pp_max(Yil, -yil_lim[l]), yil_lim[l]);
                        R Yw = (R(9.0) * (yl(p1) + yl(id)) - (yl(p2) + yl(m1))) * R(kSxtn);
                        Yi_wall[l] = pp_min(pp_max(Yw, R(1.0E-20)), R(1.0));
                        Dim_Yil = pp_min(pp_max(Dim_wall * Yil, -diffu_lim[l]), diffu_lim[l]);
                        CorrectTerm += Dim_Yil;
                        F[4] += rho_wall * hi_wall * Dim_Yil;
                    }
                    CorrectTerm *= rho_wall;
                    // every species takes the last species' Dim_Yil (MARCO_VIS_Diffu, Flux_discrete.h:57-61)
                    for (int p = 5; p < E; p++) F[p] = rho_wall * Dim_Yil - Yi_wall[p - 5] * CorrectTerm;
                } else {
                    for (int p = 5; p < E; p++) F[p] = R(0.0);
                }
                for (int c = 0; c < E; c++) Fw[E * id + c] -= F[c];
            }
}

template <class R>
void viscous_lu(const Config &cf, Fields<R> &f) {
    const xfg_block &b = cf.bl;
    const int dims[3] = {b.DimX, b.DimY, b.DimZ};
    const int NS = cf.NS();
    velocity_derivatives(cf, f);
    transport(cf, f);
    // diffusion limiters (ConVenction_block.hpp:457-503) of a single block: the Y range of the
    // inner cells (reductions seeded with 0) times Yil_limiter, and Dim_max = 0 * ... = 0 (the Dkm
    // reduction is not taken; only the MPI build resets it to 1)
    R yil[kMaxE], dlim[kMaxE];
    for (int nn = 0; nn < NS; nn++) {
        R ymin = R(0.0), ymax = R(0.0), Dmax = R(0.0);
        if (cf.sc.viscous & 4) {
            for (int k = b.Bwidth_Z; k < b.Z_inner + b.Bwidth_Z; k++)
                for (int j = b.Bwidth_Y; j < b.Y_inner + b.Bwidth_Y; j++)
                    for (int i = b.Bwidth_X; i < b.X_inner + b.Bwidth_X; i++) {
                        const size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                        const R yv = f.y[NS * id + nn];
                        ymin = pp_min(ymin, yv), ymax = pp_max(ymax, yv);
                    }
            ymax -= ymin;
            ymax *= R(cf.tr.yil_limiter);
            Dmax *= R(cf.tr.dim_limiter) * ymax;
        }
        yil[nn] = ymax, dlim[nn] = Dmax;
    }
    for (int d = 0; d < 3; d++)
        if (dims[d]) viscous_faces(cf, f, d, yil, dlim);
}

template <class R>
void compute_lu(const Config &cf, Fields<R> &f, const std::vector<R> &UI) {
    const int dims[3] = {cf.bl.DimX, cf.bl.DimY, cf.bl.DimZ};
    lu_eigen(cf, f);
    for (int d = 0; d < 3; d++)
        if (dims[d]) lu_faces(cf, f, UI, d);
    if (cf.sc.positivity)
        for (int d = 0; d < 3; d++)
            if (dims[d]) pp_limit(cf, f, UI, d);
    if (cf.sc.viscous) viscous_lu(cf, f);
    lu_divergence(cf, f);
}

// UpdateURK3rdKernel, Update_kernels.hpp:64-94, inner cells.
template <class R>
void update_rk3(const Config &cf, Fields<R> &f, int flag, R dt) {
    const xfg_block &b = cf.bl;
    const int E = cf.E();
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = b.Bwidth_Z; k < b.Z_inner + b.Bwidth_Z; k++)
        for (int j = b.Bwidth_Y; j < b.Y_inner + b.Bwidth_Y; j++)
            for (int i = b.Bwidth_X; i < b.X_inner + b.Bwidth_X; i++) {
                size_t id = (size_t)b.Xmax * b.Ymax * k + (size_t)b.Xmax * j + i;
                for (int n = 0; n < E; n++) {
                    size_t q = E * id + n;
                    if (flag == 1) f.U1[q] = f.U[q] + dt * f.LU[q];
                    else if (flag == 2) f.U1[q] = R(0.75) * f.U[q] + R(0.25) * f.U1[q] + R(0.25) * dt * f.LU[q];
                    else f.U[q] = (f.U[q] + R(2.0) * f.U1[q] + R(2.0) * dt * f.LU[q]) * R(kOT);
                }
            }
}

// GetDt, GlobalDt_block.hpp:6-114: max over all cells of |u_d| + sqrt(1.4 p / rho).
template <class R>
R get_dt(const Config &cf, Fields<R> &f) {
    using std::fabs;
    using std::fmax;
    using std::sqrt;
    const xfg_block &b = cf.bl;
    const long n = (long)cf.ncell();
    const std::vector<R> *vel[3] = {&f.u, &f.v, &f.w};
    const int dims[3] = {b.DimX, b.DimY, b.DimZ};
    for (int d = 0; d < 3; d++) {
        f.uvw_c_max[d] = R(0.0);
        if (!dims[d]) continue;
        const std::vector<R> &vd = *vel[d];
        f.uvw_c_max[d] = max_over_cells(n, R(0.0), [&](long id) {
            R c_local = sqrt(R(1.4) * f.p[id] / f.rho[id]);
            return fabs(vd[id]) + c_local;
        });
    }
    R dtref = f.uvw_c_max[0] * b._dx + f.uvw_c_max[1] * b._dy + f.uvw_c_max[2] * b._dz;
    return R(b.CFLnumber) / dtref;
}

}  // namespace xfo
