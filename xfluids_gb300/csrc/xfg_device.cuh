// xfg_device.cuh - device functions of the convective right-hand side (FP64 and FP32 forms).
//
// Each function restates one reference device function (cited per function) with its operation
// order. The state lives in HBM as SoA arrays (component n of cell id at n*pitch + id), so that a
// warp reads 32 consecutive cells of one component per load. Compile-time template parameters:
//   NS  - NUM_SPECIES (1 without COP), E = NS + 4 with COP else 5
//   COP - multi-component mixture
//   D   - sweep direction 0/1/2 (x/y/z)
//   T   - arithmetic type of the reconstruction (double, or float in the mixed form)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/xfluids_gb300.h"

#ifndef XFG_KNS
#define XFG_KNS fast
#endif

// Units compiled with -DXFG_STRICT (and --fmad=false) keep the reference's operation sequence
// everywhere; the others may use the rearranged single-gas FP64 fast path.
#ifdef XFG_STRICT
#define XFG_STRICT_BUILD 1
#else
#define XFG_STRICT_BUILD 0
#endif

namespace xfg {

constexpr double kRu = 6.02214076e26 * 1.380649e-23 * 1.0E-3;  // global_setup.h:48-54
constexpr double kOT = 1.0 / 3.0;
constexpr double kSix = 1.0 / 6.0;

template <bool COP, int NS>
struct Sys {
    static constexpr int E = COP ? NS + 4 : 5;
    static constexpr int NCOP = COP ? NS - 1 : 0;
};

// Thermo tables passed by value to the kernels (lands in the constant bank).
struct DevThermo {
    double Ri[XFG_MAX_SPECIES];
    double _Wi[XFG_MAX_SPECIES];
    double Hia[XFG_MAX_SPECIES * 21];
    double Hib[XFG_MAX_SPECIES * 6];
    int nasa;
    double ncop_gamma;
    const double *hsc;  // mixed mixtures: device copy of scaled_thermo_table (THERMO_SC_DOUBLES)
    const float *hscf;  // the same table rounded to FP32 (the FP32 sound-speed cell terms)
};

// Enthalpy polynomials scaled by R_n for the mixed form, per species n and temperature range rg
// (JANAF: rg 0 above 1000 K, 1 below; NASA-9: nasa_range), 8 coefficients at (n * 3 + rg) * 8:
//   JANAF   h_n = T (c0 + T (c1 + T (c2 + T (c3 + T c4)))) + c5,
//           c = R_n (a0, a1 / 2, a2 / 3, a3 / 4, a4 / 5, a5) (HeatCapacity / get_Enthalpy_JANAF);
//   NASA-9  h_n = c0 / T + c1 ln T + T (c2 + T (c3 + T (c4 + T (c5 + T c6)))) + c7,
//           c = R_n (-a0, a1, a2, a3 / 2, a4 / 3, a5 / 4, a6 / 5, b0);
// then Cp_n(200 K) at THERMO_SC_CP200 + n (the tables' linear extrapolation below 200 K). The
// same polynomials as enthalpy() / heat_capacity() with the constant factors applied once.
constexpr int THERMO_SC_CP200 = XFG_MAX_SPECIES * 3 * 8;
constexpr int THERMO_SC_DOUBLES = THERMO_SC_CP200 + XFG_MAX_SPECIES;
// device bytes of the table in both precisions (the FP32 copy follows the FP64 one)
constexpr int THERMO_SC_BYTES = THERMO_SC_DOUBLES * 12;
inline void scaled_thermo_table(const DevThermo &t, double *out) {
    for (int q = 0; q < THERMO_SC_DOUBLES; q++) out[q] = 0.0;
    for (int n = 0; n < XFG_MAX_SPECIES; n++) {
        const double R = t.Ri[n];
        for (int rg = 0; rg < (t.nasa ? 3 : 2); rg++) {
            const double *a = t.Hia + n * 21 + rg;
            double *c = out + (n * 3 + rg) * 8;
            if (t.nasa) {
                c[0] = -R * a[0], c[1] = R * a[3], c[2] = R * a[6], c[3] = R * (0.5 * a[9]);
                c[4] = R * (a[12] / 3.0), c[5] = R * (0.25 * a[15]), c[6] = R * (0.2 * a[18]), c[7] = R * t.Hib[n * 6 + rg];
            } else {
                c[0] = R * a[0], c[1] = R * (0.5 * a[3]), c[2] = R * (a[6] / 3.0), c[3] = R * (0.25 * a[9]);
                c[4] = R * (0.2 * a[12]), c[5] = R * a[15];
            }
        }
        const double T = 200.0;
        const double *a = t.Hia + n * 21 + (t.nasa ? 0 : 1);  // the range holding 200 K
        out[THERMO_SC_CP200 + n] =
            t.nasa ? R * ((a[0] / T + a[3]) / T + a[6] + (a[9] + (a[12] + (a[15] + a[18] * T) * T) * T) * T)
                   : R * (a[0] + (a[3] + (a[6] + (a[9] + a[12] * T) * T) * T) * T);
    }
}

// Geometry of a block, x fastest.
struct Geo {
    int Xmax, Ymax, Zmax;
    int Xi, Yi, Zi;   // inner sizes
    int Bx, By, Bz;   // ghost widths
    int dimx, dimy, dimz;
    double _dx, _dy, _dz;
    long long pitch;  // elements between components of a SoA array
    double dx, dy, dz;  // cell sizes (the WENO-CU6 epsilon)
    int bc[6];          // boundary kinds (the ghost layers of the viscous derivatives)
    float idh[3], idl[3];  // 1/dx, 1/dy, 1/dz as float pairs, hi + lo (the mixed divergence)
    __host__ __device__ long long ncell() const { return (long long)Xmax * Ymax * Zmax; }
};

// Fills Geo::idh / idl from _dx, _dy, _dz: hi = the nearest float, lo = the nearest float to the
// remainder, so hi + lo carries the inverse spacing to about 2^-48 relative.
inline void geo_split_spacing(Geo &g) {
    const double v[3] = {g._dx, g._dy, g._dz};
    for (int d = 0; d < 3; d++) {
        const bool ok = v[d] == v[d] && v[d] <= 3.0e38 && v[d] >= -3.0e38;   // finite, in float range
        g.idh[d] = ok ? (float)v[d] : 0.f;
        g.idl[d] = ok ? (float)(v[d] - (double)g.idh[d]) : 0.f;
    }
}

// Device arrays of one block. All SoA with the block pitch.
struct DevFields {
    double *U, *U1, *LU;
    double *U2;                // third stage buffer of the fused mixed stage (stage 1 output)
    double *rho, *u, *v, *w, *p, *H, *c, *T, *gamma, *e, *Cp, *R;
    double *y;                 // NS components (COP)
    double *F[3];              // physical fluxes per direction (E components)
    double *Fw[3];             // face fluxes per direction (E components)
    float *Uf, *Ff[3];         // FP32 copies of U and of the physical fluxes (mixed form)
    float *primf;              // FP32 rho, u, v, w, H, p, c (7 components, mixed form)
    float *Fwf[3];             // FP32 face fluxes (mixed form)
    double *sr, *isr;          // sqrt(rho) and 1/sqrt(rho) per cell (single-gas FP64 fast path)
    float *yf, *xcf;           // mixed mixtures: FP32 y (NS) and sound-speed cell terms (3 + NCOP)
    double *eab[3];            // |u_d - c|, |u_d|, |u_d + c| per cell and direction (same path)
    double *vde;               // viscous: the 9 cell-centre velocity derivatives (ducx..dwcz)
    double *mu, *kappa;        // viscous: mixture viscosity and thermal conductivity per cell
    float *vdef, *muf, *kappaf, *Tf;  // viscous, mixed form: FP32 derivatives, mu, kappa and T
    const double *tr;          // viscous: device transport table (see xfg_api.cu, pack_transport)
    const float *trf;          // viscous, mixed form: FP32 transport table (xfg_set_transport)
    double *xc;                // mixtures: per-cell terms of the interface sound speed (3 + NCOP
                               // components, see cop_cell_terms); null = the faces compute them
    unsigned long long *lam;   // dt wave-speed maxima (3 x bit patterns of non-negative doubles)
    double *dtbuf;             // [0] dt of the step, [1] time, [2] target time, [3] steps done
    int *err;                  // error words: [0] state NaN code, [1] primitive error, [2] i, [3] j, [4] k
};

// Roe state of a face: MARCO_ROE (global_marco.h:26-37), c^2 and MARCO_PREEIGEN.
template <class T, int NS>
struct FaceStateT {
    T _u, _v, _w, _H, _P, _rho, D, D1;
    T c2, b1, b3, q2, _c, b2, _c1;
    T ent0;  // (1 - b2 - b3) / b1, column 0 of the entropy row of L
    T z[NS > 1 ? NS - 1 : 1];
    T _yi[NS];
};
template <int NS>
using FaceState = FaceStateT<double, NS>;

// Device code lives in a namespace per translation unit (XFG_KNS) so that the same template
// compiled with different floating-point contraction flags in two units stays two kernels.
namespace XFG_KNS {

// Reciprocal and inverse square root for the single-gas FP64 fast path and the mixed form's
// mixture states and Roe state: the hardware
// approximation refined by two Newton-Raphson steps (r <- r (2 - x r); y <- y (1.5 - x y^2 / 2)),
// within a few ulp of the correctly rounded value for normal finite x.
__device__ __forceinline__ double rcp_nr(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}
// (i, j, k) of the linear index t of an nx x ny x nz box, x fastest: unsigned 32-bit division when
// t fits in 32 bits (the 64-bit division is a long instruction sequence), the 64-bit form otherwise.
__device__ __forceinline__ void split_index(long long t, int nx, int ny, int &i, int &j, int &k) {
    if (t <= 0xffffffffLL) {
        const unsigned u = (unsigned)t, r = u / (unsigned)nx, q = r / (unsigned)ny;
        i = (int)(u - r * (unsigned)nx), j = (int)(r - q * (unsigned)ny), k = (int)q;
    } else {
        const long long r = t / nx;
        i = (int)(t - r * nx), j = (int)(r % ny), k = (int)(r / ny);
    }
}

// One refinement step only: about 2^-40 relative, enough for a Newton step whose iteration
// continues until the step itself is below the tolerance.
__device__ __forceinline__ double rcp_nr1(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return fma(r, fma(-x, r, 1.0), r);
}
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = 0.5 * x;
    double e = fma(-h * y, y, 0.5);
    y = fma(y, e, y);
    e = fma(-h * y, y, 0.5);
    return fma(y, e, y);
}

// ---------------------------------------------------------------------------------------------
// Thermodynamics, src/solver_Ini/Thermo_device.h
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int nasa_range(double T) {
    return (T >= 1000.0 && T < 6000.0) ? 1 : (T < 1000.0 ? 0 : (T >= 6000.0 ? 2 : -1));
}
// HeatCapacity_NASA :10-23 / HeatCapacity_JANAF :29-40
__device__ __forceinline__ double heat_capacity(const DevThermo &t, double T0, int n) {
    const double Ri = t.Ri[n];
    double T = fmax(T0, 200.0);
    if (t.nasa) {
        double _T = 1.0 / T;
        int rg = nasa_range(T);
        if (rg < 0) return 0.0;
        const double *a = t.Hia + n * 21 + rg;
        return Ri * ((a[0] * _T + a[3]) * _T + a[6] + (a[9] + (a[12] + (a[15] + a[18] * T) * T) * T) * T);
    }
    int rg = (T > 1000.0) ? 0 : 1;
    const double *a = t.Hia + n * 21 + rg;
    return Ri * (a[0] + (a[3] + (a[6] + (a[9] + a[12] * T) * T) * T) * T);
}
// get_Enthalpy_NASA :62-80 / get_Enthalpy_JANAF :86-102
__device__ __forceinline__ double enthalpy(const DevThermo &t, double T0, int n) {
    const double Ri = t.Ri[n];
    double TT = T0, T = fmax(T0, 200.0), hi = 0.0;
    if (t.nasa) {
        int rg = nasa_range(T);
        if (rg >= 0) {
            const double *a = t.Hia + n * 21 + rg;
            const double b0 = t.Hib[n * 6 + rg];
            hi = Ri * (-a[0] / T + a[3] * log(T) +
                       (a[6] + (0.5 * a[9] + (a[12] * kOT + (0.25 * a[15] + 0.2 * a[18] * T) * T) * T) * T) * T + b0);
        }
    } else {
        int rg = (T > 1000.0) ? 0 : 1;
        const double *a = t.Hia + n * 21 + rg;
        hi = Ri * (T * (a[0] + T * (a[3] * 0.5 + T * (a[6] * kOT + T * (a[9] * 0.25 + a[12] * T * 0.2)))) + a[15]);
    }
    if (TT < 200.0) hi += heat_capacity(t, 200.0, n) * (TT - 200.0);
    return hi;
}

// Mixture functions, src/solver_Ini/Mixing_device.h
template <int NS>
__device__ __forceinline__ double mix_R(const DevThermo &t, const double *yi) {  // get_CopR :49-56
    double s = 0.0;
#pragma unroll
    for (int n = 0; n < NS; n++) s += yi[n] * t._Wi[n];
    return s * kRu;
}
template <int NS>
__device__ __forceinline__ double mix_W_inv(const DevThermo &t, const double *yi) {
    double s = 0.0;
#pragma unroll
    for (int n = 0; n < NS; n++) s += yi[n] * t._Wi[n];
    return s;
}
template <int NS>
__device__ __forceinline__ double mix_Cp(const DevThermo &t, const double *yi, double T) {  // get_CopCp :61-68
    double s = 0.0;
#pragma unroll
    for (int n = 0; n < NS; n++) s += yi[n] * heat_capacity(t, T, n);
    return s;
}
template <int NS>
__device__ __forceinline__ double mix_h(const DevThermo &t, const double *yi, double T) {  // get_Coph :131-140
    double h = 0.0;
#pragma unroll
    for (int n = 0; n < NS; n++) h += enthalpy(t, T, n) * yi[n];
    return h;
}
// get_T :171-193 (Newton on h(T) - R T - e, clamped steps, <= 100 iterations, |dT| <= 1e-6 K)
template <int NS>
__device__ double newton_T(const DevThermo &t, const double *yi, double e, double T0) {
    double T = T0;
    const double Rm = mix_R<NS>(t, yi);
    for (int it = 1; it < 101; it++) {
        double h = 0.0, Cp = 0.0;
#pragma unroll
        for (int n = 0; n < NS; n++) {
            h += enthalpy(t, T, n) * yi[n];
            Cp += yi[n] * heat_capacity(t, T, n);
        }
        double f = h - Rm * T - e;
        double df_ = Cp - Rm;
        double df = fmin(f / (df_ + 1.0e-30), 1e-3 * T);
        df = fmax(df, -1e-2 * T);
        T = T - df;
        if (fabs(df) <= 1.0e-6) break;
    }
    return T;
}

// ---------------------------------------------------------------------------------------------
// Eigensystem entries (Eigen_matrix.hpp OROC form). Kinds: 0 structural zero, 1 +1, 2 -1,
// 3 general. They depend only on (direction, E, row/column, component) and fold at compile time.
// ---------------------------------------------------------------------------------------------
__host__ __device__ constexpr int left_kind(int D, int E, int n, int k) {
    if (n == 0 || n == E - 1) return 3;
    if (n >= 1 && n <= 3) {
        if (n == D + 1) return k == 4 ? 2 : 3;
        // shear rows: x: n=2 (v,0,-1,0,0), n=3 (-w,0,0,1,0); y: n=1 (-u,1,..), n=3 (w,0,0,-1,0);
        // z: n=1 (u,-1,0,0,0), n=2 (-v,0,1,0,0)
        if (k == 0) return 3;
        if (D == 0) return (n == 2) ? (k == 2 ? 2 : 0) : (k == 3 ? 1 : 0);
        if (D == 1) return (n == 1) ? (k == 1 ? 1 : 0) : (k == 3 ? 2 : 0);
        return (n == 1) ? (k == 1 ? 2 : 0) : (k == 2 ? 1 : 0);
    }
    // species rows n = 4..E-2: (-y_s, 0, 0, 0, 0, delta_{s})
    if (k == 0) return 3;
    return (k == 5 + (n - 4)) ? 1 : 0;
}
__host__ __device__ constexpr int right_kind(int D, int E, int n, int k) {
    if (n == 0 || n == E - 1) return k == 0 ? 1 : 3;
    if (n >= 1 && n <= 3) {
        if (n == D + 1) return 3;
        if (k == 4) return 3;
        if (D == 0) return (n == 2) ? (k == 2 ? 2 : 0) : (k == 3 ? 1 : 0);
        if (D == 1) return (n == 1) ? (k == 1 ? 1 : 0) : (k == 3 ? 2 : 0);
        return (n == 1) ? (k == 1 ? 2 : 0) : (k == 2 ? 1 : 0);
    }
    if (k == 4) return 3;
    return (k == 5 + (n - 4)) ? 1 : 0;
}

// General entry (kind 3) of row n of L for direction D, component k (RoeAverageLeft_*).
template <int D, int E, class T, int NS>
__device__ __forceinline__ T left_val(const FaceStateT<T, NS> &F, int n, int k) {
    const T b1 = F.b1, b2 = F.b2, b3 = F.b3, _c1 = F._c1;
    const T vel[3] = {F._u, F._v, F._w};
    const T un = vel[D];
    const T h = T(0.5);
    if (n == 0) {
        if (k == 0) return h * (b2 + un * _c1 + b3);
        if (k >= 1 && k <= 3) return (k - 1 == D) ? -h * (b1 * vel[k - 1] + _c1) : -h * (b1 * vel[k - 1]);
        if (k == 4) return h * b1;
        return -h * b1 * F.z[k - 5];
    }
    if (n == E - 1) {
        if (k == 0) return h * (b2 - un * _c1 + b3);
        if (k >= 1 && k <= 3) return (k - 1 == D) ? h * (-b1 * vel[k - 1] + _c1) : h * (-b1 * vel[k - 1]);
        if (k == 4) return h * b1;
        return -h * b1 * F.z[k - 5];
    }
    if (n >= 1 && n <= 3) {
        if (n == D + 1) {
            if (k == 0) return F.ent0;
            if (k >= 1 && k <= 3) return vel[k - 1];
            return F.z[k - 5];
        }
        // column 0 of the shear rows
        if (D == 0) return n == 2 ? F._v : -F._w;
        if (D == 1) return n == 1 ? -F._u : F._w;
        return n == 1 ? F._u : -F._v;
    }
    return -F._yi[n - 4];
}

// General entry (kind 3) of column n of R for direction D, component k (RoeAverageRight_*).
template <int D, int E, class T, int NS>
__device__ __forceinline__ T right_val(const FaceStateT<T, NS> &F, int n, int k) {
    const T vel[3] = {F._u, F._v, F._w};
    const T un = vel[D], _c = F._c, _H = F._H, b1 = F.b1;
    if (n == 0 || n == E - 1) {
        const bool m = n == 0;
        if (k >= 1 && k <= 3) return (k - 1 == D) ? (m ? vel[k - 1] - _c : vel[k - 1] + _c) : vel[k - 1];
        if (k == 4) return m ? _H - un * _c : _H + un * _c;
        return F._yi[k - 5];
    }
    if (n >= 1 && n <= 3) {
        if (n == D + 1) {
            if (k == 0) return b1;
            if (k >= 1 && k <= 3) return vel[k - 1] * b1;
            if (k == 4) return _H * b1 - T(1.0);
            return b1 * F._yi[k - 5];
        }
        if (D == 0) return n == 2 ? -F._v : F._w;
        if (D == 1) return n == 1 ? F._u : -F._w;
        return n == 1 ? -F._u : F._v;
    }
    return F.z[n - 4];
}

// ---------------------------------------------------------------------------------------------
// WENO schemes
// ---------------------------------------------------------------------------------------------
// weno5old_BODY, WENO5s_schemes.hpp:12-69 (double branch; product-form weights)
__device__ __forceinline__ double weno5_body(double v1, double v2, double v3, double v4, double v5) {
    double a1, a2, a3;
    a1 = v1 - 2.0 * v2 + v3;
    double s1 = 13.0 * a1 * a1;
    a1 = v1 - 4.0 * v2 + 3.0 * v3;
    s1 += 3.0 * a1 * a1;
    a1 = v2 - 2.0 * v3 + v4;
    double s2 = 13.0 * a1 * a1;
    a1 = v2 - v4;
    s2 += 3.0 * a1 * a1;
    a1 = v3 - 2.0 * v4 + v5;
    double s3 = 13.0 * a1 * a1;
    a1 = 3.0 * v3 - 4.0 * v4 + v5;
    s3 += 3.0 * a1 * a1;
    s1 += 1.0E-6, s2 += 1.0E-6, s3 += 1.0E-6;
    a1 = 0.1 * s2 * s2 * s3 * s3;
    a2 = 0.6 * s1 * s1 * s3 * s3;
    a3 = 0.3 * s1 * s1 * s2 * s2;
    double tw1 = 1.0 / (a1 + a2 + a3);
    a1 = a1 * tw1, a2 = a2 * tw1, a3 = a3 * tw1;
    s1 = a1 * (2.0 * v1 - 7.0 * v2 + 11.0 * v3);
    s2 = a2 * (-v2 + 5.0 * v3 + 2.0 * v4);
    s3 = a3 * (2.0 * v3 + 5.0 * v4 - v5);
    return (s1 + s2 + s3);
}
// FP64 fast form of the body: the same smoothness indicators, weights and candidates arranged for
// fused multiply-adds. The indicators are carried as s_k / 13 (13 a^2 + 3 b^2 + eps, all over 13):
// the weights are homogeneous of degree zero in the s_k, so the factor cancels. The linear
// weights d_k and the 1/6 of the candidates are folded into the candidate coefficients. Returns
// the weighted candidate sum and the weight sum separately (the caller normalises both sides of a
// face with one reciprocal).
constexpr double kW313 = 3.0 / 13.0, kWeps13 = 1.0e-6 / 13.0;
constexpr double kQ1a = 0.1 * 2.0 / 6.0, kQ1b = 0.1 * -7.0 / 6.0, kQ1c = 0.1 * 11.0 / 6.0;
constexpr double kQ2a = -0.1, kQ2b = 0.5, kQ2c = 0.2;         // 0.6 / 6 * (-1, 5, 2)
constexpr double kQ3a = 0.1, kQ3b = 0.25, kQ3c = -0.05;       // 0.3 / 6 * (2, 5, -1)
__device__ __forceinline__ void weno5_body_nd(double v1, double v2, double v3, double v4, double v5, double &num,
                                              double &den) {
    double a = fma(-2.0, v2, v1) + v3;
    double b = fma(3.0, v3, fma(-4.0, v2, v1));
    const double s1 = fma(a, a, fma(kW313 * b, b, kWeps13));
    a = fma(-2.0, v3, v2) + v4;
    b = v2 - v4;
    const double s2 = fma(a, a, fma(kW313 * b, b, kWeps13));
    a = fma(-2.0, v4, v3) + v5;
    b = fma(3.0, v3, fma(-4.0, v4, v5));
    const double s3 = fma(a, a, fma(kW313 * b, b, kWeps13));
    const double p23 = s2 * s3, p13 = s1 * s3, p12 = s1 * s2;
    const double P1 = p23 * p23, P2 = p13 * p13, P3 = p12 * p12;
    const double q1 = fma(kQ1c, v3, fma(kQ1b, v2, kQ1a * v1));
    const double q2 = fma(kQ2c, v4, fma(kQ2b, v3, kQ2a * v2));
    const double q3 = fma(kQ3c, v5, fma(kQ3b, v4, kQ3a * v3));
    num = fma(P3, q3, fma(P2, q2, P1 * q1));
    den = fma(0.3, P3, fma(0.6, P2, 0.1 * P1));
}
// nf / df + nm / dm with one reciprocal: for indicators s_k between 1e-6 and 1e17 each weight sum
// lies in [1e-30, 1e64] and their product in [1e-60, 1e128], far from overflow and subnormals
__device__ __forceinline__ double weno5_fast(const double *pp, const double *mm) {
    double nf, df, nm, dm;
    weno5_body_nd(pp[1], pp[2], pp[3], pp[4], pp[5], nf, df);
    weno5_body_nd(mm[6], mm[5], mm[4], mm[3], mm[2], nm, dm);
    return fma(nf, dm, nm * df) * rcp_nr(df * dm);
}

// Form of the body for doubled inputs v' = 2 v (the split fluxes f +- a u without the factor 1/2)
// written around the centre value: each candidate is q_k / 6 = v3 + r_k with
// r_1 = a_1/12 + b_1/4, r_2 = a_2/12 - b_2/4, r_3 = a_3/12 - b_3/4 (a_k, b_k the differences of the
// smoothness indicators), so that with weights summing to one WENO(v) = v3 + sum w_k r_k. Doubling
// the input multiplies the indicators by 4: with eps scaled by 4 the weights are unchanged and
// WENO(v) = WENO'(v') / 2; the 1/2 and the linear weights d_k are folded into the r coefficients.
constexpr double kWeps13x4 = 4.0 * kWeps13;
constexpr double kRa1 = 0.5 * 0.1 / 12.0, kRb1 = 0.5 * 0.1 / 4.0;
constexpr double kRa2 = 0.5 * 0.6 / 12.0, kRb2 = -0.5 * 0.6 / 4.0;
constexpr double kRa3 = 0.5 * 0.3 / 12.0, kRb3 = -0.5 * 0.3 / 4.0;
__device__ __forceinline__ void weno5_body_r(double v1, double v2, double v3, double v4, double v5, double &num,
                                             double &den) {
    const double a1 = fma(-2.0, v2, v1) + v3;
    const double b1 = fma(3.0, v3, fma(-4.0, v2, v1));
    const double s1 = fma(a1, a1, fma(kW313 * b1, b1, kWeps13x4));
    const double a2 = fma(-2.0, v3, v2) + v4;
    const double b2 = v2 - v4;
    const double s2 = fma(a2, a2, fma(kW313 * b2, b2, kWeps13x4));
    const double a3 = fma(-2.0, v4, v3) + v5;
    const double b3 = fma(3.0, v3, fma(-4.0, v4, v5));
    const double s3 = fma(a3, a3, fma(kW313 * b3, b3, kWeps13x4));
    const double p23 = s2 * s3, p13 = s1 * s3, p12 = s1 * s2;
    const double P1 = p23 * p23, P2 = p13 * p13, P3 = p12 * p12;
    const double r1 = fma(kRa1, a1, kRb1 * b1);
    const double r2 = fma(kRa2, a2, kRb2 * b2);
    const double r3 = fma(kRa3, a3, kRb3 * b3);
    num = fma(P3, r3, fma(P2, r2, P1 * r1));
    den = fma(0.3, P3, fma(0.6, P2, 0.1 * P1));
}
// WENO5 face flux (both sides) from the doubled split fluxes pp2 = f + a u, mm2 = f - a u
// (indices m + 3 for stencil offsets m = -2..3), one reciprocal for both sides
__device__ __forceinline__ double weno5_fast2(const double *pp2, const double *mm2) {
    double nf, df, nm, dm;
    weno5_body_r(pp2[1], pp2[2], pp2[3], pp2[4], pp2[5], nf, df);
    weno5_body_r(mm2[6], mm2[5], mm2[4], mm2[3], mm2[2], nm, dm);
    return fma(0.5, pp2[3] + mm2[4], fma(nf, dm, nm * df) * rcp_nr(df * dm));
}

// WENOCU6_BODYGPU / WENOCU6_GPU (WENO6s_schemes.hpp:5-84): the WENO5 indicators, the sixth-order
// indicator s6 of the tau_6k differences, the CU6 weights 20 + |s6 - s55| / (s_k + eps) with linear
// weights (0.05, 0.45, 0.45, 0.05), eps = 1e-8 dl^2; the reference's operation order.
template <class T>
__device__ __forceinline__ T wenocu6_body(T v1, T v2, T v3, T v4, T v5, T v6, T eps) {
    T s11 = v1 - T(2.0) * v2 + v3;
    T s12 = v1 - T(4.0) * v2 + T(3.0) * v3;
    T s1 = T(13.0) * s11 * s11 + T(3.0) * s12 * s12;
    T s21 = v2 - T(2.0) * v3 + v4;
    T s22 = v2 - v4;
    T s2 = T(13.0) * s21 * s21 + T(3.0) * s22 * s22;
    T s31 = v3 - T(2.0) * v4 + v5;
    T s32 = T(3.0) * v3 - T(4.0) * v4 + v5;
    T s3 = T(13.0) * s31 * s31 + T(3.0) * s32 * s32;
    T tau61 = (T(259.0) * v6 - T(1895.0) * v5 + T(6670.0) * v4 - T(2590.0) * v3 - T(2785.0) * v2 + T(341.0) * v1) *
              T(1.0 / 5760.0);
    T tau62 = -(v5 - T(12.0) * v4 + T(22.0) * v3 - T(12.0) * v2 + v1) * T(1.0 / 16.0);
    T tau63 = -(T(7.0) * v6 - T(47.0) * v5 + T(94.0) * v4 - T(70.0) * v3 + T(11.0) * v2 + T(5.0) * v1) * T(1.0 / 144.0);
    T tau64 = (v5 - T(4.0) * v4 + T(6.0) * v3 - T(4.0) * v2 + v1) * T(1.0 / 24.0);
    T tau65 = -(-v6 + T(5.0) * v5 - T(10.0) * v4 + T(10.0) * v3 - T(5.0) * v2 + v1) * T(1.0 / 120.0);
    const T a1a1 = T(1.0), a2a2 = T(13.0 / 3.0), a1a3 = T(0.5), a3a3 = T(3129.0 / 80.0), a2a4 = T(4.2);
    const T a1a5 = T(0.125), a4a4 = T(87617.0 / 140.0), a3a5 = T(14127.0 / 224.0), a5a5 = T(252337135.0 / 16128.0);
    T s6 = (tau61 * tau61 * a1a1 + tau62 * tau62 * a2a2 + tau61 * tau63 * a1a3 + tau63 * tau63 * a3a3 +
            tau62 * tau64 * a2a4 + tau61 * tau65 * a1a5 + tau64 * tau64 * a4a4 + tau63 * tau65 * a3a5 +
            tau65 * tau65 * a5a5) * T(12.0);
    T s55 = (s1 + s3 + T(4.0) * s2) * T(kSix);
    T s5 = fabs(s6 - s55);
    T r0 = T(20.0);
    T r1 = r0 + s5 / (s1 + eps);
    T r2 = r0 + s5 / (s2 + eps);
    T r3 = r0 + s5 / (s3 + eps);
    T r4 = r0 + s5 / (s6 + eps);
    T a1 = T(0.05) * r1, a2 = T(0.45) * r2, a3 = T(0.45) * r3, a4 = T(0.05) * r4;
    T tw1 = T(1.0) / (a1 + a2 + a3 + a4);
    T w1 = a1 * tw1, w2 = a2 * tw1, w3 = a3 * tw1, w4 = a4 * tw1;
    T temp = T(0.0);
    temp += w1 * (T(2.0) * v1 - T(7.0) * v2 + T(11.0) * v3);
    temp += w2 * (-v2 + T(5.0) * v3 + T(2.0) * v4);
    temp += w3 * (T(2.0) * v3 + T(5.0) * v4 - v5);
    temp += w4 * (T(11.0) * v4 - T(7.0) * v5 + T(2.0) * v6);
    return temp;
}
// pp, mm indexed by stencil offset m + 3, m = -2..3 used
template <class T>
__device__ __forceinline__ T wenocu6(const T *pp, const T *mm, T dl) {
    const T eps = T(1.e-8) * dl * dl;
    T temf = wenocu6_body(pp[1], pp[2], pp[3], pp[4], pp[5], pp[6], eps);
    T temm = wenocu6_body(mm[6], mm[5], mm[4], mm[3], mm[2], mm[1], eps);
    return (temf + temm) * T(kSix);
}

// Hardware FP32 reciprocal approximation (rcp.approx.ftz.f32, about 1 ulp) for the nonlinear
// weights of the FP32 WENO forms, where it replaces IEEE divisions.
__device__ __forceinline__ float rcp_approx_f(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// FP32 form: the same candidates and smoothness indicators; the weights use the division form
// d_k / s_k^2 (equal to the product form) so that s^4 cannot overflow single precision, scaled by
// the smallest s: d_k (s_min / s_k)^2 lies in [0, d_k] whatever the scale of the data, and the
// reciprocals are the hardware approximation.
__device__ __forceinline__ float weno5_body(float v1, float v2, float v3, float v4, float v5) {
    float a1;
    a1 = v1 - 2.0f * v2 + v3;
    float s1 = 13.0f * a1 * a1;
    a1 = v1 - 4.0f * v2 + 3.0f * v3;
    s1 += 3.0f * a1 * a1;
    a1 = v2 - 2.0f * v3 + v4;
    float s2 = 13.0f * a1 * a1;
    a1 = v2 - v4;
    s2 += 3.0f * a1 * a1;
    a1 = v3 - 2.0f * v4 + v5;
    float s3 = 13.0f * a1 * a1;
    a1 = 3.0f * v3 - 4.0f * v4 + v5;
    s3 += 3.0f * a1 * a1;
    s1 += 1.0E-6f, s2 += 1.0E-6f, s3 += 1.0E-6f;
    const float sm = fminf(s1, fminf(s2, s3));
    const float r1 = sm * rcp_approx_f(s1), r2 = sm * rcp_approx_f(s2), r3 = sm * rcp_approx_f(s3);
    const float w1 = 0.1f * r1 * r1, w2 = 0.6f * r2 * r2, w3 = 0.3f * r3 * r3;
    const float tw = rcp_approx_f(w1 + w2 + w3);
    return tw * (w1 * (2.0f * v1 - 7.0f * v2 + 11.0f * v3) + w2 * (-v2 + 5.0f * v3 + 2.0f * v4) +
                 w3 * (2.0f * v3 + 5.0f * v4 - v5));
}
// weno5old_GPU :71-95 on 8-point stencil arrays indexed m+3
template <class T>
__device__ __forceinline__ T weno5(const T *pp, const T *mm) {
    T temf = weno5_body(pp[1], pp[2], pp[3], pp[4], pp[5]);
    T temm = weno5_body(mm[6], mm[5], mm[4], mm[3], mm[2]);
    return (temf + temm) * T(kSix);
}
// weno7_P / weno7_M body, WENO7s_schemes.hpp:8-128
template <class T>
__device__ __forceinline__ T weno7_body(T v1, T v2, T v3, T v4, T v5, T v6, T v7) {
    const T ep = T(1.0e-7);
    const T C0 = T(1.0 / 35.0), C1 = T(12.0 / 35.0), C2 = T(18.0 / 35.0), C3 = T(4.0 / 35.0);
    T S10 = T(-2.0 / 6.0) * v1 + T(9.0 / 6.0) * v2 - T(18.0 / 6.0) * v3 + T(11.0 / 6.0) * v4;
    T S11 = T(1.0 / 6.0) * v2 - v3 + T(3.0 / 6.0) * v4 + T(2.0 / 6.0) * v5;
    T S12 = T(-2.0 / 6.0) * v3 - T(3.0 / 6.0) * v4 + v5 - T(1.0 / 6.0) * v6;
    T S13 = T(-11.0 / 6.0) * v4 + T(18.0 / 6.0) * v5 - T(9.0 / 6.0) * v6 + T(2.0 / 6.0) * v7;
    T S20 = -v1 + T(4.0) * v2 - T(5.0) * v3 + T(2.0) * v4;
    T S21 = v3 - T(2.0) * v4 + v5;
    T S22 = v4 - T(2.0) * v5 + v6;
    T S23 = T(2.0) * v4 - T(5.0) * v5 + T(4.0) * v6 - v7;
    T S30 = -v1 + T(3.0) * v2 - T(3.0) * v3 + v4;
    T S31 = -v2 + T(3.0) * v3 - T(3.0) * v4 + v5;
    T S32 = -v3 + T(3.0) * v4 - T(3.0) * v5 + v6;
    T S33 = -v4 + T(3.0) * v5 - T(3.0) * v6 + v7;
    const T k13 = T(13.0 / 12.0), k1043 = T(1043.0 / 960.0), k112 = T(1.0 / 12.0);
    T S0 = S10 * S10 + k13 * S20 * S20 + k1043 * S30 * S30 + k112 * S10 * S30;
    T S1 = S11 * S11 + k13 * S21 * S21 + k1043 * S31 * S31 + k112 * S11 * S31;
    T S2 = S12 * S12 + k13 * S22 * S22 + k1043 * S32 * S32 + k112 * S12 * S32;
    T S3 = S13 * S13 + k13 * S23 * S23 + k1043 * S33 * S33 + k112 * S13 * S33;
    T a0 = C0 / ((ep + S0) * (ep + S0));
    T a1 = C1 / ((ep + S1) * (ep + S1));
    T a2 = C2 / ((ep + S2) * (ep + S2));
    T a3 = C3 / ((ep + S3) * (ep + S3));
    T sum = a0 + a1 + a2 + a3;
    T W0 = a0 / sum, W1 = a1 / sum, W2 = a2 / sum, W3 = a3 / sum;
    T q0 = T(-3.0 / 12.0) * v1 + T(13.0 / 12.0) * v2 - T(23.0 / 12.0) * v3 + T(25.0 / 12.0) * v4;
    T q1 = T(1.0 / 12.0) * v2 - T(5.0 / 12.0) * v3 + T(13.0 / 12.0) * v4 + T(3.0 / 12.0) * v5;
    T q2 = T(-1.0 / 12.0) * v3 + T(7.0 / 12.0) * v4 + T(7.0 / 12.0) * v5 - T(1.0 / 12.0) * v6;
    T q3 = T(3.0 / 12.0) * v4 + T(13.0 / 12.0) * v5 - T(5.0 / 12.0) * v6 + T(1.0 / 12.0) * v7;
    return W0 * q0 + W1 * q1 + W2 * q2 + W3 * q3;
}
// FP32 form of weno7_body: the same indicators and candidates; the weights C_k / (eps + S_k)^2
// scaled by the smallest (eps + S_k), as in the FP32 WENO5, with hardware reciprocals.
__device__ __forceinline__ float weno7_body_f(float v1, float v2, float v3, float v4, float v5, float v6, float v7) {
    const float ep = 1.0e-7f;
    const float S10 = (-2.0f / 6.0f) * v1 + (9.0f / 6.0f) * v2 - (18.0f / 6.0f) * v3 + (11.0f / 6.0f) * v4;
    const float S11 = (1.0f / 6.0f) * v2 - v3 + (3.0f / 6.0f) * v4 + (2.0f / 6.0f) * v5;
    const float S12 = (-2.0f / 6.0f) * v3 - (3.0f / 6.0f) * v4 + v5 - (1.0f / 6.0f) * v6;
    const float S13 = (-11.0f / 6.0f) * v4 + (18.0f / 6.0f) * v5 - (9.0f / 6.0f) * v6 + (2.0f / 6.0f) * v7;
    const float S20 = -v1 + 4.0f * v2 - 5.0f * v3 + 2.0f * v4;
    const float S21 = v3 - 2.0f * v4 + v5;
    const float S22 = v4 - 2.0f * v5 + v6;
    const float S23 = 2.0f * v4 - 5.0f * v5 + 4.0f * v6 - v7;
    const float S30 = -v1 + 3.0f * v2 - 3.0f * v3 + v4;
    const float S31 = -v2 + 3.0f * v3 - 3.0f * v4 + v5;
    const float S32 = -v3 + 3.0f * v4 - 3.0f * v5 + v6;
    const float S33 = -v4 + 3.0f * v5 - 3.0f * v6 + v7;
    const float k13 = 13.0f / 12.0f, k1043 = 1043.0f / 960.0f, k112 = 1.0f / 12.0f;
    const float e0 = ep + (S10 * S10 + k13 * S20 * S20 + k1043 * S30 * S30 + k112 * S10 * S30);
    const float e1 = ep + (S11 * S11 + k13 * S21 * S21 + k1043 * S31 * S31 + k112 * S11 * S31);
    const float e2 = ep + (S12 * S12 + k13 * S22 * S22 + k1043 * S32 * S32 + k112 * S12 * S32);
    const float e3 = ep + (S13 * S13 + k13 * S23 * S23 + k1043 * S33 * S33 + k112 * S13 * S33);
    const float em = fminf(fminf(e0, e1), fminf(e2, e3));
    const float r0 = em * rcp_approx_f(e0), r1 = em * rcp_approx_f(e1);
    const float r2 = em * rcp_approx_f(e2), r3 = em * rcp_approx_f(e3);
    const float a0 = (1.0f / 35.0f) * r0 * r0, a1 = (12.0f / 35.0f) * r1 * r1;
    const float a2 = (18.0f / 35.0f) * r2 * r2, a3 = (4.0f / 35.0f) * r3 * r3;
    const float isum = 1.0f / (a0 + a1 + a2 + a3);
    const float q0 = (-3.0f / 12.0f) * v1 + (13.0f / 12.0f) * v2 - (23.0f / 12.0f) * v3 + (25.0f / 12.0f) * v4;
    const float q1 = (1.0f / 12.0f) * v2 - (5.0f / 12.0f) * v3 + (13.0f / 12.0f) * v4 + (3.0f / 12.0f) * v5;
    const float q2 = (-1.0f / 12.0f) * v3 + (7.0f / 12.0f) * v4 + (7.0f / 12.0f) * v5 - (1.0f / 12.0f) * v6;
    const float q3 = (3.0f / 12.0f) * v4 + (13.0f / 12.0f) * v5 - (5.0f / 12.0f) * v6 + (1.0f / 12.0f) * v7;
    return (a0 * q0 + a1 * q1 + a2 * q2 + a3 * q3) * isum;
}
template <class T>
__device__ __forceinline__ T weno7(const T *pp, const T *mm) {
    if constexpr (sizeof(T) == 4)
        return weno7_body_f(pp[0], pp[1], pp[2], pp[3], pp[4], pp[5], pp[6]) +
               weno7_body_f(mm[7], mm[6], mm[5], mm[4], mm[3], mm[2], mm[1]);
    T tp = weno7_body(pp[0], pp[1], pp[2], pp[3], pp[4], pp[5], pp[6]);
    T tm = weno7_body(mm[7], mm[6], mm[5], mm[4], mm[3], mm[2], mm[1]);
    return tp + tm;
}

// WENO7 of the contracted FP64 forms: the same indicators, candidates and weights, the weights in
// the product form W_k = C_k prod_{j != k} (eps + S_j)^2 / sum (one division instead of eight; the
// products stay far inside the FP64 range: (eps + S)^2 is at least 1e-14, three of them of large
// indicators ~1e144 at the steepest jumps met here). Not for FP32, where they would overflow.
__device__ __forceinline__ double weno7_prod_body(double v1, double v2, double v3, double v4, double v5, double v6,
                                                  double v7) {
    const double ep = 1.0e-7;
    const double C0 = 1.0 / 35.0, C1 = 12.0 / 35.0, C2 = 18.0 / 35.0, C3 = 4.0 / 35.0;
    const double S10 = (-2.0 / 6.0) * v1 + (9.0 / 6.0) * v2 - (18.0 / 6.0) * v3 + (11.0 / 6.0) * v4;
    const double S11 = (1.0 / 6.0) * v2 - v3 + (3.0 / 6.0) * v4 + (2.0 / 6.0) * v5;
    const double S12 = (-2.0 / 6.0) * v3 - (3.0 / 6.0) * v4 + v5 - (1.0 / 6.0) * v6;
    const double S13 = (-11.0 / 6.0) * v4 + (18.0 / 6.0) * v5 - (9.0 / 6.0) * v6 + (2.0 / 6.0) * v7;
    const double S20 = -v1 + 4.0 * v2 - 5.0 * v3 + 2.0 * v4;
    const double S21 = v3 - 2.0 * v4 + v5;
    const double S22 = v4 - 2.0 * v5 + v6;
    const double S23 = 2.0 * v4 - 5.0 * v5 + 4.0 * v6 - v7;
    const double S30 = -v1 + 3.0 * v2 - 3.0 * v3 + v4;
    const double S31 = -v2 + 3.0 * v3 - 3.0 * v4 + v5;
    const double S32 = -v3 + 3.0 * v4 - 3.0 * v5 + v6;
    const double S33 = -v4 + 3.0 * v5 - 3.0 * v6 + v7;
    const double k13 = 13.0 / 12.0, k1043 = 1043.0 / 960.0, k112 = 1.0 / 12.0;
    const double S0 = S10 * S10 + k13 * S20 * S20 + k1043 * S30 * S30 + k112 * S10 * S30;
    const double S1 = S11 * S11 + k13 * S21 * S21 + k1043 * S31 * S31 + k112 * S11 * S31;
    const double S2 = S12 * S12 + k13 * S22 * S22 + k1043 * S32 * S32 + k112 * S12 * S32;
    const double S3 = S13 * S13 + k13 * S23 * S23 + k1043 * S33 * S33 + k112 * S13 * S33;
    const double d0 = (ep + S0) * (ep + S0), d1 = (ep + S1) * (ep + S1);
    const double d2 = (ep + S2) * (ep + S2), d3 = (ep + S3) * (ep + S3);
    const double d01 = d0 * d1, d23 = d2 * d3;
    const double p0 = C0 * d1 * d23, p1 = C1 * d0 * d23, p2 = C2 * d01 * d3, p3 = C3 * d01 * d2;
    const double q0 = (-3.0 / 12.0) * v1 + (13.0 / 12.0) * v2 - (23.0 / 12.0) * v3 + (25.0 / 12.0) * v4;
    const double q1 = (1.0 / 12.0) * v2 - (5.0 / 12.0) * v3 + (13.0 / 12.0) * v4 + (3.0 / 12.0) * v5;
    const double q2 = (-1.0 / 12.0) * v3 + (7.0 / 12.0) * v4 + (7.0 / 12.0) * v5 - (1.0 / 12.0) * v6;
    const double q3 = (3.0 / 12.0) * v4 + (13.0 / 12.0) * v5 - (5.0 / 12.0) * v6 + (1.0 / 12.0) * v7;
    return (p0 * q0 + p1 * q1 + p2 * q2 + p3 * q3) / (p0 + p1 + p2 + p3);
}
__device__ __forceinline__ double weno7_prod(const double *pp, const double *mm) {
    return weno7_prod_body(pp[0], pp[1], pp[2], pp[3], pp[4], pp[5], pp[6]) +
           weno7_prod_body(mm[7], mm[6], mm[5], mm[4], mm[3], mm[2], mm[1]);
}

// atomic max of a non-negative double through its bit pattern (monotone for x >= 0)
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v) {
    if (!(v >= 0.0)) v = __longlong_as_double(0x7ff0000000000000LL);  // NaN -> +inf (flags the step)
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

}  // namespace XFG_KNS
}  // namespace xfg
