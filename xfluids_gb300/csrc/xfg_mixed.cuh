// xfg_mixed.cuh - mixed-precision form of the stage kernels.
//
// The conserved state U and the RK stage combination stay FP64; the characteristic projection,
// the flux splitting, the WENO smoothness indicators and weights run in FP32 on FP32 copies of
// U, of the physical fluxes and of the face primitives written by k_states_mixed. The FP32 right-
// hand side is accumulated into the FP64 state by the RK stage. The multi-component temperature
// Newton iteration stays FP64, and so do the jumps across a face from which the multi-component
// Roe sound speed's near-degenerate correction is formed (face_state_mixed); the rest of the
// mixture Roe state is FP32.
#pragma once

#include "xfg_kernels.cuh"

namespace xfg {
namespace XFG_KNS {

// FP64 -> FP32 rounded to nearest even by integer operations (the conversion instruction runs on
// the FP64 pipe, the mixture path's bottleneck): exact for results in the FP32 normal range;
// magnitudes below 2^-126 give a signed zero, 2^128 and above an infinity, NaN a NaN.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned e = (hi >> 20) & 0x7ffu, sgn = hi & 0x80000000u, mh = hi & 0xfffffu;
    unsigned fb = ((e - 896u) << 23) + ((mh << 3) | (lo >> 29));  // exponent rebiased, top 23 bits
    const unsigned rem = lo & 0x1fffffffu;                         // the 29 bits dropped
    fb += (rem > 0x10000000u || (rem == 0x10000000u && (fb & 1u))) ? 1u : 0u;  // a carry is the next binade
    fb = e < 897u ? 0u : fb;
    fb = e > 1150u ? ((e == 0x7ffu && (mh | lo)) ? 0x7fc00000u : 0x7f800000u) : fb;
    return __uint_as_float(sgn | fb);
}

// Mixture thermodynamics of the mixed form with the species folded into one polynomial.
// h(T) = sum_n y_n h_n(T) and Cp(T) = sum_n y_n Cp_n(T) are linear in the species, and the
// temperature ranges of both tables do not depend on the species (JANAF breaks at 1000 K, NASA-9
// at 1000 / 6000 K), so within a range the mixture enthalpy has the coefficients
// H_c = sum_n y_n c_{n,c} of the R_n-scaled species tables (DevThermo::hsc) and Cp = dh/dT those
// times their powers; folded once per cell and range: each Newton iteration is one polynomial (and
// one log for NASA-9) instead of NS. Below 200 K (the tables' linear extrapolation) the
// per-species functions are used. Same mathematics as the reference's sums, different rounding:
// the mixed form only.
__device__ __forceinline__ int thermo_range(bool nasa, double T) { return nasa ? nasa_range(T) : (T > 1000.0 ? 0 : 1); }

template <int NS>
struct FoldedThermo {
    double H[8], A[7];  // enthalpy coefficients (layout of DevThermo::hsc); Cp coefficients
    int rg = -9;
    __device__ __forceinline__ bool fold(const DevThermo &t, const double *yi, double T) {
        const int r = thermo_range(t.nasa, T);
        if (r < 0) return false;
        if (r == rg) return true;
        rg = r;
        const int nc = t.nasa ? 8 : 6;
#pragma unroll
        for (int c = 0; c < 8; c++) H[c] = 0.0;
#pragma unroll
        for (int n = 0; n < NS; n++) {
            const double *c = t.hsc + (n * 3 + r) * 8;
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (q < nc) H[q] = fma(yi[n], c[q], H[q]);
        }
        if (t.nasa) {  // Cp = -H0 / T^2 + H1 / T + H2 + 2 H3 T + 3 H4 T^2 + 4 H5 T^3 + 5 H6 T^4
            A[0] = -H[0], A[1] = H[1], A[2] = H[2], A[3] = 2.0 * H[3], A[4] = 3.0 * H[4], A[5] = 4.0 * H[5];
            A[6] = 5.0 * H[6];
        } else {       // Cp = H0 + 2 H1 T + 3 H2 T^2 + 4 H3 T^3 + 5 H4 T^4
            A[0] = H[0], A[1] = 2.0 * H[1], A[2] = 3.0 * H[2], A[3] = 4.0 * H[3], A[4] = 5.0 * H[4];
        }
        return true;
    }
    // h of the mixture at T >= 200 K within the folded range
    __device__ __forceinline__ double eval_h(bool nasa, double T) const {
        if (nasa)
            return fma(H[0], rcp_nr(T), fma(H[1], log(T), fma(fma(fma(fma(fma(H[6], T, H[5]), T, H[4]), T, H[3]), T, H[2]), T, H[7])));
        return fma(fma(fma(fma(fma(H[4], T, H[3]), T, H[2]), T, H[1]), T, H[0]), T, H[5]);
    }
    // h and Cp of the mixture at T >= 200 K within the folded range
    __device__ __forceinline__ void eval(bool nasa, double T, double &h, double &Cp) const {
        if (nasa) {
            const double iT = rcp_nr(T);
            Cp = fma(fma(A[0], iT, A[1]), iT, fma(fma(fma(fma(A[6], T, A[5]), T, A[4]), T, A[3]), T, A[2]));
            h = fma(H[0], iT, fma(H[1], log(T), fma(fma(fma(fma(fma(H[6], T, H[5]), T, H[4]), T, H[3]), T, H[2]), T, H[7])));
        } else {
            Cp = fma(fma(fma(fma(A[4], T, A[3]), T, A[2]), T, A[1]), T, A[0]);
            h = fma(fma(fma(fma(fma(H[4], T, H[3]), T, H[2]), T, H[1]), T, H[0]), T, H[5]);
        }
    }
};

// cop_cell_terms for the mixed form, in FP32: the faces' Roe state averages these terms in FP32
// (face_state_mixed), so they are formed from the FP32 values of T, Cp, gamma and R with the FP32
// copy of the scaled species tables; e = E / rho - |u|^2 / 2 (equal to H - |u|^2 / 2 - p / rho) is
// the caller's. The species sums (h_N - h_n) + (R_n - R_N) Cp T / R cancel by a factor of a few at
// most for the tables here (formation enthalpies included), so the terms carry FP32 rounding.
template <int NS>
__device__ __forceinline__ void cop_cell_terms_mixed(const DevThermo &th, float T0, float Cp, float gm, float R,
                                                     float u, float v, float w, float e, float *xcf, long long P,
                                                     long long id) {
    constexpr int NCOP = NS - 1;
    const float *tab = th.hscf;
    const float T = fmaxf(T0, 200.0f), dT = fminf(T0 - 200.0f, 0.0f);
    const bool nasa = th.nasa;
    int rg = nasa ? (T >= 1000.0f && T < 6000.0f ? 1 : (T < 1000.0f ? 0 : 2)) : (T > 1000.0f ? 0 : 1);
    const float lT = nasa ? logf(T) : 0.0f, iT = nasa ? 1.0f / T : 0.0f;
    float h[NS];
#pragma unroll
    for (int n = 0; n < NS; n++) {
        const float *c = tab + (n * 3 + rg) * 8;
        const float hp = nasa ? fmaf(c[0], iT, fmaf(c[1], lT, fmaf(fmaf(fmaf(fmaf(fmaf(c[6], T, c[5]), T, c[4]), T, c[3]), T, c[2]), T, c[7])))
                              : fmaf(fmaf(fmaf(fmaf(fmaf(c[4], T, c[3]), T, c[2]), T, c[1]), T, c[0]), T, c[5]);
        h[n] = fmaf(tab[THERMO_SC_CP200 + n], dT, hp);
    }
    const float q2 = u * u + v * v + w * w;
    const float CpT_R = Cp * T0 / R;
    const float RN = (float)th.Ri[NCOP];
    const float g1 = gm - 1.0f;
    xcf[id] = gm;
    xcf[P + id] = g1 * (0.5f * q2 - h[NCOP] + RN * CpT_R);
    xcf[2 * P + id] = e;
#pragma unroll
    for (int n = 0; n < NCOP; n++) xcf[(3 + n) * P + id] = g1 * ((h[NCOP] - h[n]) + ((float)th.Ri[n] - RN) * CpT_R);
}

// h and Cp of the mixture by the per-species functions (below 200 K, or a temperature outside the
// tables): a called function, so that the rare path costs the iteration nothing when not taken
template <int NS>
__device__ __noinline__ void mix_h_cp_species(const DevThermo &t, const double *yi, double T, double &h, double &Cp) {
    h = mix_h<NS>(t, yi, T);
    Cp = mix_Cp<NS>(t, yi, T);
}

// The folded mixture polynomials in FP32 (the FP32 copy of the scaled tables), T >= 200 K.
template <int NS>
struct FoldedThermo32 {
    float H[8], A[7];
    int rg = -9;
    __device__ __forceinline__ void fold(const DevThermo &t, const float *yf, int r) {
        if (r == rg) return;
        rg = r;
        const int nc = t.nasa ? 8 : 6;
#pragma unroll
        for (int c = 0; c < 8; c++) H[c] = 0.0f;
#pragma unroll
        for (int n = 0; n < NS; n++) {
            const float *c = t.hscf + (n * 3 + r) * 8;
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (q < nc) H[q] = fmaf(yf[n], c[q], H[q]);
        }
        if (t.nasa) {
            A[0] = -H[0], A[1] = H[1], A[2] = H[2], A[3] = 2.0f * H[3], A[4] = 3.0f * H[4], A[5] = 4.0f * H[5];
            A[6] = 5.0f * H[6];
        } else {
            A[0] = H[0], A[1] = 2.0f * H[1], A[2] = 3.0f * H[2], A[3] = 4.0f * H[3], A[4] = 5.0f * H[4];
        }
    }
    __device__ __forceinline__ void eval(bool nasa, float T, float &h, float &Cp) const {
        if (nasa) {
            const float iT = 1.0f / T;
            Cp = fmaf(fmaf(A[0], iT, A[1]), iT, fmaf(fmaf(fmaf(fmaf(A[6], T, A[5]), T, A[4]), T, A[3]), T, A[2]));
            h = fmaf(H[0], iT, fmaf(H[1], logf(T), fmaf(fmaf(fmaf(fmaf(fmaf(H[6], T, H[5]), T, H[4]), T, H[3]), T, H[2]), T, H[7])));
        } else {
            Cp = fmaf(fmaf(fmaf(fmaf(A[4], T, A[3]), T, A[2]), T, A[1]), T, A[0]);
            h = fmaf(fmaf(fmaf(fmaf(fmaf(H[4], T, H[3]), T, H[2]), T, H[1]), T, H[0]), T, H[5]);
        }
    }
};

// get_T (Mixing_device.h:171-193): the same clamped Newton iteration and stopping test on the
// folded mixture polynomials (Rm the mixture R), the step f / f' with a once-refined reciprocal of
// f' (the iteration goes on until the step is below 1e-6 K, so the step needs no more); returns T
// and the mixture Cp at T.
template <int NS>
__device__ __forceinline__ double newton_T_folded(const DevThermo &t, const double *yi, double Rm, double e,
                                                  double T0, double &Cp_out) {
    FoldedThermo<NS> ft;
    double T = T0;
    for (int it = 1; it < 101; it++) {
        double h, Cp;
        if (T >= 200.0 && ft.fold(t, yi, T))
            ft.eval(t.nasa, T, h, Cp);
        else
            mix_h_cp_species<NS>(t, yi, T, h, Cp);
        double f = h - Rm * T - e;
        double df_ = Cp - Rm;
        double df = fmin(f * rcp_nr1(df_ + 1.0e-30), 1e-3 * T);
        df = fmax(df, -1e-2 * T);
        T = T - df;
        if (fabs(df) <= 1.0e-6) break;
    }
    double h;
    if (T >= 200.0 && ft.fold(t, yi, T)) ft.eval(t.nasa, T, h, Cp_out);
    else mix_h_cp_species<NS>(t, yi, T, h, Cp_out);
    return T;
}

// Temperature of the mixed form: the clamped Newton iteration of get_T run in FP32 on the FP32
// folded polynomials until its step is below 1e-5 T, then one FP64 Newton step on the FP64 folded
// polynomial with the FP32 derivative. The FP32 iterate is within ~1e-3 K of the root (the FP32
// rounding of h - R T - e), so the FP64 step lands within ~1e-10 K of it (the error of a Newton
// step is about (h'' / 2 (h' - R)) times the squared distance, ~1e-4 / K here; a step of up to
// 2e-5 T is accepted), inside the reference's 1e-6 K tolerance. Returns T and the mixture Cp at the FP32 iterate (FP32 accuracy, for gamma and
// the cell terms, which are FP32 downstream);
// below 200 K, across a table range, or without FP32 convergence in 30 iterations it returns the
// FP64 iteration's result instead (newton_T_folded).
template <int NS>
__device__ __forceinline__ double newton_T_mixed(const DevThermo &t, const double *yi, double Rm, double e,
                                                 double T0, double &Cp_out) {
    float yf[NS];
#pragma unroll
    for (int n = 0; n < NS; n++) yf[n] = d2f_rn(yi[n]);
    const float Rf = d2f_rn(Rm), ef = d2f_rn(e);
    const bool nasa = t.nasa;
    FoldedThermo32<NS> ft;
    float T = d2f_rn(T0), Cp = 0.0f;
    bool ok = false;
    for (int it = 0; it < 30; it++) {
        const int r = thermo_range(nasa, T);
        if (!(T >= 200.0f) || r < 0) break;
        ft.fold(t, yf, r);
        float h;
        ft.eval(nasa, T, h, Cp);
        float df = fminf((h - Rf * T - ef) / (Cp - Rf + 1.0e-30f), 1e-3f * T);
        df = fmaxf(df, -1e-2f * T);
        T -= df;
        if (fabsf(df) <= 1.0e-5f * T) {
            ok = T >= 200.0f && thermo_range(nasa, T) == r;
            break;
        }
    }
    if (ok) {  // one FP64 step, with the FP32 derivative
        FoldedThermo<NS> fd;
        const double Td = T;
        if (fd.fold(t, yi, Td)) {
            const double df = (fd.eval_h(nasa, Td) - Rm * Td - e) * rcp_nr1((double)(Cp - Rf));
            if (fabs(df) <= 2.0e-5 * Td) {
                Cp_out = Cp;
                return Td - df;
            }
        }
    }
    return newton_T_folded<NS>(t, yi, Rm, e, T0, Cp_out);
}

// Primitive recovery of the mixed form. Single gas: from the FP64 state converted once to FP32.
// Mixture: the FP64 recovery of k_states (Newton in FP64, refined reciprocals instead of
// divisions) and the FP64 cell terms of the sound speed, their FP32 copies (and those of y) for the
// faces' FP32 Roe averages, converted by integer operations; the sound speed in FP32.
template <bool COP, int NS>
__device__ __forceinline__ void states_mixed_body(const Geo &g, const DevFields &f, const DevThermo &th,
                                                  double *__restrict__ UI, int ghost, int want_lam, long long id,
                                                  float &lamx, float &lamy, float &lamz) {
    using S = Sys<COP, NS>;
    constexpr int E = S::E, NCOP = S::NCOP;
    const long long P = g.pitch, N = g.ncell();
    if (id < N) {
        float Uf[E];
        float rho, u, v, w, p, H, c;
        float yf[NS];
        if (!COP) {
#pragma unroll
            for (int n = 0; n < E; n++) Uf[n] = (float)UI[n * P + id];
            rho = Uf[0];
            const float rho1 = 1.0f / rho;
            u = Uf[1] * rho1, v = Uf[2] * rho1, w = Uf[3] * rho1;
            const float tme = Uf[4] * rho1 - 0.5f * (u * u + v * v + w * w);
            const float gm = (float)th.ncop_gamma;
            p = (gm - 1.0f) * rho * tme;
            H = (Uf[4] + p) * rho1;
            c = sqrtf(gm * p * rho1);
            yf[0] = 1.0f;
        } else {
            double U[E];
#pragma unroll
            for (int n = 0; n < E; n++) U[n] = UI[n * P + id];
            const double rhod = U[0], rho1 = rcp_nr(rhod);
            double yi[NS];
            if (ghost) {
                yi[NCOP] = 0.0;
                double sum = 0.0;
#pragma unroll
                for (int s = 0; s < NCOP; s++) yi[s] = U[s + 5] * rho1, sum += yi[s];
                sum = rcp_nr(sum);
#pragma unroll
                for (int s = 0; s < NCOP; s++) {
                    yi[s] *= sum;
                    U[s + 5] = rhod * yi[s];
                    UI[(s + 5) * P + id] = U[s + 5];
                }
            } else {
                yi[NCOP] = 1.0;
#pragma unroll
                for (int s = 0; s < NCOP; s++) yi[s] = U[s + 5] * rho1, yi[NCOP] += -yi[s];
            }
            const double ud = U[1] * rho1, vd = U[2] * rho1, wd = U[3] * rho1;
            const double tme = U[4] * rho1 - 0.5 * (ud * ud + vd * vd + wd * wd);
            const double wi = mix_W_inv<NS>(th, yi), Rm = wi * kRu;  // sum y_n / W_n; the mixture R
            double Cp;
            const double T = newton_T_mixed<NS>(th, yi, Rm, tme, f.T[id], Cp);
            const double pd = rhod * Rm * T;
            // gamma feeds only FP32 quantities (the sound speed, the cell terms): FP32 from the FP32 Cp
            const float Cpf = d2f_rn(Cp), Rf = d2f_rn(Rm), gmx = Cpf / (Cpf - Rf);
            const double gamma = gmx > 1.0f ? (double)gmx : -1.0;
            const double Hd = (U[4] + pd) * rho1;
            f.rho[id] = rhod, f.u[id] = ud, f.v[id] = vd, f.w[id] = wd, f.p[id] = pd, f.H[id] = Hd;
            f.e[id] = tme, f.gamma[id] = gamma, f.T[id] = T, f.Cp[id] = Cp, f.R[id] = Rm;
            if (f.Tf) f.Tf[id] = d2f_rn(T);  // viscous schemes: the heat flux's FP32 temperature
            cop_cell_terms_mixed<NS>(th, d2f_rn(T), Cpf, gmx, Rf, d2f_rn(ud), d2f_rn(vd), d2f_rn(wd), d2f_rn(tme),
                                     f.xcf, P, id);
#pragma unroll
            for (int s = 0; s < NS; s++) f.y[s * P + id] = yi[s], yf[s] = d2f_rn(yi[s]), f.yf[s * P + id] = yf[s];
#pragma unroll
            for (int n = 0; n < E; n++) Uf[n] = d2f_rn(U[n]);
            rho = d2f_rn(rhod), u = d2f_rn(ud), v = d2f_rn(vd), w = d2f_rn(wd), p = d2f_rn(pd), H = d2f_rn(Hd);
            // the sound speed feeds only the FP32 face primitives (LLF maxima, dt): FP32
            c = sqrtf(d2f_rn(gamma) * p / rho);
            f.c[id] = (double)c;
        }
#pragma unroll
        for (int n = 0; n < E; n++) f.Uf[n * P + id] = Uf[n];
        float *pf = f.primf;
        pf[0 * P + id] = rho, pf[1 * P + id] = u, pf[2 * P + id] = v, pf[3 * P + id] = w;
        pf[4 * P + id] = H, pf[5 * P + id] = p, pf[6 * P + id] = c;
        const float Ep = Uf[4] + p;
        const float mom[3] = {Uf[1], Uf[2], Uf[3]}, vel[3] = {u, v, w};
        const int dims[3] = {g.dimx, g.dimy, g.dimz};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (!dims[d]) continue;
            float *F = f.Ff[d];
            F[0 * P + id] = mom[d];
            F[1 * P + id] = mom[d] * u + (d == 0 ? p : 0.f);
            F[2 * P + id] = mom[d] * v + (d == 1 ? p : 0.f);
            F[3 * P + id] = mom[d] * w + (d == 2 ? p : 0.f);
            F[4 * P + id] = Ep * vel[d];
#pragma unroll
            for (int n = 5; n < E; n++) F[n * P + id] = mom[d] * yf[n - 5];
        }
        int i, j, k;
        split_index(id, g.Xmax, g.Ymax, i, j, k);
        const bool inner = i >= g.Bx && i < g.Xmax - g.Bx && j >= g.By && j < g.Ymax - g.By && k >= g.Bz && k < g.Zmax - g.Bz;
        if (inner && (!(rho >= 0.f) || !(p >= 0.f) || isinf(rho) || isinf(p))) {
            atomicOr(&f.err[ERR_PRIM], 1);
            f.err[ERR_I] = i, f.err[ERR_J] = j, f.err[ERR_K] = k;
        }
        if (want_lam) {
            const float c_local = sqrtf(1.4f * p / rho);
            lamx = fabsf(u) + c_local, lamy = fabsf(v) + c_local, lamz = fabsf(w) + c_local;
            if (!(lamx >= 0.f)) lamx = __int_as_float(0x7f800000);
            if (!(lamy >= 0.f)) lamy = __int_as_float(0x7f800000);
            if (!(lamz >= 0.f)) lamz = __int_as_float(0x7f800000);
        }
    }
}

__device__ __forceinline__ void lam_block_reduce_f(const Geo &g, const DevFields &f, float lamx, float lamy, float lamz) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lamx = fmaxf(lamx, __shfl_xor_sync(0xffffffffu, lamx, o));
        lamy = fmaxf(lamy, __shfl_xor_sync(0xffffffffu, lamy, o));
        lamz = fmaxf(lamz, __shfl_xor_sync(0xffffffffu, lamz, o));
    }
    __shared__ float red[3][kThreads / 32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[0][wid] = lamx, red[1][wid] = lamy, red[2][wid] = lamz;
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = red[0][0], b = red[1][0], c = red[2][0];
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) a = fmaxf(a, red[0][q]), b = fmaxf(b, red[1][q]), c = fmaxf(c, red[2][q]);
        if (g.dimx) atomic_max_nonneg(&f.lam[0], (double)a);
        if (g.dimy) atomic_max_nonneg(&f.lam[1], (double)b);
        if (g.dimz) atomic_max_nonneg(&f.lam[2], (double)c);
    }
}

template <bool COP, int NS>
__global__ void __launch_bounds__(kThreads) k_states_mixed(Geo g, DevFields f, DevThermo th, double *__restrict__ UI,
                                                           int ghost, int want_lam, int guard) {
    if (guard && step_done(f)) return;
    float lamx = 0.f, lamy = 0.f, lamz = 0.f;
    states_mixed_body<COP, NS>(g, f, th, UI, ghost, want_lam, (long long)blockIdx.x * blockDim.x + threadIdx.x, lamx,
                               lamy, lamz);
    if (want_lam) lam_block_reduce_f(g, f, lamx, lamy, lamz);
}

// GLF maxima of the single-gas mixed form from its FP32 face primitives (this form writes no FP64
// primitives): max over all cells of |u_d - c|, |u_d|, |u_d + c| (ConVenction_block.hpp:115-215).
static __global__ void __launch_bounds__(kThreads) k_glf_mixed(Geo g, DevFields f, unsigned long long *glf, int guard) {
    if (guard && step_done(f)) return;
    const long long N = g.ncell(), P = g.pitch;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double m[9];
    for (int q = 0; q < 9; q++) m[q] = 0.0;
    if (id < N) {
        const double c = f.primf[6 * P + id];
        for (int d = 0; d < 3; d++) {
            const double v = f.primf[(1 + d) * P + id];
            m[3 * d + 0] = fabs(v - c);
            m[3 * d + 1] = fabs(v);
            m[3 * d + 2] = fabs(v + c);
        }
    }
    for (int q = 0; q < 9; q++) {
        double x = m[q];
        for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&glf[q], x);
    }
}

template <int D, int E>
__device__ __forceinline__ float project_f(const float *lrow, int n, const float *__restrict__ A, long long P, long long q) {
    float acc = 0.f;
    bool first = true;
#pragma unroll
    for (int k = 0; k < E; k++) {
        const int kind = left_kind(D, E, n, k);
        if (kind == 0) continue;
        const float x = __ldg(A + k * P + q);
        float t = kind == 1 ? x : (kind == 2 ? -x : x * lrow[k]);
        acc = first ? t : acc + t;
        first = false;
    }
    return acc;
}

template <int D, int E>
__device__ __forceinline__ float project_r(const float *lrow, int n, const float *x) {
    float acc = 0.f;
    bool first = true;
#pragma unroll
    for (int k = 0; k < E; k++) {
        const int kind = left_kind(D, E, n, k);
        if (kind == 0) continue;
        float t = kind == 1 ? x[k] : (kind == 2 ? -x[k] : x[k] * lrow[k]);
        acc = first ? t : acc + t;
        first = false;
    }
    return acc;
}

// Roe state of a mixture face for the mixed form: the quantities of face_state's mixture branch
// (MARCO_ROE, Eigen_callback.h:87-91 and Utils_device.hpp:42-140: Roe averages, the pressure-
// derivative correction of the multi-component sound speed, the MARCO_PREEIGEN terms) in FP32,
// except the jumps across the face. The correction temp = (dp - dp/drho drho - dp/de de -
// sum dp/drho_n drho_n) / den is a second-order residual of first-order jumps: from jumps of
// FP32-rounded states its rounding would be eps / |jump| relative, while jumps taken in FP64 and
// then rounded leave it, and the sound speed it corrects, at FP32 rounding (eps) like the other
// averages. So the jumps of rho, p, e, u, v, w and rho_n come from the FP64 states (11 FP64
// operations a face), everything else from the FP32 copies of k_states_mixed.
template <int NS>
__device__ __forceinline__ void face_state_mixed(const DevFields &f, long long P, long long l, long long r,
                                                 FaceStateT<float, NS> &F) {
    constexpr int NCOP = NS - 1;
    const float *pf = f.primf, *yf = f.yf, *xf = f.xcf;
    const float rl = pf[l], rr = pf[r];
    const float D = sqrtf(rr / rl);
    const float D1 = 1.0f / (D + 1.0f);
    auto roe = [&](float a, float b) { return fmaf(D, b, a) * D1; };  // (a + D b) / (1 + D)
    const float _u = roe(pf[P + l], pf[P + r]), _v = roe(pf[2 * P + l], pf[2 * P + r]);
    const float _w = roe(pf[3 * P + l], pf[3 * P + r]), _H = roe(pf[4 * P + l], pf[4 * P + r]);
    const float pl = pf[5 * P + l], pr = pf[5 * P + r], _P = roe(pl, pr);
    const float _rho = sqrtf(rr * rl);
    float yi[NS];
#pragma unroll
    for (int n = 0; n < NS; n++) yi[n] = roe(yf[n * P + l], yf[n * P + r]);
    const float gl = xf[l], gr = xf[r];
    const float _dpdrho = roe(xf[P + l], xf[P + r]);
    float dpdrhoi[NCOP > 0 ? NCOP : 1], drhoi[NCOP > 0 ? NCOP : 1];
    // the jumps, from the FP64 states
    const double rl64 = f.rho[l], rr64 = f.rho[r];
    const float drho = d2f_rn(rr64 - rl64), dp = d2f_rn(f.p[r] - f.p[l]);
    const float de = d2f_rn(f.e[r] - f.e[l]);
    const float du = d2f_rn(f.u[r] - f.u[l]), dv = d2f_rn(f.v[r] - f.v[l]), dw = d2f_rn(f.w[r] - f.w[l]);
#pragma unroll
    for (int n = 0; n < NCOP; n++) {
        dpdrhoi[n] = roe(xf[(3 + n) * P + l], xf[(3 + n) * P + r]);
        drhoi[n] = d2f_rn(fma(rr64, f.y[n * P + r], -(rl64 * f.y[n * P + l])));
    }
    const float Gamma0 = roe(gl, gr);
    const float _prho = roe(pl / rl, pr / rr) + 0.5f * D * D1 * D1 * (du * du + dv * dv + dw * dw);
    const float _dpdE = roe(gl - 1.0f, gr - 1.0f);
    const float _dpde = ((gl - 1.0f) * rl + D * ((gr - 1.0f) * rr)) * D1;
    float S1 = 0.0f, S2 = 0.0f, SY = 0.0f;
#pragma unroll
    for (int n = 0; n < NCOP; n++) {
        const float t = dpdrhoi[n] * drhoi[n];
        S1 += t, S2 += t * t;
    }
    const float temp1 = dp - ((_dpdrho * drho + _dpde * de) + S1);
    const float den = ((_dpdrho * _dpdrho * drho * drho + _dpde * de * _dpde * de) + S2) + 1e-19f;
    const float temp = temp1 / den;
#pragma unroll
    for (int n = 0; n < NCOP; n++) SY += yi[n] * dpdrhoi[n];
    const float _dpdE_new = _dpdE + _dpdE * _dpdE * de * _rho * temp;
    const float _dpdrho_new = _dpdrho + _dpdrho * _dpdrho * drho * temp;
    const float csqr = (_dpdrho_new + _dpdE_new * _prho) + SY;
    const float b1 = _dpdE_new / csqr;
    const float inv_dpdE = 1.0f / _dpdE_new;
    float b3 = 0.0f;
#pragma unroll
    for (int n = 0; n < NCOP; n++) {
        const float z = -(dpdrhoi[n] + dpdrhoi[n] * dpdrhoi[n] * drhoi[n] * temp) * inv_dpdE;
        F.z[n] = z;
        b3 += yi[n] * z;
    }
    b3 *= b1;
    const float c2w = (0.0f < csqr) ? 0.0f : 1.0f;
    const float c2 = Gamma0 * _P * _rho * c2w + (1.0f - c2w) * csqr;
    const float q2 = _u * _u + _v * _v + _w * _w;
    const float b2 = (1.0f + b1 * q2) - b1 * _H;
    F._u = _u, F._v = _v, F._w = _w, F._H = _H, F._P = _P, F._rho = _rho;
    F.c2 = c2, F.b1 = b1, F.b3 = b3, F.q2 = q2, F.b2 = b2;
    F._c = sqrtf(c2), F._c1 = 1.0f / F._c;
    F.ent0 = ((1.0f - b2) - b3) * (csqr * inv_dpdE);
#pragma unroll
    for (int n = 0; n < NS; n++) F._yi[n] = yi[n];
}

// FP32 characteristic WENO flux at face (i+1/2) of direction D (same structure as k_faces).
template <int D, bool COP, int NS, int ORDER>
__device__ __forceinline__ void faces_mixed_body(const Geo &g, const DevFields &f, const DevThermo &th, int artificial,
                                                 const double *__restrict__ glf_d, int i, int j, int k) {
    using S = Sys<COP, NS>;
    constexpr int E = S::E;
    const long long P = g.pitch;
    const long long stride = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long idl = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long idr = idl + stride;
    const float *__restrict__ pf = f.primf;

    FaceStateT<float, NS> F;
    if (!COP) {
        const float rl = pf[idl], rr = pf[idr];
        const float Dd = sqrtf(rr / rl);
        const float D1 = 1.0f / (Dd + 1.0f);
        F._u = (pf[1 * P + idl] + Dd * pf[1 * P + idr]) * D1;
        F._v = (pf[2 * P + idl] + Dd * pf[2 * P + idr]) * D1;
        F._w = (pf[3 * P + idl] + Dd * pf[3 * P + idr]) * D1;
        F._H = (pf[4 * P + idl] + Dd * pf[4 * P + idr]) * D1;
        F._P = (pf[5 * P + idl] + Dd * pf[5 * P + idr]) * D1;
        F._rho = sqrtf(rr * rl);
        const float gm = (float)th.ncop_gamma;
        F.c2 = gm * F._P / F._rho;
        F.b1 = (gm - 1.0f) / F.c2;
        F.b3 = 0.f;
        F._yi[0] = 1.f;
        F.q2 = F._u * F._u + F._v * F._v + F._w * F._w;
        F._c = sqrtf(F.c2);
        F.b2 = 1.0f + F.b1 * F.q2 - F.b1 * F._H;
        F._c1 = 1.0f / F._c;
        F.ent0 = (1.0f - F.b2 - F.b3) / F.b1;
    } else {
        face_state_mixed<NS>(f, P, idl, idr, F);
    }
    const float un = D == 0 ? F._u : (D == 1 ? F._v : F._w);
    const float *__restrict__ Fl = f.Ff[D];
    const float *__restrict__ Ua = f.Uf;
    const float *__restrict__ vd = pf + (1 + D) * P;
    const float *__restrict__ cf = pf + 6 * P;
    float lm0 = 0.f, lm1 = 0.f, lm2 = 0.f;
    if (ORDER != 7 && artificial == XFG_LLF) {
#pragma unroll
        for (int m = -2; m <= 3; m++) {
            const long long q = idl + m * stride;
            const float ud = __ldg(vd + q), cc = __ldg(cf + q);
            lm0 = fmaxf(lm0, fabsf(ud - cc));
            lm1 = fmaxf(lm1, fabsf(ud));
            lm2 = fmaxf(lm2, fabsf(ud + cc));
        }
    }
    constexpr int M0 = ORDER == 7 ? -3 : -2, M1 = ORDER == 7 ? 4 : 3;
    constexpr int NP = M1 - M0 + 1;
    // single gas: every stencil value is loaded once into registers and projected on all fields;
    // mixtures (larger E) re-read the stencil from L1 per field to bound register use
    constexpr bool PRELOAD = E <= 6;
    float Us[PRELOAD ? NP : 1][PRELOAD ? E : 1], Fs[PRELOAD ? NP : 1][PRELOAD ? E : 1];
    if constexpr (PRELOAD) {
#pragma unroll
        for (int m = 0; m < NP; m++) {
            const long long q = idl + (m + M0) * stride;
#pragma unroll
            for (int kk = 0; kk < E; kk++) Us[m][kk] = __ldg(Ua + kk * P + q), Fs[m][kk] = __ldg(Fl + kk * P + q);
        }
    }
    float acc[E];
#pragma unroll
    for (int n = 0; n < E; n++) {
        // Mixtures across the sweep (strided stencil): the stencil addresses are the same for every
        // field, and computed once they would stay live through the field loop (8 points x E
        // components x 2 arrays of 64-bit addresses, 255 registers). An opaque copy of the stride
        // per field makes them cheap integer work recomputed per field instead.
        long long stride_n = stride;
        if constexpr (!PRELOAD && D != 0) asm volatile("mov.b64 %0, %0;" : "+l"(stride_n));
        const float ev = n == 0 ? fabsf(un - F._c) : (n == E - 1 ? fabsf(un + F._c) : fabsf(un));
        float av;
        if (artificial == XFG_ROE || ORDER == 7) {
            av = ev;
            if (ORDER == 7 && artificial == XFG_GLF) av = 0.f;
        } else if (artificial == XFG_LLF) {
            av = n == 0 ? lm0 : (n == E - 1 ? lm2 : lm1);
        } else {
            av = (float)glf_d[n == 0 ? 0 : (n == E - 1 ? 2 : 1)];
        }
        float lrow[E];
#pragma unroll
        for (int kk = 0; kk < E; kk++) lrow[kk] = left_kind(D, E, n, kk) == 3 ? left_val<D, E>(F, n, kk) : 0.f;
        float pp[8], mm[8];
#pragma unroll
        for (int m = M0; m <= M1; m++) {
            float uf, ff;
            if constexpr (PRELOAD) {
                uf = project_r<D, E>(lrow, n, Us[m - M0]);
                ff = project_r<D, E>(lrow, n, Fs[m - M0]);
            } else {
                const long long q = idl + m * stride_n;
                uf = project_f<D, E>(lrow, n, Ua, P, q);
                ff = project_f<D, E>(lrow, n, Fl, P, q);
            }
            pp[m + 3] = 0.5f * (ff + av * uf);
            mm[m + 3] = 0.5f * (ff - av * uf);
        }
        float fl;
        if constexpr (ORDER == 7) fl = weno7(pp, mm);
        else if constexpr (ORDER == 6) fl = wenocu6(pp, mm, (float)(D == 0 ? g.dx : (D == 1 ? g.dy : g.dz)));
        else fl = weno5(pp, mm);
#pragma unroll
        for (int kk = 0; kk < E; kk++) {
            const int kind = right_kind(D, E, n, kk);
            if (kind == 0) continue;
            const float tv = kind == 1 ? fl : (kind == 2 ? -fl : fl * right_val<D, E>(F, n, kk));
            acc[kk] = (n == 0) ? tv : acc[kk] + tv;
        }
    }
    float *Fw = f.Fwf[D];
#pragma unroll
    for (int n = 0; n < E; n++) Fw[n * P + idl] = acc[n];
}

template <int D, bool COP, int NS, int ORDER>
__global__ void __launch_bounds__(kThreads) k_faces_mixed(Geo g, DevFields f, DevThermo th, int artificial,
                                                          const double *__restrict__ glf_d, int guard) {
    if (guard && step_done(f)) return;
    int i, j, k;
    if (!face_of_thread<D>(g, i, j, k)) return;
    faces_mixed_body<D, COP, NS, ORDER>(g, f, th, artificial, glf_d, i, j, k);
}

// The single-gas WENO5 kernel with its registers fitted to XFG_FACES_MIXED_MINB resident blocks
// per SM: 5 blocks of 128 threads give 96 registers (120 unbounded) and an 84-byte spill, measured
// +2.7 % on the 4096^2 vortex. Other orders and the mixtures stay unbounded (a bound spilled them
// more and cost the mixture kernels 2 %).
#ifndef XFG_FACES_MIXED_MINB
#define XFG_FACES_MIXED_MINB 5
#endif
template <int D>
__global__ void __launch_bounds__(kThreads, XFG_FACES_MIXED_MINB)
    k_faces_mixed_w5(Geo g, DevFields f, DevThermo th, int artificial, const double *__restrict__ glf_d, int guard) {
    if (guard && step_done(f)) return;
    int i, j, k;
    if (!face_of_thread<D>(g, i, j, k)) return;
    faces_mixed_body<D, false, 1, 5>(g, f, th, artificial, glf_d, i, j, k);
}

// Positivity limiter of the mixed form: the FP32 physical and face fluxes, the FP64 state.
template <int D, bool COP, int NS>
__global__ void __launch_bounds__(kThreads) k_pp_mixed(Geo g, DevFields f, const double *__restrict__ UI,
                                                       const double *__restrict__ lam0, double cfl, int guard) {
    if (guard && step_done(f)) return;
    using S = Sys<COP, NS>;
    const double l0 = lam0[D];
    pp_body<D, S::E, S::NCOP, float>(g, UI, f.Ff[D], f.Fwf[D], l0, cfl / l0,
                                     (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Knuth's TwoSum: a + b = s + e exactly (round to nearest, no overflow). The _rn intrinsics keep
// the compiler from contracting or reordering the steps.
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
    return s;
}

// float -> double through the bit patterns of IEEE 754 binary32 and binary64 (exponent rebias
// 127 -> 1023, mantissa shifted by 29), integer operations only, so nothing of it runs on the FP64
// pipe: exact for zeros, normal floats, infinities and NaNs (payload kept); subnormal floats
// (|x| < 2^-126) become zero.
__device__ __forceinline__ double f2d_bits(float x) {
    const unsigned u = __float_as_uint(x), mag = u & 0x7fffffffu, sign = u & 0x80000000u;
    const bool normal = mag - 0x00800000u < 0x7f000000u, special = mag >= 0x7f800000u;
    const unsigned hi = sign | (normal ? (mag >> 3) + (896u << 20) : special ? 0x7ff00000u | ((mag & 0x7fffffu) >> 3) : 0u);
    const unsigned lo = (normal || special) ? u << 29 : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

// One direction's share of the divergence of component q, added to the float pair (s, c):
// (Fa - Fb) * (1/dx) with the difference taken exactly (TwoSum) and the product with the float
// pair 1/dx = sh + sl to about 2^-48, so that every face flux enters its two cells with equal and
// opposite weight up to that level and the sum over cells telescopes.
__device__ __forceinline__ void div_acc(float a, float b, float sh, float sl, float &s, float &c) {
    float e;
    const float d = two_sum(a, -b, e);
    const float p = __fmul_rn(d, sh);
    const float pe = fmaf(e, sh, fmaf(d, sl, fmaf(d, sh, -p)));
    float e2;
    s = two_sum(s, p, e2);
    c = __fadd_rn(c, __fadd_rn(e2, pe));
}

// Divergence of the FP32 face fluxes and the SSP-RK3 stage in FP64 (a12, a13: the reference's
// UpdateFluidLU, Reconstruction_kernels.hpp:201-234, and UpdateURK3rdKernel, Update_kernels.hpp:64-94).
// The divergence is accumulated as an unevaluated float pair (s + c, compensated summation) and
// enters the FP64 stage sum as two exactly converted doubles, so the FP32 fluxes' rounding stays in
// the fluxes, where it cancels between neighbouring cells, and the conserved sums of U move only by
// the FP64 stage arithmetic.
template <int E>
__device__ __forceinline__ void div_rk_mixed_body(const Geo &g, const DevFields &f, int flag, double dt, int do_rk,
                                                  int store_lu, long long t) {
    const long long P = g.pitch;
    if (t >= (long long)g.Xi * g.Yi * g.Zi) return;
    int i, j, k;
    split_index(t, g.Xi, g.Yi, i, j, k);
    i += g.Bx, j += g.By, k += g.Bz;
    const long long id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long sy = g.Xmax, sz = (long long)g.Xmax * g.Ymax;
    int code = 0;
#pragma unroll
    for (int n = 0; n < E; n++) {
        const long long q = n * P + id;
        float s = 0.f, c = 0.f;
        if (g.dimx) div_acc(f.Fwf[0][q - 1], f.Fwf[0][q], g.idh[0], g.idl[0], s, c);
        if (g.dimy) div_acc(f.Fwf[1][q - sy], f.Fwf[1][q], g.idh[1], g.idl[1], s, c);
        if (g.dimz) div_acc(f.Fwf[2][q - sz], f.Fwf[2][q], g.idh[2], g.idl[2], s, c);
        const double LU0 = f2d_bits(s) + f2d_bits(c);
        if (store_lu) f.LU[q] = LU0;
        if (!isfinite(s)) code = 1;
        if (do_rk) {
            double out;
            if (flag == 1) {
                out = f.U[q] + dt * LU0;
                f.U1[q] = out;
            } else if (flag == 2) {
                out = 0.75 * f.U[q] + 0.25 * f.U1[q] + 0.25 * dt * LU0;
                f.U1[q] = out;
            } else {
                out = (f.U[q] + 2.0 * f.U1[q] + 2.0 * dt * LU0) * kOT;
                f.U[q] = out;
            }
            if (bad(out) || (n == 0 && out < 0.0)) code = 1;
        }
    }
    if (code) {
        atomicOr(&f.err[ERR_STATE], 1);
        f.err[ERR_I] = i, f.err[ERR_J] = j, f.err[ERR_K] = k;
    }
}

template <int E>
__global__ void __launch_bounds__(kThreads) k_div_rk_mixed(Geo g, DevFields f, int flag, double dt_arg,
                                                           const double *__restrict__ dt_dev, int do_rk, int store_lu,
                                                           int guard) {
    if (guard && step_done(f)) return;
    div_rk_mixed_body<E>(g, f, flag, dt_dev ? dt_dev[0] : dt_arg, do_rk, store_lu,
                         (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace XFG_KNS
}  // namespace xfg
