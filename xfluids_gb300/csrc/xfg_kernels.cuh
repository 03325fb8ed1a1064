// xfg_kernels.cuh - CUDA kernels of the convective right-hand side (FP64 path).
//
// Stage pipeline per RK stage (the reference's kernels in brackets):
//   k_bc          ghost fill, one launch per active direction   [FluidBCKernelX/Y/Z]
//   k_states      rho, Y, primitives, T Newton, physical fluxes [Updaterhoyi + UpdateFuidStatesKernel]
//                 + NaN/negativity check + GetDt wave-speed maxima (block reduce + atomicMax)
//   k_faces<D>    characteristic WENO flux at every face of direction D
//                 [GetLocalEigen + ReconstructFlux{X,Y,Z}], one thread per face
//   k_div_rk      flux divergence and the SSP-RK3 stage combination, fused, with the NaN check
//                 [UpdateFluidLU + EstimateFluidNANKernel + UpdateURK3rdKernel]
// and once per step k_dt_step [GetDt host arithmetic + the time clip of XFLUIDS::Evolution].
#pragma once

#include "xfg_device.cuh"

namespace xfg {

constexpr int kThreads = 128;

// error words in DevFields::err
enum { ERR_STATE = 0, ERR_PRIM = 1, ERR_I = 2, ERR_J = 3, ERR_K = 4, ERR_TMA = 5, ERR_NWORDS = 8 };

namespace XFG_KNS {

__device__ __forceinline__ bool bad(double x) {  // NaN or Inf through the exponent bits
    return ((__double2hiint(x) & 0x7ff00000) == 0x7ff00000);
}

__device__ __forceinline__ bool step_done(const DevFields &f) { return f.dtbuf && f.dtbuf[4] != 0.0; }

// ---------------------------------------------------------------------------------------------
// Boundary conditions, BCs_kernels.hpp:9-258 with the launch arguments of BCs_block.cpp:4-218.
// One thread per (ghost layer, transverse cell) covering both faces of direction D.
// ---------------------------------------------------------------------------------------------
template <int D, int E>
__device__ __forceinline__ void bc_body(const Geo &g, double *__restrict__ U, int bc_lo, int bc_hi, long long t) {
    const int bw = D == 0 ? g.Bx : (D == 1 ? g.By : g.Bz);
    const int inner = D == 0 ? g.Xi : (D == 1 ? g.Yi : g.Zi);
    const int nmax = D == 0 ? g.Xmax : (D == 1 ? g.Ymax : g.Zmax);
    // transverse extents (full, ghosts included)
    const int ta = D == 0 ? g.Ymax : g.Xmax;
    const int tb = D == 2 ? g.Ymax : g.Zmax;
    long long total = (long long)bw * ta * tb;
    if (t >= total) return;
    int gl = (int)(t % bw);
    long long r = t / bw;
    int a = (int)(r % ta), b = (int)(r / ta);
    const long long P = g.pitch;
    auto cell = [&](int cn) -> long long {
        int i = D == 0 ? cn : a;
        int j = D == 0 ? a : (D == 1 ? cn : b);
        int k = D == 2 ? cn : b;
        return (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    };
    for (int side = 0; side < 2; side++) {
        const int BC = side == 0 ? bc_lo : bc_hi;
        const int cn = side == 0 ? gl : gl + nmax - bw;
        const int mirror_offset = side == 0 ? 0 : inner;
        const int index_inner = side == 0 ? bw : nmax - bw - 1;
        const int sign = side == 0 ? 1 : -1;
        const long long id = cell(cn);
        long long src;
        switch (BC) {
        case XFG_SYMMETRY:
            src = cell(2 * (bw + mirror_offset) - 1 - cn);
#pragma unroll
            for (int n = 0; n < E; n++) U[n * P + id] = (n == 1 + D) ? -U[n * P + src] : U[n * P + src];
            break;
        case XFG_PERIODIC:
            src = cell(cn + sign * inner);
#pragma unroll
            for (int n = 0; n < E; n++) U[n * P + id] = U[n * P + src];
            break;
        case XFG_OUTFLOW:
            src = cell(index_inner);
#pragma unroll
            for (int n = 0; n < E; n++) U[n * P + id] = U[n * P + src];
            break;
        case XFG_NSLIPWALL:
        case XFG_VISCWALL:
        case XFG_SLIPWALL:
            // FluidBCKernelY/Z mirror nslipWall only (viscWall / slipWall are no-ops there);
            // FluidBCKernelX mirrors all three walls
            if (D != 0 && BC != XFG_NSLIPWALL) break;
            src = cell(2 * (bw + mirror_offset) - 1 - cn);
#pragma unroll
            for (int n = 0; n < E; n++) U[n * P + id] = (n >= 1 && n <= 3) ? -U[n * P + src] : U[n * P + src];
            break;
        default:
            break;
        }
    }
}
template <int D, int E>
__global__ void __launch_bounds__(kThreads) k_bc(Geo g, double *__restrict__ U, int bc_lo, int bc_hi,
                                                 const double *__restrict__ guard_dtbuf) {
    if (guard_dtbuf && guard_dtbuf[4] != 0.0) return;
    bc_body<D, E>(g, U, bc_lo, bc_hi, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------------------------
// Primitive recovery and physical fluxes on all cells: Getrhoyi (Update_device.hpp:7-29),
// GetStates (:33-54), GetPhysFlux (:81-110); the inner-cell checks of EstimateYiKernel /
// EstimatePrimitiveVarKernel (Estimate_kernels.hpp); the GetDt maxima of |u_d| + sqrt(1.4 p/rho)
// over all cells (GlobalDt_block.hpp:31-66) when want_lam.
// ---------------------------------------------------------------------------------------------
// Per-cell terms of the multi-component interface sound speed (SoundSpeedMultiSpecies,
// Utils_device.hpp:42-140): the cell halves of every Roe-weighted average the face forms, with the
// reference's expressions, so a face reading them gets the values it would compute itself.
//   xc[0] gamma = Cp / (Cp - Ru / W)           xc[1] (gamma - 1) (q^2/2 - h_N + Cp R_N T / R)
//   xc[2] e = H - q^2/2 - p / rho               xc[3 + n] (gamma - 1) ((h_N - h_n) + Cp (R_n - R_N) T / R)
template <int NS>
__device__ __forceinline__ void cop_cell_terms(const DevThermo &th, const double *yi, double T, double Cp, double u,
                                               double v, double w, double H, double p, double rho, double *xc,
                                               long long P, long long id) {
    constexpr int NCOP = NS - 1;
    double h[NS];
#pragma unroll
    for (int n = 0; n < NS; n++) h[n] = enthalpy(th, T, n);
    const double wi = mix_W_inv<NS>(th, yi);
    const double gm = Cp / (Cp - kRu * wi);
    const double q2 = u * u + v * v + w * w;
    const double Rm = wi * kRu;
    const double RN = th.Ri[NCOP];
    const double RNT = RN * T;
    xc[id] = gm;
    xc[P + id] = (gm - 1.0) * (0.5 * q2 - h[NCOP] + Cp * RNT / Rm);
    xc[2 * P + id] = H - 0.5 * q2 - p / rho;
#pragma unroll
    for (int n = 0; n < NCOP; n++) {
        const double Rin_RN = th.Ri[n] - RN;
        xc[(3 + n) * P + id] = (gm - 1.0) * ((-h[n] + h[NCOP]) + Cp * Rin_RN * T / Rm);
    }
}

template <bool COP, int NS>
__device__ __forceinline__ void states_body(const Geo &g, const DevFields &f, const DevThermo &th,
                                            double *__restrict__ UI, int ghost, int want_lam, long long id,
                                            double &lamx, double &lamy, double &lamz) {
    using S = Sys<COP, NS>;
    constexpr int E = S::E, NCOP = S::NCOP;
    const long long P = g.pitch, N = g.ncell();
    if (id < N) {
        double U[E];
#pragma unroll
        for (int n = 0; n < E; n++) U[n] = UI[n * P + id];
        const double rho = U[0];
        const double rho1 = 1.0 / rho;
        double yi[NS];
        if (COP) {
            if (ghost) {
                yi[NCOP] = 0.0;
                double sum = 0.0;
#pragma unroll
                for (int s = 0; s < NCOP; s++) yi[s] = U[s + 5] * rho1, sum += yi[s];
                sum = 1.0 / sum;
#pragma unroll
                for (int s = 0; s < NCOP; s++) {
                    yi[s] *= sum;
                    U[s + 5] = rho * yi[s];
                    UI[(s + 5) * P + id] = U[s + 5];
                }
            } else {
                yi[NCOP] = 1.0;
#pragma unroll
                for (int s = 0; s < NCOP; s++) yi[s] = U[s + 5] * rho1, yi[NCOP] += -yi[s];
            }
        }
        const double u = U[1] * rho1, v = U[2] * rho1, w = U[3] * rho1;
        const double tme = U[4] * rho1 - 0.5 * (u * u + v * v + w * w);
        double p, gamma, T = 0.0, Cp = 0.0, Rm = 0.0;
        if (COP) {
            Rm = mix_R<NS>(th, yi);
            T = newton_T<NS>(th, yi, tme, f.T[id]);
            p = rho * Rm * T;
            Cp = mix_Cp<NS>(th, yi, T);
            const double CopW = 1.0 / mix_W_inv<NS>(th, yi);
            const double gm = Cp / (Cp - kRu / CopW);
            gamma = gm > 1.0 ? gm : -1.0;
        } else {
            gamma = th.ncop_gamma;
            p = (th.ncop_gamma - 1.0) * rho * tme;
        }
        const double H = (U[4] + p) * rho1;
        const double c = sqrt(gamma * p * rho1);
        f.rho[id] = rho, f.u[id] = u, f.v[id] = v, f.w[id] = w, f.p[id] = p, f.H[id] = H, f.c[id] = c;
        f.e[id] = tme, f.gamma[id] = gamma;
        if (COP && f.xc) cop_cell_terms<NS>(th, yi, T, Cp, u, v, w, H, p, rho, f.xc, P, id);
        if (!COP && !XFG_STRICT_BUILD && f.sr) {  // inputs of the single-gas fast face kernel
            const double isr = rsqrt_nr(rho);
            f.isr[id] = isr;
            f.sr[id] = rho * isr;
            const double vel[3] = {u, v, w};
            const int dims[3] = {g.dimx, g.dimy, g.dimz};
#pragma unroll
            for (int d = 0; d < 3; d++)
                if (dims[d]) {
                    f.eab[d][id] = fabs(vel[d] - c);
                    f.eab[d][P + id] = fabs(vel[d]);
                    f.eab[d][2 * P + id] = fabs(vel[d] + c);
                }
        }
        if (COP) {
            f.T[id] = T, f.Cp[id] = Cp, f.R[id] = Rm;
#pragma unroll
            for (int s = 0; s < NS; s++) f.y[s * P + id] = yi[s];
        }
        // physical fluxes of the active directions
        const double Ep = U[4] + p;
        if (g.dimx) {
            double *F = f.F[0];
            F[0 * P + id] = U[1];
            F[1 * P + id] = U[1] * u + p;
            F[2 * P + id] = U[1] * v;
            F[3 * P + id] = U[1] * w;
            F[4 * P + id] = Ep * u;
#pragma unroll
            for (int n = 5; n < E; n++) F[n * P + id] = U[1] * yi[n - 5];
        }
        if (g.dimy) {
            double *F = f.F[1];
            F[0 * P + id] = U[2];
            F[1 * P + id] = U[2] * u;
            F[2 * P + id] = U[2] * v + p;
            F[3 * P + id] = U[2] * w;
            F[4 * P + id] = Ep * v;
#pragma unroll
            for (int n = 5; n < E; n++) F[n * P + id] = U[2] * yi[n - 5];
        }
        if (g.dimz) {
            double *F = f.F[2];
            F[0 * P + id] = U[3];
            F[1 * P + id] = U[3] * u;
            F[2 * P + id] = U[3] * v;
            F[3 * P + id] = U[3] * w + p;
            F[4 * P + id] = Ep * w;
#pragma unroll
            for (int n = 5; n < E; n++) F[n * P + id] = U[3] * yi[n - 5];
        }
        // inner-cell checks (rho, p, T negative / NaN / Inf; Y NaN / Inf)
        int i, j, k;
        split_index(id, g.Xmax, g.Ymax, i, j, k);
        const bool inner = i >= g.Bx && i < g.Xmax - g.Bx && j >= g.By && j < g.Ymax - g.By && k >= g.Bz && k < g.Zmax - g.Bz;
        if (inner) {
            bool e1 = rho < 0.0 || bad(rho) || p < 0.0 || bad(p) || (COP && (T < 0.0 || bad(T)));
            if (COP)
#pragma unroll
                for (int s = 0; s < NS; s++) e1 = e1 || bad(yi[s]);
            if (e1) {
                atomicOr(&f.err[ERR_PRIM], 1);
                f.err[ERR_I] = i, f.err[ERR_J] = j, f.err[ERR_K] = k;
            }
        }
        if (want_lam) {
            const double c_local = sqrt(1.4 * p / rho);
            lamx = fabs(u) + c_local, lamy = fabs(v) + c_local, lamz = fabs(w) + c_local;
            if (!(lamx >= 0.0)) lamx = __longlong_as_double(0x7ff0000000000000LL);
            if (!(lamy >= 0.0)) lamy = __longlong_as_double(0x7ff0000000000000LL);
            if (!(lamz >= 0.0)) lamz = __longlong_as_double(0x7ff0000000000000LL);
        }
    }
}

// Warp then block max of the GetDt wave speeds, one atomic per block and direction. Every thread
// of the block calls it (a block never spans two grids).
__device__ __forceinline__ void lam_block_reduce(const Geo &g, const DevFields &f, double lamx, double lamy, double lamz) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lamx = fmax(lamx, __shfl_xor_sync(0xffffffffu, lamx, o));
        lamy = fmax(lamy, __shfl_xor_sync(0xffffffffu, lamy, o));
        lamz = fmax(lamz, __shfl_xor_sync(0xffffffffu, lamz, o));
    }
    __shared__ double red[3][kThreads / 32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[0][wid] = lamx, red[1][wid] = lamy, red[2][wid] = lamz;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = red[0][0], b = red[1][0], c = red[2][0];
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) a = fmax(a, red[0][q]), b = fmax(b, red[1][q]), c = fmax(c, red[2][q]);
        if (g.dimx) atomic_max_nonneg(&f.lam[0], a);
        if (g.dimy) atomic_max_nonneg(&f.lam[1], b);
        if (g.dimz) atomic_max_nonneg(&f.lam[2], c);
    }
}

template <bool COP, int NS>
__global__ void __launch_bounds__(kThreads) k_states(Geo g, DevFields f, DevThermo th, double *__restrict__ UI,
                                                     int ghost, int want_lam, int guard) {
    if (guard && step_done(f)) return;
    double lamx = 0.0, lamy = 0.0, lamz = 0.0;
    states_body<COP, NS>(g, f, th, UI, ghost, want_lam, (long long)blockIdx.x * blockDim.x + threadIdx.x, lamx, lamy,
                         lamz);
    if (want_lam) lam_block_reduce(g, f, lamx, lamy, lamz);
}

// ---------------------------------------------------------------------------------------------
// Global LF maxima eigen_block[d][n] = max over all cells |lambda_n| (ConVenction_block.hpp:115-215)
// for WENO5 (u_d - c, u_d, u_d + c); WENO7 local eigenvalues are zero. Folded by atomicMax into
// the bit patterns glf[d*3 + {0,1,2}], which keep the maxima of all earlier calls.
// ---------------------------------------------------------------------------------------------
static __global__ void __launch_bounds__(kThreads) k_glf(Geo g, DevFields f, unsigned long long *glf, int guard) {
    if (guard && step_done(f)) return;
    const long long N = g.ncell();
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double m[9];
    for (int q = 0; q < 9; q++) m[q] = 0.0;
    if (id < N) {
        const double c = f.c[id];
        const double vel[3] = {f.u[id], f.v[id], f.w[id]};
        for (int d = 0; d < 3; d++) {
            m[3 * d + 0] = fabs(vel[d] - c);
            m[3 * d + 1] = fabs(vel[d]);
            m[3 * d + 2] = fabs(vel[d] + c);
        }
    }
    for (int q = 0; q < 9; q++) {
        double x = m[q];
        for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&glf[q], x);
    }
}

// ---------------------------------------------------------------------------------------------
// Characteristic WENO flux at face (i+1/2) of direction D, one thread per face:
// ReconstructFlux{X,Y,Z} (Reconstruction_kernels.hpp:8-199) with MARCO_ROE, MARCO_NOCOPC2 /
// MARCO_COPC2 (ReconstructSoundSpeed, Utils_device.hpp:102-140), RoeAverageLeft/Right
// (Eigen_matrix.hpp:7-455) and MARCO_FLUXWALL_WENO5 / _WENO7 (Eigen_callback.h:127-230), with
// WENO5-JS, WENO-CU6 (scheme order 6) or WENO7.
// Local eigenvalues (GetLocalEigen) are formed on the fly from u_d and c of the window cells.
// ---------------------------------------------------------------------------------------------
// The mixture's Roe-linearised sound speed (ReconstructSoundSpeed) is ill-conditioned: in smooth
// flow temp1 = dp - (dp/drho drho + dp/de de + sum dp/drho_i drho_i) is rounding noise divided by
// a sum of squared small jumps, and it corrects dp/dE, dp/drho and c^2. Its result depends on the
// rounding of every operation before it, so the mixture branch is written with round-to-nearest
// operations the compiler never contracts into an FMA (pm / pa / ps), in the reference's operation
// order; units built with --fmad=false get the same bits, and units that contract the rest of
// the face (projections, WENO, back-projection) keep this state exact. (The mixed form builds its
// own mixture Roe state, face_state_mixed in xfg_mixed.cuh.)
__device__ __forceinline__ double pm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double pa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ps(double a, double b) { return __dsub_rn(a, b); }

template <bool COP, int NS>
__device__ __forceinline__ void face_state(const Geo &g, const DevFields &f, const DevThermo &th, long long l,
                                           long long r, FaceState<NS> &F, double &Gamma0) {
    const long long P = g.pitch;
    const double rl = f.rho[l], rr = f.rho[r];
    const double ul = f.u[l], ur = f.u[r], vl = f.v[l], vr = f.v[r], wl = f.w[l], wr = f.w[r];
    const double Hl = f.H[l], Hr = f.H[r], pl = f.p[l], pr = f.p[r];
    const double D = sqrt(rr / rl);
    const double D1 = 1.0 / (D + 1.0);
    F.D = D, F.D1 = D1;
    if constexpr (!COP) {
        F._u = (ul + D * ur) * D1;
        F._v = (vl + D * vr) * D1;
        F._w = (wl + D * wr) * D1;
        F._H = (Hl + D * Hr) * D1;
        F._P = (pl + D * pr) * D1;
        F._rho = sqrt(rr * rl);
        Gamma0 = th.ncop_gamma;
        F.c2 = Gamma0 * F._P / F._rho;
        F.b1 = (Gamma0 - 1.0) / F.c2;
        F.b3 = 0.0;
        F._yi[0] = 1.0;
        F.q2 = F._u * F._u + F._v * F._v + F._w * F._w;
        F._c = sqrt(F.c2);
        F.b2 = 1.0 + F.b1 * F.q2 - F.b1 * F._H;
        F._c1 = 1.0 / F._c;
        F.ent0 = (1.0 - F.b2 - F.b3) / F.b1;
    } else {
        constexpr int NCOP = NS - 1;
        auto roe = [&](double a, double b) { return pm(pa(a, pm(D, b)), D1); };  // (a + D b) D1
        F._u = roe(ul, ur), F._v = roe(vl, vr), F._w = roe(wl, wr);
        F._H = roe(Hl, Hr), F._P = roe(pl, pr);
        F._rho = sqrt(pm(rr, rl));
        double yl[NS], yr[NS];
#pragma unroll
        for (int n = 0; n < NS; n++) {
            yl[n] = f.y[n * P + l];
            yr[n] = f.y[n * P + r];
            F._yi[n] = roe(yl[n], yr[n]);
        }
        // cell terms (cop_cell_terms, written by the states kernel of every mixture path):
        // gamma, dp/drho, e, dp/drho_i of each side
        const double *xc = f.xc;
        const double gl = xc[l], gr = xc[r];
        const double _dpdrho = roe(xc[P + l], xc[P + r]);
        const double el = xc[2 * P + l], er = xc[2 * P + r];
        double dpdrhoi[NCOP > 0 ? NCOP : 1], drhoi[NCOP > 0 ? NCOP : 1];
#pragma unroll
        for (int n = 0; n < NCOP; n++) {
            dpdrhoi[n] = roe(xc[(3 + n) * P + l], xc[(3 + n) * P + r]);
            drhoi[n] = ps(pm(rr, yr[n]), pm(rl, yl[n]));
        }
        Gamma0 = roe(gl, gr);
        const double du = ps(ur, ul), dv = ps(vr, vl), dw = ps(wr, wl);
        const double _prho = pa(pm(pa(pl / rl, pm(D, pr / rr)), D1),
                                pm(pm(pm(pm(0.5, D), D1), D1), pa(pa(pm(du, du), pm(dv, dv)), pm(dw, dw))));
        const double _dpdE = roe(ps(gl, 1.0), ps(gr, 1.0));
        const double _dpde = pm(pa(pm(ps(gl, 1.0), rl), pm(D, pm(ps(gr, 1.0), rr))), D1);
        const double dp = ps(pr, pl), drho = ps(rr, rl), de = ps(er, el);
        double S1 = 0.0, S2 = 0.0, SY = 0.0;
#pragma unroll
        for (int n = 0; n < NCOP; n++) {
            S1 = pa(S1, pm(dpdrhoi[n], drhoi[n]));
            S2 = pa(S2, pm(pm(pm(dpdrhoi[n], drhoi[n]), dpdrhoi[n]), drhoi[n]));
        }
        const double temp1 = ps(dp, pa(pa(pm(_dpdrho, drho), pm(_dpde, de)), S1));
        const double den = pa(pa(pa(pm(pm(pm(_dpdrho, _dpdrho), drho), drho), pm(pm(pm(_dpde, de), _dpde), de)), S2),
                              1e-19);
        const double temp = temp1 / den;
#pragma unroll
        for (int n = 0; n < NCOP; n++) SY = pa(SY, pm(F._yi[n], dpdrhoi[n]));
        const double _dpdE_new = pa(_dpdE, pm(pm(pm(pm(_dpdE, _dpdE), de), F._rho), temp));
        const double _dpdrho_new = pa(_dpdrho, pm(pm(pm(_dpdrho, _dpdrho), drho), temp));
        const double csqr = pa(pa(_dpdrho_new, pm(_dpdE_new, _prho)), SY);
        F.b1 = _dpdE_new / csqr;
        double b3 = 0.0;
#pragma unroll
        for (int n = 0; n < NCOP; n++) {
            const double dn = pa(dpdrhoi[n], pm(pm(pm(dpdrhoi[n], dpdrhoi[n]), drhoi[n]), temp));
            F.z[n] = -dn / _dpdE_new;
            b3 = pa(b3, pm(F._yi[n], F.z[n]));
        }
        F.b3 = pm(b3, F.b1);
        const double c2w = (0.0 < csqr) ? 0.0 : 1.0;
        F.c2 = pa(pm(pm(pm(Gamma0, F._P), F._rho), c2w), pm(ps(1.0, c2w), csqr));
        F.q2 = pa(pa(pm(F._u, F._u), pm(F._v, F._v)), pm(F._w, F._w));
        F._c = sqrt(F.c2);
        F.b2 = ps(pa(1.0, pm(F.b1, F.q2)), pm(F.b1, F._H));
        F._c1 = 1.0 / F._c;
        F.ent0 = ps(ps(1.0, F.b2), F.b3) / F.b1;
    }
}

// Single-gas Roe state of the FP64 fast path from the per-cell sqrt(rho) and 1/sqrt(rho):
// D = sqrt(rho_r/rho_l), the Roe weights, sqrt(rho_r rho_l), c^2 = gamma P/rho and the
// MARCO_PREEIGEN quantities with reciprocals instead of divisions (mathematically the same state).
__device__ __forceinline__ void face_state_fast(const DevFields &f, const DevThermo &th, long long l, long long r,
                                                FaceState<1> &F) {
    const double srl = __ldg(f.sr + l), srr = __ldg(f.sr + r);
    const double iS = rcp_nr(srl + srr);
    const double wl = srl * iS, wr = srr * iS;
    F._u = fma(wl, __ldg(f.u + l), wr * __ldg(f.u + r));
    F._v = fma(wl, __ldg(f.v + l), wr * __ldg(f.v + r));
    F._w = fma(wl, __ldg(f.w + l), wr * __ldg(f.w + r));
    F._H = fma(wl, __ldg(f.H + l), wr * __ldg(f.H + r));
    F._P = fma(wl, __ldg(f.p + l), wr * __ldg(f.p + r));
    F._rho = srl * srr;
    const double irho = __ldg(f.isr + l) * __ldg(f.isr + r);
    const double g = th.ncop_gamma;
    const double gP = g * F._P;
    F.c2 = gP * irho;
    F.b1 = ((g - 1.0) * F._rho) * rcp_nr(gP);
    F.b3 = 0.0;
    F._yi[0] = 1.0;
    F.q2 = fma(F._u, F._u, fma(F._v, F._v, F._w * F._w));
    F._c1 = rsqrt_nr(F.c2);
    F._c = F.c2 * F._c1;
    F.b2 = fma(F.b1, F.q2 - F._H, 1.0);
    F.ent0 = (1.0 - F.b2) * (F.c2 * (1.0 / (g - 1.0)));
}

// Projection of the E components of cell q onto row n of L (kinds fold at compile time).
template <int D, int E>
__device__ __forceinline__ double project(const double *lrow, int n, const double *__restrict__ A, long long P,
                                          long long q) {
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int k = 0; k < E; k++) {
        const int kind = left_kind(D, E, n, k);
        if (kind == 0) continue;
        const double x = __ldg(A + k * P + q);
        double t = kind == 1 ? x : (kind == 2 ? -x : x * lrow[k]);
        acc = first ? t : acc + t;
        first = false;
    }
    return acc;
}

// Face (i+1/2) of direction D handled by this thread. Blocks are 32 x 4 threads: 32 faces along x
// and 4 along y (D = 0, 1) or z (D = 2), so the rows of a y or z stencil are shared in L1 by the
// warps of a block. Returns false outside the face range.
template <int D>
__device__ __forceinline__ bool face_of(const Geo &g, int bx, int by, int bz, int &i, int &j, int &k) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    const int fi = bx * 32 + threadIdx.x;
    const int fj = D == 2 ? by : by * 4 + (int)threadIdx.y;
    const int fk = D == 2 ? bz * 4 + (int)threadIdx.y : bz;
    if (fi >= nfx || fj >= nfy || fk >= nfz) return false;
    i = fi + g.Bx - (D == 0 ? 1 : 0);
    j = fj + g.By - (D == 1 ? 1 : 0);
    k = fk + g.Bz - (D == 2 ? 1 : 0);
    return true;
}
template <int D>
__device__ __forceinline__ bool face_of_thread(const Geo &g, int &i, int &j, int &k) {
    return face_of<D>(g, blockIdx.x, blockIdx.y, blockIdx.z, i, j, k);
}
template <int D>
__host__ __device__ inline dim3 face_grid(const Geo &g) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    if (D == 2) return dim3((nfx + 31) / 32, nfy, (nfz + 3) / 4);
    return dim3((nfx + 31) / 32, (nfy + 3) / 4, nfz);
}

// Face of a thread of a one-dimensional block of kThreads threads read as a tile of 2^ltx faces
// along x by kThreads >> ltx faces along y (D = 0, 1) or z (D = 2); (bx, by, bz) is the tile.
template <int D>
__device__ __forceinline__ bool face_of_tile(const Geo &g, int bx, int by, int bz, int ltx, int &i, int &j, int &k) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    const int lx = (int)threadIdx.x & ((1 << ltx) - 1), ly = (int)threadIdx.x >> ltx, ty = kThreads >> ltx;
    const int fi = (bx << ltx) + lx;
    const int fj = D == 2 ? by : by * ty + ly;
    const int fk = D == 2 ? bz * ty + ly : bz;
    if (fi >= nfx || fj >= nfy || fk >= nfz) return false;
    i = fi + g.Bx - (D == 0 ? 1 : 0);
    j = fj + g.By - (D == 1 ? 1 : 0);
    k = fk + g.Bz - (D == 2 ? 1 : 0);
    return true;
}
template <int D>
__host__ __device__ inline dim3 face_grid_tile(const Geo &g, int ltx) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    const int tx = 1 << ltx, ty = kThreads >> ltx;
    if (D == 2) return dim3((nfx + tx - 1) / tx, nfy, (nfz + ty - 1) / ty);
    return dim3((nfx + tx - 1) / tx, (nfy + ty - 1) / ty, nfz);
}

// Single-gas WENO5 face of the FP64 fast path with the eigenvector products factored. For a
// single gas (b3 = 0) the rows of L (RoeAverageLeft_x/y/z) share their partial sums: with
// T.x = u x1 + v x2 + w x3 - x4, A.x = b2/2 x0 - b1/2 T.x and B.x = (un x0 - x_{D+1}) / (2c),
// row 0 is A + B, row E-1 is A - B, the entropy row D+1 is ent0 x0 + T.x and the two shear rows
// are one fused multiply-add each. The columns of R (RoeAverageRight_*) factor the same way:
// with S = fl0 + fl4, Sb = S + b1 fl_{D+1} and Dc = c (fl4 - fl0), component 0 is Sb, a velocity
// component k is vel_k Sb (+ Dc for k = D+1, +- the shear flux otherwise) and the energy is
// H Sb + un Dc - fl_{D+1} + the shear terms. The split fluxes enter WENO doubled (f +- a u,
// weno5_fast2). The same flux as the general body, with the operations regrouped.
template <int D>
__device__ __forceinline__ void faces_fast5_body(const Geo &g, const DevFields &f, const DevThermo &th,
                                                 const double *__restrict__ UI, int artificial,
                                                 const double *__restrict__ glf_d, int i, int j, int k) {
    const long long P = g.pitch;
    const long long stride = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long idl = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long idr = idl + stride;
    FaceState<1> F;
    face_state_fast(f, th, idl, idr, F);
    const double vel[3] = {F._u, F._v, F._w};
    const double un = vel[D];
    const double *__restrict__ Fl = f.F[D];
    // artificial viscosity of the acoustic fields (0, 4) and of the others (1..3)
    double a0, a1, a4;
    if (artificial == XFG_LLF) {
        const double *__restrict__ ea = f.eab[D];
        a0 = 0.0, a1 = 0.0, a4 = 0.0;
#pragma unroll
        for (int m = -2; m <= 3; m++) {
            const long long q = idl + m * stride;
            a0 = fmax(a0, __ldg(ea + q));
            a1 = fmax(a1, __ldg(ea + P + q));
            a4 = fmax(a4, __ldg(ea + 2 * P + q));
        }
    } else if (artificial == XFG_ROE) {
        a0 = fabs(un - F._c), a1 = fabs(un), a4 = fabs(un + F._c);
    } else {
        a0 = glf_d[0], a1 = glf_d[1], a4 = glf_d[2];
    }
    const double hb1 = 0.5 * F.b1, hb2 = 0.5 * F.b2, hc1 = 0.5 * F._c1, ent0 = F.ent0;
    // acoustic and entropy fields; split fluxes doubled (f +- a u), see weno5_fast2
    double p0[8], m0[8], p1[8], m1[8], p4[8], m4[8];
#pragma unroll
    for (int m = -2; m <= 3; m++) {
        const long long q = idl + m * stride;
        double pa[2][3];  // [U, F][row 0, row D+1, row 4]
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const double *__restrict__ A = a == 0 ? UI : Fl;
            const double x0 = __ldg(A + q), x1 = __ldg(A + P + q), x2 = __ldg(A + 2 * P + q);
            const double x3 = __ldg(A + 3 * P + q), x4 = __ldg(A + 4 * P + q);
            const double xd = D == 0 ? x1 : (D == 1 ? x2 : x3);
            const double t = fma(F._u, x1, fma(F._v, x2, fma(F._w, x3, -x4)));
            const double av = fma(hb2, x0, -hb1 * t);
            const double bv = hc1 * fma(un, x0, -xd);
            pa[a][0] = av + bv;
            pa[a][1] = fma(ent0, x0, t);
            pa[a][2] = av - bv;
        }
        p0[m + 3] = fma(a0, pa[0][0], pa[1][0]), m0[m + 3] = fma(-a0, pa[0][0], pa[1][0]);
        p1[m + 3] = fma(a1, pa[0][1], pa[1][1]), m1[m + 3] = fma(-a1, pa[0][1], pa[1][1]);
        p4[m + 3] = fma(a4, pa[0][2], pa[1][2]), m4[m + 3] = fma(-a4, pa[0][2], pa[1][2]);
    }
    const double fl0 = weno5_fast2(p0, m0), fl1 = weno5_fast2(p1, m1), fl4 = weno5_fast2(p4, m4);
    // shear fields: sa along the first transverse velocity, sb along the second
    // (x: v, w; y: u, w; z: u, v); row of sa: (c_a x0 + s_a x_ka), with the signs of RoeAverageLeft
    constexpr int ka = D == 0 ? 2 : 1, kb = D == 2 ? 2 : 3;
    const double va = vel[ka - 1], vb = vel[kb - 1];
    // left rows: x (v,0,-1,0,0), (-w,0,0,1,0); y (-u,1,0,0,0), (w,0,0,-1,0); z (u,-1,0,0,0), (-v,0,1,0,0)
    constexpr double sa = D == 1 ? 1.0 : -1.0, sb = D == 0 ? 1.0 : (D == 1 ? -1.0 : 1.0);
    double pa_[8], ma_[8], pb_[8], mb_[8];
#pragma unroll
    for (int m = -2; m <= 3; m++) {
        const long long q = idl + m * stride;
        const double ua = fma(-sa * va, __ldg(UI + q), sa * __ldg(UI + ka * P + q));
        const double fa = fma(-sa * va, __ldg(Fl + q), sa * __ldg(Fl + ka * P + q));
        const double ub = fma(-sb * vb, __ldg(UI + q), sb * __ldg(UI + kb * P + q));
        const double fb = fma(-sb * vb, __ldg(Fl + q), sb * __ldg(Fl + kb * P + q));
        pa_[m + 3] = fma(a1, ua, fa), ma_[m + 3] = fma(-a1, ua, fa);
        pb_[m + 3] = fma(a1, ub, fb), mb_[m + 3] = fma(-a1, ub, fb);
    }
    const double fla = weno5_fast2(pa_, ma_), flb = weno5_fast2(pb_, mb_);
    // right eigenvectors: columns of the shear fields carry sa (sb) at component ka (kb) and
    // sa va (sb vb) in the energy, as RoeAverageRight_*
    const double S = fl0 + fl4;
    const double Sb = fma(F.b1, fl1, S);
    const double Dc = F._c * (fl4 - fl0);
    double acc[5];
    acc[0] = Sb;
#pragma unroll
    for (int c = 1; c <= 3; c++) {
        if (c == D + 1) acc[c] = fma(vel[c - 1], Sb, Dc);
        else if (c == ka) acc[c] = fma(vel[c - 1], Sb, sa * fla);
        else acc[c] = fma(vel[c - 1], Sb, sb * flb);
    }
    acc[4] = fma(F._H, Sb, fma(un, Dc, fma(sa * va, fla, fma(sb * vb, flb, -fl1))));
    double *Fw = f.Fw[D];
#pragma unroll
    for (int n = 0; n < 5; n++) Fw[n * P + idl] = acc[n];
}

template <int D, bool COP, int NS, int ORDER>
__device__ __forceinline__ void faces_body(const Geo &g, const DevFields &f, const DevThermo &th,
                                           const double *__restrict__ UI, int artificial,
                                           const double *__restrict__ glf_d, int i, int j, int k) {
    using S = Sys<COP, NS>;
    constexpr int E = S::E;
    const long long P = g.pitch;
    const long long stride = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long idl = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long idr = idl + stride;

    // single-gas FP64 fast path (not in the strict units): per-cell sqrt(rho), 1/sqrt(rho) and
    // |lambda| arrays written by k_states, reciprocal-based Roe state, FMA-form WENO5
    // (a handle without those arrays gets the general form)
    constexpr bool FAST_BUILD = !COP && !XFG_STRICT_BUILD;
    const bool FAST = FAST_BUILD && f.sr && f.isr && f.eab[D];
    if constexpr (FAST_BUILD && ORDER == 5) {
        if (FAST) {
            faces_fast5_body<D>(g, f, th, UI, artificial, glf_d, i, j, k);
            return;
        }
    }
    FaceState<NS> F;
    double Gamma0;
    if (FAST_BUILD && FAST) {
        face_state_fast(f, th, idl, idr, *reinterpret_cast<FaceState<1> *>(&F));
    } else {
        face_state<COP, NS>(g, f, th, idl, idr, F, Gamma0);
    }
    const double un = D == 0 ? F._u : (D == 1 ? F._v : F._w);
    const double *__restrict__ Fl = f.F[D];
    const double *__restrict__ vd = D == 0 ? f.u : (D == 1 ? f.v : f.w);

    // LLF window maxima of |u_d - c|, |u_d|, |u_d + c| over m = -2..3 (WENO5)
    double lm0 = 0.0, lm1 = 0.0, lm2 = 0.0;
    if (ORDER != 7 && artificial == XFG_LLF) {
        if (FAST_BUILD && FAST) {
            const double *__restrict__ ea = f.eab[D];
#pragma unroll
            for (int m = -2; m <= 3; m++) {
                const long long q = idl + m * stride;
                lm0 = fmax(lm0, __ldg(ea + q));
                lm1 = fmax(lm1, __ldg(ea + P + q));
                lm2 = fmax(lm2, __ldg(ea + 2 * P + q));
            }
        } else {
#pragma unroll
            for (int m = -2; m <= 3; m++) {
                const long long q = idl + m * stride;
                const double ud = __ldg(vd + q), cc = __ldg(f.c + q);
                lm0 = fmax(lm0, fabs(ud - cc));
                lm1 = fmax(lm1, fabs(ud));
                lm2 = fmax(lm2, fabs(ud + cc));
            }
        }
    }
    constexpr int M0 = ORDER == 7 ? -3 : -2, M1 = ORDER == 7 ? 4 : 3;
    double acc[E];
#pragma unroll
    for (int n = 0; n < E; n++) {
        // mixtures across the sweep: an opaque copy of the stride per field keeps the strided
        // stencil addresses (the same for every field) from being computed once and held live
        long long stride_n = stride;
        if constexpr (COP && D != 0) asm volatile("mov.b64 %0, %0;" : "+l"(stride_n));
        const double ev = n == 0 ? fabs(un - F._c) : (n == E - 1 ? fabs(un + F._c) : fabs(un));
        double av;
        if (artificial == XFG_ROE || ORDER == 7) {
            av = ev;  // WENO7: local eigenvalues are zero, so LLF reduces to |lambda_n| of the Roe state
            if (ORDER == 7 && artificial == XFG_GLF) av = 0.0;
        } else if (artificial == XFG_LLF) {
            av = n == 0 ? lm0 : (n == E - 1 ? lm2 : lm1);
        } else {
            av = glf_d[n == 0 ? 0 : (n == E - 1 ? 2 : 1)];
        }
        double lrow[E];
#pragma unroll
        for (int kk = 0; kk < E; kk++) lrow[kk] = left_kind(D, E, n, kk) == 3 ? left_val<D, E>(F, n, kk) : 0.0;
        double pp[8], mm[8];
        const double hav = 0.5 * av;
#pragma unroll
        for (int m = M0; m <= M1; m++) {
            const long long q = idl + m * stride_n;
            const double uf = project<D, E>(lrow, n, UI, P, q);
            const double ff = project<D, E>(lrow, n, Fl, P, q);
            if constexpr (FAST_BUILD) {  // 0.5 (ff +- av uf) with one rounding, as the contracted form
                const double hff = 0.5 * ff;
                pp[m + 3] = fma(hav, uf, hff);
                mm[m + 3] = fma(-hav, uf, hff);
            } else {
                pp[m + 3] = 0.5 * (ff + av * uf);
                mm[m + 3] = 0.5 * (ff - av * uf);
            }
        }
        double fl;
        if constexpr (ORDER == 7) fl = XFG_STRICT_BUILD ? weno7(pp, mm) : weno7_prod(pp, mm);
        else if constexpr (ORDER == 6) fl = wenocu6(pp, mm, D == 0 ? g.dx : (D == 1 ? g.dy : g.dz));
        else fl = FAST_BUILD ? weno5_fast(pp, mm) : weno5(pp, mm);
#pragma unroll
        for (int kk = 0; kk < E; kk++) {
            const int kind = right_kind(D, E, n, kk);
            if (kind == 0) continue;
            const double tv = kind == 1 ? fl : (kind == 2 ? -fl : fl * right_val<D, E>(F, n, kk));
            acc[kk] = (n == 0) ? tv : acc[kk] + tv;  // column 0 of R has no structural zero
        }
    }
    double *Fw = f.Fw[D];
#pragma unroll
    for (int n = 0; n < E; n++) Fw[n * P + idl] = acc[n];
}

template <int D, bool COP, int NS, int ORDER>
__global__ void __launch_bounds__(kThreads) k_faces(Geo g, DevFields f, DevThermo th, const double *__restrict__ UI,
                                                    int artificial, const double *__restrict__ glf_d, int guard) {
    if (guard && step_done(f)) return;
    int i, j, k;
    if (!face_of_thread<D>(g, i, j, k)) return;
    faces_body<D, COP, NS, ORDER>(g, f, th, UI, artificial, glf_d, i, j, k);
}

// ---------------------------------------------------------------------------------------------
// Positivity-preserving flux limiter (PositivityPreservingKernel, FDM_Method/positive-definite_eigen/
// PositivityPreserving_kernels.hpp:5-76), one thread per inner cell i and its face i+1/2 along D,
// launched after the face sweeps (ConVenction_block.hpp:328-410). The face flux is blended toward
// the Lax-Friedrichs flux 0.5 (F_l + F_r + lambda_0 (U_l - U_r)), lambda_0 = the GetDt wave-speed
// maximum of the step along D and lambda = CFL / lambda_0, with the largest theta that keeps
// rho_l - 2 lambda F and rho_r + 2 lambda F above min(rho, 1e-13); mixtures then limit each mass
// fraction against 0 the same way. FT is the storage type of the fluxes (FP64, or FP32 in the
// mixed form); the limiter computes in FP64.
// ---------------------------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R pp_min(R a, R b) { return (b < a) ? b : a; }

template <int D, int E, int NCOP, class FT>
__device__ __forceinline__ void pp_body(const Geo &g, const double *__restrict__ UI, const FT *__restrict__ Fl,
                                        FT *__restrict__ Fw, double lambda_0, double lambda, long long t) {
    if (t >= (long long)g.Xi * g.Yi * g.Zi) return;
    const long long P = g.pitch;
    int i, j, k;
    split_index(t, g.Xi, g.Yi, i, j, k);
    i += g.Bx, j += g.By, k += g.Bz;
    const long long stride = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long l = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i, rr = l + stride;
    double F_LF[E], FF_LF[E], FF[E], Fwall[E];
#pragma unroll
    for (int n = 0; n < E; n++) {
        const double ul = UI[n * P + l], ur = UI[n * P + rr];
        F_LF[n] = 0.5 * ((double)Fl[n * P + l] + (double)Fl[n * P + rr] + lambda_0 * (ul - ur));
        FF_LF[n] = 2.0 * lambda * F_LF[n];
        Fwall[n] = (double)Fw[n * P + l];
        FF[n] = 2.0 * lambda * Fwall[n];
    }
    const double UU0 = UI[l], UP0 = UI[rr];
    double theta_u = 1.0, theta_p = 1.0;
    double rho_min = pp_min(UU0, 1.0e-13);
    if (UU0 - FF[0] < rho_min) theta_u = (UU0 - FF_LF[0] - rho_min) / (FF[0] - FF_LF[0]);
    rho_min = pp_min(UP0, 1.0e-13);
    if (UP0 + FF[0] < rho_min) theta_p = (UP0 + FF_LF[0] - rho_min) / (FF_LF[0] - FF[0]);
    double theta = pp_min(theta_u, theta_p);
#pragma unroll
    for (int n = 0; n < E; n++) {
        FF[n] = (1.0 - theta) * FF_LF[n] + theta * FF[n];
        Fwall[n] = (1.0 - theta) * F_LF[n] + theta * Fwall[n];
    }
    if (NCOP > 0) {
        const double _rhoq = 1.0 / (UU0 - FF[0]), _rhou = 1.0 / (UU0 - FF_LF[0]);
        const double _rhoqp = 1.0 / (UP0 + FF[0]), _rhoup = 1.0 / (UP0 + FF_LF[0]);
#pragma unroll
        for (int n = 0; n < NCOP; n++) {
            const int tid = n + 5;
            const double ul = UI[tid * P + l], ur = UI[tid * P + rr];
            const double yq = (ul - FF[tid]) * _rhoq, yu = (ul - FF_LF[tid]) * _rhou;
            const double yqp = (ur + FF[tid]) * _rhoqp, yup = (ur + FF_LF[tid]) * _rhoup;
            theta_u = 1.0, theta_p = 1.0;
            if (yq < 0.0) {
                const double yi_min = pp_min(yu, 0.0);
                theta_u = (yu - yi_min + 1.0e-40) / (yu - yq + 1.0e-40);
            }
            if (yqp < 0.0) {
                const double yi_min = pp_min(yup, 0.0);
                theta_p = (yup - yi_min + 1.0e-40) / (yup - yqp + 1.0e-40);
            }
            theta = pp_min(theta_u, theta_p);
#pragma unroll
            for (int nn = 0; nn < E; nn++) Fwall[nn] = (1.0 - theta) * F_LF[nn] + theta * Fwall[nn];
        }
    }
#pragma unroll
    for (int n = 0; n < E; n++) Fw[n * P + l] = (FT)Fwall[n];
}

// lam0: the step's GetDt maxima (3 doubles on the device: saved by k_dt_step, or by xfg_get_dt)
template <int D, bool COP, int NS>
__global__ void __launch_bounds__(kThreads) k_pp(Geo g, DevFields f, const double *__restrict__ UI,
                                                 const double *__restrict__ lam0, double cfl, int guard) {
    if (guard && step_done(f)) return;
    using S = Sys<COP, NS>;
    const double l0 = lam0[D];
    pp_body<D, S::E, S::NCOP, double>(g, UI, f.F[D], f.Fw[D], l0, cfl / l0,
                                      (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------------------------
// Flux divergence (UpdateFluidLU, Reconstruction_kernels.hpp:201-234) fused with the SSP-RK3
// stage (UpdateURK3rdKernel, Update_kernels.hpp:64-94) and the NaN / Inf / negative density check
// of EstimateFluidNANKernel (src/Fluids.cpp:43-86), on inner cells. store_lu keeps LU in memory.
// dt_dev != nullptr reads dt from the device (graph replay), else dt is the argument.
// ---------------------------------------------------------------------------------------------
template <int E>
__device__ __forceinline__ void div_rk_body(const Geo &g, const DevFields &f, int flag, double dt, int do_rk,
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
        double LU0 = 0.0;
        bool first = true;
        if (g.dimx) { double tt = (f.Fw[0][n * P + id - 1] - f.Fw[0][n * P + id]) * g._dx; LU0 = tt; first = false; }
        if (g.dimy) { double tt = (f.Fw[1][n * P + id - sy] - f.Fw[1][n * P + id]) * g._dy; LU0 = first ? tt : LU0 + tt; first = false; }
        if (g.dimz) { double tt = (f.Fw[2][n * P + id - sz] - f.Fw[2][n * P + id]) * g._dz; LU0 = first ? tt : LU0 + tt; first = false; }
        if (store_lu) f.LU[n * P + id] = LU0;
        if (bad(LU0)) code = 1;
        if (do_rk) {
            const long long q = n * P + id;
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
__global__ void __launch_bounds__(kThreads) k_div_rk(Geo g, DevFields f, int flag, double dt_arg,
                                                     const double *__restrict__ dt_dev, int do_rk, int store_lu,
                                                     int guard) {
    if (guard && step_done(f)) return;
    div_rk_body<E>(g, f, flag, dt_dev ? dt_dev[0] : dt_arg, do_rk, store_lu,
                   (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// SSP-RK3 stage from a stored LU (UpdateURK3rdKernel, Update_kernels.hpp:64-94), inner cells.
template <int E>
__global__ void __launch_bounds__(kThreads) k_rk(Geo g, DevFields f, int flag, double dt) {
    const long long P = g.pitch;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.Xi * g.Yi * g.Zi) return;
    int i, j, k;
    split_index(t, g.Xi, g.Yi, i, j, k);
    i += g.Bx, j += g.By, k += g.Bz;
    const long long id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
#pragma unroll
    for (int n = 0; n < E; n++) {
        const long long q = n * P + id;
        if (flag == 1) f.U1[q] = f.U[q] + dt * f.LU[q];
        else if (flag == 2) f.U1[q] = 0.75 * f.U[q] + 0.25 * f.U1[q] + 0.25 * dt * f.LU[q];
        else f.U[q] = (f.U[q] + 2.0 * f.U1[q] + 2.0 * dt * f.LU[q]) * kOT;
    }
}

// EstimateFluidNANKernel (src/Fluids.cpp:43-86) on inner cells of UI and LU: per component
// 10000 (negative density, component 0), 1100 / 1200 (NaN / Inf state), 21 / 22 (NaN / Inf LU),
// accumulated over cells; pos[E+1..E+3] the (i, j, k) of a failing cell; pos[E] the flag.
template <int E>
__global__ void __launch_bounds__(kThreads) k_estimate_nan(Geo g, const double *__restrict__ UI,
                                                           const double *__restrict__ LU, int *pos) {
    const long long P = g.pitch;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.Xi * g.Yi * g.Zi) return;
    int i, j, k;
    split_index(t, g.Xi, g.Yi, i, j, k);
    i += g.Bx, j += g.By, k += g.Bz;
    const long long id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    bool e = UI[id] < 0.0;
    if (e) atomicAdd(&pos[0], 10000);
#pragma unroll
    for (int n = 0; n < E; n++) {
        const double a = UI[n * P + id], b = LU[n * P + id];
        if (isnan(a)) atomicAdd(&pos[n], 1100), e = true;
        if (isinf(a)) atomicAdd(&pos[n], 1200), e = true;
        if (isnan(b)) atomicAdd(&pos[n], 21), e = true;
        if (isinf(b)) atomicAdd(&pos[n], 22), e = true;
    }
    if (e) {
        pos[E] = 1;
        pos[E + 1] = i, pos[E + 2] = j, pos[E + 3] = k;
    }
}

// One-thread kernel: dt = CFL / sum(lambda_d / delta_d) from the maxima of the last k_states,
// clipped to the target time as XFLUIDS::Evolution does (src/XFLUIDS.cpp:196-200); resets the
// maxima; marks the step done when the target time is reached.
__device__ __forceinline__ void dt_step_body(const Geo &g, const DevFields &f, double cfl) {
    double *b = f.dtbuf;
    if (b[4] != 0.0) return;
    const double t = b[1], target = b[2];
    if (!(t < target)) {
        b[4] = 1.0;
        b[0] = 0.0;
        return;
    }
    const double lx = __longlong_as_double((long long)f.lam[0]);
    const double ly = __longlong_as_double((long long)f.lam[1]);
    const double lz = __longlong_as_double((long long)f.lam[2]);
    const double dtref = lx * g._dx + ly * g._dy + lz * g._dz;
    double dt = cfl / dtref;
    if (t + dt > target) dt = target - t;
    b[0] = dt;
    b[1] = t + dt;
    b[3] += 1.0;
    b[5] = lx, b[6] = ly, b[7] = lz;  // lambda_0 of the positivity limiter during this step
    f.lam[0] = f.lam[1] = f.lam[2] = 0ull;
}
static __global__ void k_dt_step(Geo g, DevFields f, double cfl) { dt_step_body(g, f, cfl); }

}  // namespace XFG_KNS
}  // namespace xfg
