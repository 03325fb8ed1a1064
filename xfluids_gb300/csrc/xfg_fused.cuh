// xfg_fused.cuh - the mixed-precision RK stage of a two-dimensional single-gas block as one kernel.
//
// One CTA owns a tile of 32 x 7 inner cells. It reads the stage's FP64 state once for the tile and
// a halo of three cells in x and in y (the WENO5 stencil), recovers the primitives and the physical
// fluxes of those cells into shared memory, computes every x and y face flux of the tile from
// shared memory, takes the divergence and the SSP-RK3 stage combination in FP64, and writes the
// stage's output state: the reference's UpdateFluidStates (Update_device.hpp:33-110),
// ReconstructFluxX/Y with GetLocalEigen (Reconstruction_kernels.hpp:8-133, Eigen_value.hpp:5-36),
// UpdateFluidLU (Reconstruction_kernels.hpp:201-234) and UpdateURK3rdKernel (Update_kernels.hpp:
// 64-94) in one launch per stage.
//
// Arithmetic (the mixed form's FP32 reconstruction on deviations). Every face reconstructs, in FP32,
// the deviations of its stencil values from its left cell: U_m - Uh_L and F_m - Fh_L, with Uh_L, Fh_L
// the FP32 high parts of the left cell's state and flux. WENO5 reproduces a constant shift of its
// input exactly and the single-gas eigenvectors R, L are exact inverses, so the face flux is
//     Fh_L + R WENO(L (F~ +- alpha U~) / 2)
// mathematically equal to the reference's MARCO_FLUXWALL_WENO5 (Eigen_callback.h:179-230), while
// the FP32 rounding applies to the deviations (a few cells' variation of the flow) instead of to
// the values (free-stream momentum and energy fluxes). The stencil values enter exactly: the state
// is split into FP32 high and low parts and the physical fluxes are evaluated in float-pair
// arithmetic (exact products and sums of the high parts, first-order low parts), about 2^-44 of
// the flux. The divergence differences the left cells' high fluxes and the deviation fluxes with
// error-free transformations and accumulates them as a float pair, so a face flux leaves one cell
// exactly what it brings to the next; the RK stage sum is FP64.
#pragma once

#include "xfg_mixed.cuh"

namespace xfg {
namespace XFG_KNS {

namespace fz {
constexpr int TX = 32, TY = 7, HW = 3;     // tile of inner cells, stencil halo
constexpr int RW = TX + 2 * HW;            // 38 region columns
constexpr int RH = TY + 2 * HW;            // 13 region rows
constexpr int RC = RW * RH;                // region cells (corners unused)
constexpr int FXN = TY * RW;               // x fluxes: the tile's rows, all region columns
constexpr int FYN = RH * TX;               // y fluxes: all region rows, the tile's columns
constexpr int NXF = TY * (TX + 1);         // x faces of the tile
constexpr int NYF = (TY + 1) * TX;         // y faces of the tile
constexpr int THREADS = 256;               // 8 warps
constexpr int N_INNER = TY * TX;           // phase-A items: the tile's cells (both fluxes),
constexpr int N_YHALO = 2 * HW * TX;       // the three rows below and above (y fluxes),
constexpr int N_XHALO = TY * 2 * HW;       // the three columns left and right (x fluxes)
constexpr int NITEMS = N_INNER + N_YHALO + N_XHALO;
static_assert(TX == 32, "one warp per tile row");
static_assert(THREADS == 8 * 32 && TY + 1 == 8, "x face rows + 1 warp, y face rows = warps");
}  // namespace fz

// Shared memory of one tile (70.6 KB): SoA per quantity, region index (r + 3) * RW + (c + 3) for
// tile row r in [-3, TY + 3) and column c in [-3, TX + 3).
struct FusedTile {
    float uh[5][fz::RC], ul[5][fz::RC];       // U = uh + ul
    float sr[fz::RC];                         // sqrt(rho)
    float vx[fz::RC], vy[fz::RC], vz[fz::RC]; // velocity
    float hh[fz::RC], pr[fz::RC], cs[fz::RC]; // total enthalpy, pressure, sound speed
    float fxh[5][fz::FXN], fxl[5][fz::FXN];   // x flux = fxh + fxl, index r * RW + (c + 3)
    float fyh[5][fz::FYN], fyl[5][fz::FYN];   // y flux, index (r + 3) * TX + c
    float dvx[5][fz::NXF];                    // x face flux minus the left cell's fxh, r * (TX + 1) + c
    float dvy[5][fz::NYF];                    // y face flux minus the lower cell's fyh, r * TX + c
};

// Constants of the single-gas equation of state.
struct FusedK {
    float gamma;        // NCOP_Gamma
    float gm1h, gm1l;   // gamma - 1 as a float pair
    float igm1;         // 1 / (gamma - 1)
};

// Float pair h + l (unnormalised: |l| is a few ulp of h).
struct fp2 {
    float h, l;
};
__device__ __forceinline__ fp2 split_d(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};  // x - h is exact in FP64
}
// Product: the high parts' product and its exact rounding error (FMA), plus the cross terms.
__device__ __forceinline__ fp2 mul22(fp2 a, fp2 b) {
    const float h = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.h, -h);
    return {h, fmaf(a.h, b.l, fmaf(a.l, b.h, e))};
}
// Sum: the high parts' sum and its exact rounding error (TwoSum), plus the low parts.
__device__ __forceinline__ fp2 add22(fp2 a, fp2 b) {
    float e;
    const float s = two_sum(a.h, b.h, e);
    return {s, e + (a.l + b.l)};
}
// Hardware reciprocal (within 1 ulp): the weights and the Roe state of the deviation form.
__device__ __forceinline__ float frcp_a(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// WENO5-JS of one side on doubled inputs v = 2 (f +- a u), about the centre value v3: returns the
// weighted sum num of the candidate offsets and the weight sum den, so that the side's WENO value
// is v3 / 2 + num / den (weno5old_BODY, WENO5s_schemes.hpp:12-69: indicators 13 a^2 + 3 b^2 + 1e-6,
// here over 13 with the epsilon scaled by 4 for the doubled input; candidates q_k = v3 + r_k with
// r_1 = a_1/12 + b_1/4, r_2 = a_2/12 - b_2/4, r_3 = a_3/12 - b_3/4, halved for the doubled input).
// The weights d_k / s_k^2 are formed against the smallest indicator, d_k (s_min / s_k)^2, so that
// they lie in [0, d_k] and their sum in [0.1, 1] whatever the scale of the data.
__device__ __forceinline__ void fz_side(float v1, float v2, float v3, float v4, float v5, float &num, float &den) {
    constexpr float kW = 3.0f / 13.0f, kEps = 4.0e-6f / 13.0f, kA = 1.0f / 24.0f, kB = 1.0f / 8.0f;
    const float a1 = fmaf(-2.f, v2, v1) + v3;
    const float b1 = fmaf(3.f, v3, fmaf(-4.f, v2, v1));
    const float s1 = fmaf(a1, a1, fmaf(kW * b1, b1, kEps));
    const float a2 = fmaf(-2.f, v3, v2) + v4;
    const float b2 = v2 - v4;
    const float s2 = fmaf(a2, a2, fmaf(kW * b2, b2, kEps));
    const float a3 = fmaf(-2.f, v4, v3) + v5;
    const float b3 = fmaf(3.f, v3, fmaf(-4.f, v4, v5));
    const float s3 = fmaf(a3, a3, fmaf(kW * b3, b3, kEps));
    const float r1 = fmaf(kA, a1, kB * b1), r2 = fmaf(kA, a2, -kB * b2), r3 = fmaf(kA, a3, -kB * b3);
    const float sm = fminf(s1, fminf(s2, s3));
    const float i1 = sm * frcp_a(s1), i2 = sm * frcp_a(s2), i3 = sm * frcp_a(s3);
    const float w1 = 0.1f * i1 * i1, w2 = 0.6f * i2 * i2, w3 = 0.3f * i3 * i3;
    den = w1 + w2 + w3;
    num = fmaf(w3, r3, fmaf(w2, r2, w1 * r1));
}
// Face value of one characteristic field from the doubled split values of offsets -2..3 (index
// 0..5): the plus side reads offsets -2..2, the minus side offsets 3..-1 (weno5old_GPU :71-95).
__device__ __forceinline__ float fz_weno5(const float *P, const float *M) {
    float np, dp, nm, dm;
    fz_side(P[0], P[1], P[2], P[3], P[4], np, dp);
    fz_side(M[5], M[4], M[3], M[2], M[1], nm, dm);
    return fmaf(0.5f, P[2] + M[3], fmaf(np, dm, nm * dp) * frcp_a(dp * dm));
}

// Deviation flux of one face of direction D (0 = x, 1 = y) of the tile: the face flux minus the
// left cell's high flux. rcL: region index of the left cell; fL: its index in the D flux arrays.
// The single-gas eigenvectors in the factored form of the FP64 fast face (RoeAverageLeft/Right_x/y,
// Eigen_matrix.hpp:7-305, with T.x = u x1 + v x2 + w x3 - x4 shared by the acoustic and entropy
// rows); LLF (GetLocalEigen maxima over the window m = -2..3) or Roe artificial viscosity.
template <int D, bool LLF>
__device__ __forceinline__ void fused_face(const FusedTile &s, int rcL, int fL, const FusedK &k, float out[5]) {
    constexpr int SU = D == 0 ? 1 : fz::RW, SF = D == 0 ? 1 : fz::TX, FN = D == 0 ? fz::FXN : fz::FYN;
    const float *__restrict__ Fh = D == 0 ? &s.fxh[0][0] : &s.fyh[0][0];
    const float *__restrict__ Fl = D == 0 ? &s.fxl[0][0] : &s.fyl[0][0];
    // Roe state (MARCO_ROE, global_marco.h:26-37) and MARCO_PREEIGEN with gamma P / rho
    const int rcR = rcL + SU;
    const float srl = s.sr[rcL], srr = s.sr[rcR];
    const float iS = frcp_a(srl + srr);
    const float wl = srl * iS, wr = srr * iS;
    const float _u = fmaf(wl, s.vx[rcL], wr * s.vx[rcR]);
    const float _v = fmaf(wl, s.vy[rcL], wr * s.vy[rcR]);
    const float _w = fmaf(wl, s.vz[rcL], wr * s.vz[rcR]);
    const float _H = fmaf(wl, s.hh[rcL], wr * s.hh[rcR]);
    const float _P = fmaf(wl, s.pr[rcL], wr * s.pr[rcR]);
    const float _rho = srl * srr;
    const float c2 = k.gamma * _P * frcp_a(_rho);
    const float b1 = k.gm1h * frcp_a(c2);
    const float q2 = fmaf(_u, _u, fmaf(_v, _v, _w * _w));
    const float _c1 = rsqrtf(c2);
    const float _c = c2 * _c1;
    const float b2 = fmaf(b1, q2 - _H, 1.0f);
    const float ent0 = (1.0f - b2) * c2 * k.igm1;
    const float vel[3] = {_u, _v, _w};
    const float un = vel[D];
    // artificial viscosity of the acoustic fields (a0, a4) and of the others (a1)
    float a0, a1, a4;
    if constexpr (LLF) {
        const float *__restrict__ vd = D == 0 ? s.vx : s.vy;
        a0 = 0.f, a1 = 0.f, a4 = 0.f;
#pragma unroll
        for (int m = -2; m <= 3; m++) {
            const float ud = vd[rcL + m * SU], cc = s.cs[rcL + m * SU];
            a0 = fmaxf(a0, fabsf(ud - cc));
            a1 = fmaxf(a1, fabsf(ud));
            a4 = fmaxf(a4, fabsf(ud + cc));
        }
    } else {
        a0 = fabsf(un - _c), a1 = fabsf(un), a4 = fabsf(un + _c);
    }
    const float hb1 = 0.5f * b1, hb2 = 0.5f * b2, hc1 = 0.5f * _c1;
    // shear fields: along v and w (x faces), along u and w (y faces), with the signs of
    // RoeAverageLeft: x (v, 0, -1, 0, 0), (-w, 0, 0, 1, 0); y (-u, 1, 0, 0, 0), (w, 0, 0, -1, 0)
    constexpr int ka = D == 0 ? 2 : 1, kb = 3;
    constexpr float sa = D == 1 ? 1.f : -1.f, sb = D == 0 ? 1.f : -1.f;
    const float va = vel[ka - 1], vb = vel[kb - 1];
    float uhL[5], fhL[5];
#pragma unroll
    for (int n = 0; n < 5; n++) uhL[n] = s.uh[n][rcL], fhL[n] = Fh[n * FN + fL];
    float P0[6], M0[6], P1[6], M1[6], P4[6], M4[6], PA[6], MA[6], PB[6], MB[6];
#pragma unroll
    for (int m = 0; m < 6; m++) {
        const int rc = rcL + (m - 2) * SU, fi = fL + (m - 2) * SF;
        float x[5], y[5];
#pragma unroll
        for (int n = 0; n < 5; n++) {
            x[n] = (s.uh[n][rc] - uhL[n]) + s.ul[n][rc];
            y[n] = (Fh[n * FN + fi] - fhL[n]) + Fl[n * FN + fi];
        }
        float pa[2][3];
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const float *X = a == 0 ? x : y;
            const float t = fmaf(_u, X[1], fmaf(_v, X[2], fmaf(_w, X[3], -X[4])));
            const float av = fmaf(hb2, X[0], -hb1 * t);
            const float bv = hc1 * fmaf(un, X[0], -X[D + 1]);
            pa[a][0] = av + bv;
            pa[a][1] = fmaf(ent0, X[0], t);
            pa[a][2] = av - bv;
        }
        P0[m] = fmaf(a0, pa[0][0], pa[1][0]), M0[m] = fmaf(-a0, pa[0][0], pa[1][0]);
        P1[m] = fmaf(a1, pa[0][1], pa[1][1]), M1[m] = fmaf(-a1, pa[0][1], pa[1][1]);
        P4[m] = fmaf(a4, pa[0][2], pa[1][2]), M4[m] = fmaf(-a4, pa[0][2], pa[1][2]);
        const float ua = fmaf(-sa * va, x[0], sa * x[ka]), fa = fmaf(-sa * va, y[0], sa * y[ka]);
        const float ub = fmaf(-sb * vb, x[0], sb * x[kb]), fb = fmaf(-sb * vb, y[0], sb * y[kb]);
        PA[m] = fmaf(a1, ua, fa), MA[m] = fmaf(-a1, ua, fa);
        PB[m] = fmaf(a1, ub, fb), MB[m] = fmaf(-a1, ub, fb);
    }
    const float fl0 = fz_weno5(P0, M0), fl1 = fz_weno5(P1, M1), fl4 = fz_weno5(P4, M4);
    const float fla = fz_weno5(PA, MA), flb = fz_weno5(PB, MB);
    // right eigenvectors (RoeAverageRight_x/y) in the factored form: S = fl0 + fl4,
    // Sb = S + b1 fl1, Dc = c (fl4 - fl0)
    const float S = fl0 + fl4;
    const float Sb = fmaf(b1, fl1, S);
    const float Dc = _c * (fl4 - fl0);
    out[0] = Sb;
#pragma unroll
    for (int c = 1; c <= 3; c++) {
        if (c == D + 1) out[c] = fmaf(vel[c - 1], Sb, Dc);
        else if (c == ka) out[c] = fmaf(vel[c - 1], Sb, sa * fla);
        else out[c] = fmaf(vel[c - 1], Sb, sb * flb);
    }
    out[4] = fmaf(_H, Sb, fmaf(un, Dc, fmaf(sa * va, fla, fmaf(sb * vb, flb, -fl1))));
}

// One RK stage of a 2D single-gas block, mixed form (see the file comment). UI: the stage's input
// state (ghost cells filled); Uprev: U of the step (stages 2 and 3); Uout: the stage's output
// (a buffer other than UI: the halo of a tile is another tile's output). flag 1:
// Uout = UI + dt LU; 2: Uout = 3/4 Uprev + 1/4 UI + 1/4 dt LU; 3: Uout = (Uprev + 2 UI + 2 dt LU)/3.
// store_lu keeps LU; want_lam adds the GetDt maxima of the inner cells (GlobalDt_block.hpp:31-66)
// and writes their FP32 primitives (the last UpdateFluidStates a caller can read).
template <bool LLF>
__global__ void __launch_bounds__(fz::THREADS, 2)
    k_fused_stage(Geo g, DevFields f, FusedK k, const double *__restrict__ UI, const double *__restrict__ Uprev,
                  double *__restrict__ Uout, int flag, double dt_arg, const double *__restrict__ dt_dev, int do_rk,
                  int store_lu, int want_lam, int guard) {
    if (guard && step_done(f)) return;
    extern __shared__ float4 fz_smem[];
    FusedTile &s = *reinterpret_cast<FusedTile *>(fz_smem);
    __shared__ float red[2][fz::THREADS / 32];
    const int x0 = blockIdx.x * fz::TX, y0 = blockIdx.y * fz::TY;
    const long long P = g.pitch;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // ---- phase A: states and physical fluxes of the tile and its halo ----------------------------
    float lamx = 0.f, lamy = 0.f;
#pragma unroll 1
    for (int it = tid; it < fz::NITEMS; it += fz::THREADS) {
        int r, c, kind;  // kind bit 0: x flux, bit 1: y flux
        if (it < fz::N_INNER) {
            r = it >> 5, c = it & 31, kind = 3;
        } else if (it < fz::N_INNER + fz::N_YHALO) {
            const int q = it - fz::N_INNER, rr = q >> 5;
            r = rr < fz::HW ? rr - fz::HW : rr - fz::HW + fz::TY, c = q & 31, kind = 2;
        } else {
            const int q = it - fz::N_INNER - fz::N_YHALO;
            r = q / (2 * fz::HW);
            const int cc = q - 2 * fz::HW * r;
            c = cc < fz::HW ? cc - fz::HW : cc - fz::HW + fz::TX, kind = 1;
        }
        const int i = g.Bx + x0 + c, j = g.By + y0 + r;
        if (i >= g.Xmax || j >= g.Ymax) continue;
        const long long id = (long long)j * g.Xmax + i;
        const fp2 rho = split_d(UI[id]), mx = split_d(UI[P + id]), my = split_d(UI[2 * P + id]);
        const fp2 mz = split_d(UI[3 * P + id]), en = split_d(UI[4 * P + id]);
        // 1 / rho as a pair: r0 the rounded reciprocal, 1 - rho r0 its exact residual
        const float r0 = __frcp_rn(rho.h);
        const float re = fmaf(-rho.l, r0, fmaf(-rho.h, r0, 1.0f));
        const fp2 ri = {r0, r0 * re};
        const fp2 u = mul22(mx, ri), v = mul22(my, ri), w = mul22(mz, ri);
        const fp2 mu = mul22(mx, u), nv = mul22(my, v), ow = mul22(mz, w);
        const fp2 q = add22(add22(mu, nv), ow);                       // rho |u|^2
        const fp2 ei = add22(en, fp2{-0.5f * q.h, -0.5f * q.l});      // rho e
        const fp2 p = mul22(ei, fp2{k.gm1h, k.gm1l});
        const fp2 ep = add22(en, p);                                  // E + p
        const float pf = p.h + p.l, rf = rho.h + rho.l;
        const float uf = u.h + u.l, vf = v.h + v.l, wf = w.h + w.l;
        const float Hf = (ep.h + ep.l) * r0, cf = sqrtf(k.gamma * pf * r0);
        const int rc = (r + fz::HW) * fz::RW + (c + fz::HW);
        s.uh[0][rc] = rho.h, s.ul[0][rc] = rho.l;
        s.uh[1][rc] = mx.h, s.ul[1][rc] = mx.l;
        s.uh[2][rc] = my.h, s.ul[2][rc] = my.l;
        s.uh[3][rc] = mz.h, s.ul[3][rc] = mz.l;
        s.uh[4][rc] = en.h, s.ul[4][rc] = en.l;
        s.sr[rc] = sqrtf(rf);
        s.vx[rc] = uf, s.vy[rc] = vf, s.vz[rc] = wf;
        s.hh[rc] = Hf, s.pr[rc] = pf, s.cs[rc] = cf;
        if (kind & 1) {  // GetPhysFlux x: (m, m u + p, m v, m w, (E + p) u)
            const int fi = r * fz::RW + (c + fz::HW);
            const fp2 F1 = add22(mu, p), F2 = mul22(mx, v), F3 = mul22(mx, w), F4 = mul22(ep, u);
            s.fxh[0][fi] = mx.h, s.fxl[0][fi] = mx.l;
            s.fxh[1][fi] = F1.h, s.fxl[1][fi] = F1.l;
            s.fxh[2][fi] = F2.h, s.fxl[2][fi] = F2.l;
            s.fxh[3][fi] = F3.h, s.fxl[3][fi] = F3.l;
            s.fxh[4][fi] = F4.h, s.fxl[4][fi] = F4.l;
        }
        if (kind & 2) {  // GetPhysFlux y: (n, n u, n v + p, n w, (E + p) v)
            const int fi = (r + fz::HW) * fz::TX + c;
            const fp2 G1 = mul22(my, u), G2 = add22(nv, p), G3 = mul22(my, w), G4 = mul22(ep, v);
            s.fyh[0][fi] = my.h, s.fyl[0][fi] = my.l;
            s.fyh[1][fi] = G1.h, s.fyl[1][fi] = G1.l;
            s.fyh[2][fi] = G2.h, s.fyl[2][fi] = G2.l;
            s.fyh[3][fi] = G3.h, s.fyl[3][fi] = G3.l;
            s.fyh[4][fi] = G4.h, s.fyl[4][fi] = G4.l;
        }
        if (kind == 3 && x0 + c < g.Xi && y0 + r < g.Yi) {  // an inner cell of the block
            if (!(rf >= 0.f) || !(pf >= 0.f) || isinf(rf) || isinf(pf)) {
                atomicOr(&f.err[ERR_PRIM], 1);
                f.err[ERR_I] = i, f.err[ERR_J] = j, f.err[ERR_K] = 0;
            }
            if (want_lam) {
                const float cl = sqrtf(1.4f * pf * r0);
                lamx = fmaxf(lamx, fabsf(uf) + cl), lamy = fmaxf(lamy, fabsf(vf) + cl);
                if (!(lamx >= 0.f)) lamx = __int_as_float(0x7f800000);
                if (!(lamy >= 0.f)) lamy = __int_as_float(0x7f800000);
                float *pf_out = f.primf;
                pf_out[id] = rf, pf_out[P + id] = uf, pf_out[2 * P + id] = vf, pf_out[3 * P + id] = wf;
                pf_out[4 * P + id] = Hf, pf_out[5 * P + id] = pf, pf_out[6 * P + id] = cf;
            }
        }
    }
    if (want_lam) {  // block maxima of the GetDt wave speeds, one atomic per direction
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lamx = fmaxf(lamx, __shfl_xor_sync(0xffffffffu, lamx, o));
            lamy = fmaxf(lamy, __shfl_xor_sync(0xffffffffu, lamy, o));
        }
        if (lane == 0) red[0][warp] = lamx, red[1][warp] = lamy;
    }
    __syncthreads();
    if (want_lam && tid == 0) {
        float a = red[0][0], b = red[1][0];
        for (int q = 1; q < fz::THREADS / 32; q++) a = fmaxf(a, red[0][q]), b = fmaxf(b, red[1][q]);
        atomic_max_nonneg(&f.lam[0], (double)a);
        atomic_max_nonneg(&f.lam[1], (double)b);
    }

    // ---- phase B: face fluxes. Sixteen warp tasks over two rounds: x faces of rows 0..6 (the
    // left faces of columns 0..31), y faces of face rows 0..7 (the lower faces of rows 0..7), and
    // the x faces right of column 31 (one lane per row). One call site per direction, so a face
    // shared with the neighbouring tile gets the same instructions there and the same bits.
#pragma unroll 1
    for (int task = warp; task < 16; task += 8) {
        const bool xface = task < fz::TY || task == 15;
        int r, c;
        if (xface) {
            r = task < fz::TY ? task : lane, c = task < fz::TY ? lane : fz::TX;
            if (r < fz::TY && x0 + c <= g.Xi && y0 + r < g.Yi) {
                float out[5];
                fused_face<0, LLF>(s, (r + fz::HW) * fz::RW + (c + fz::HW) - 1, r * fz::RW + (c + fz::HW) - 1, k, out);
#pragma unroll
                for (int n = 0; n < 5; n++) s.dvx[n][r * (fz::TX + 1) + c] = out[n];
            }
        } else {
            r = task - fz::TY, c = lane;  // face row r: between rows r - 1 and r
            if (x0 + c < g.Xi && y0 + r <= g.Yi) {
                float out[5];
                fused_face<1, LLF>(s, (r - 1 + fz::HW) * fz::RW + (c + fz::HW), (r - 1 + fz::HW) * fz::TX + c, k, out);
#pragma unroll
                for (int n = 0; n < 5; n++) s.dvy[n][r * fz::TX + c] = out[n];
            }
        }
    }
    __syncthreads();

    // ---- phase C: divergence and RK stage of the tile's cells ------------------------------------
    if (tid < fz::N_INNER) {
        const int r = tid >> 5, c = tid & 31;
        if (x0 + c < g.Xi && y0 + r < g.Yi) {
            const int i = g.Bx + x0 + c, j = g.By + y0 + r;
            const long long id = (long long)j * g.Xmax + i;
            const double dt = dt_dev ? dt_dev[0] : dt_arg;
            const int fxc = r * fz::RW + (c + fz::HW), fyc = (r + fz::HW) * fz::TX + c;
            const int dx_ = r * (fz::TX + 1) + c, dy_ = r * fz::TX + c;
            int code = 0;
#pragma unroll
            for (int n = 0; n < 5; n++) {
                // (Phi_{i-1/2} - Phi_{i+1/2}) / dx with Phi = the left cell's high flux + deviation
                float sa = 0.f, ca = 0.f;
                div_acc(s.fxh[n][fxc - 1], s.fxh[n][fxc], g.idh[0], g.idl[0], sa, ca);
                div_acc(s.dvx[n][dx_], s.dvx[n][dx_ + 1], g.idh[0], g.idl[0], sa, ca);
                div_acc(s.fyh[n][fyc - fz::TX], s.fyh[n][fyc], g.idh[1], g.idl[1], sa, ca);
                div_acc(s.dvy[n][dy_], s.dvy[n][dy_ + fz::TX], g.idh[1], g.idl[1], sa, ca);
                const double LU0 = f2d_bits(sa) + f2d_bits(ca);
                const long long q = n * P + id;
                if (store_lu) f.LU[q] = LU0;
                if (!isfinite(sa)) code = 1;
                if (do_rk) {
                    double out;
                    if (flag == 1) out = UI[q] + dt * LU0;
                    else if (flag == 2) out = 0.75 * Uprev[q] + 0.25 * UI[q] + 0.25 * dt * LU0;
                    else out = (Uprev[q] + 2.0 * UI[q] + 2.0 * dt * LU0) * kOT;
                    Uout[q] = out;
                    if (bad(out) || (n == 0 && out < 0.0)) code = 1;
                }
            }
            if (code) {
                atomicOr(&f.err[ERR_STATE], 1);
                f.err[ERR_I] = i, f.err[ERR_J] = j, f.err[ERR_K] = 0;
            }
        }
    }
}

// GetDt maxima and FP32 primitives of the ghost cells of a 2D block (the stage-3 fused kernel
// covers the inner cells): one thread per ghost cell, the FP32 recovery of k_states_mixed.
static __global__ void __launch_bounds__(kThreads) k_fused_ghost_lam(Geo g, DevFields f, float gamma,
                                                                     const double *__restrict__ UI, int guard) {
    if (guard && step_done(f)) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)g.By * g.Xmax, sides = 2LL * g.Bx * g.Yi;
    float lamx = 0.f, lamy = 0.f;
    if (t < 2 * rows + sides) {
        int i, j;
        if (t < rows) j = (int)(t / g.Xmax), i = (int)(t % g.Xmax);
        else if (t < 2 * rows) j = g.Ymax - g.By + (int)((t - rows) / g.Xmax), i = (int)((t - rows) % g.Xmax);
        else {
            const long long q = t - 2 * rows;
            j = g.By + (int)(q / (2 * g.Bx));
            const int cc = (int)(q % (2 * g.Bx));
            i = cc < g.Bx ? cc : g.Xmax - 2 * g.Bx + cc;
        }
        const long long P = g.pitch, id = (long long)j * g.Xmax + i;
        const float rho = (float)UI[id], rho1 = 1.0f / rho;
        const float u = (float)UI[P + id] * rho1, v = (float)UI[2 * P + id] * rho1, w = (float)UI[3 * P + id] * rho1;
        const float E = (float)UI[4 * P + id];
        const float p = (gamma - 1.0f) * (E - 0.5f * rho * (u * u + v * v + w * w));
        const float c = sqrtf(gamma * p * rho1);
        float *pf = f.primf;
        pf[id] = rho, pf[P + id] = u, pf[2 * P + id] = v, pf[3 * P + id] = w;
        pf[4 * P + id] = (E + p) * rho1, pf[5 * P + id] = p, pf[6 * P + id] = c;
        const float cl = sqrtf(1.4f * p * rho1);
        lamx = fabsf(u) + cl, lamy = fabsf(v) + cl;
        if (!(lamx >= 0.f)) lamx = __int_as_float(0x7f800000);
        if (!(lamy >= 0.f)) lamy = __int_as_float(0x7f800000);
    }
    lam_block_reduce_f(g, f, lamx, lamy, 0.f);
}

}  // namespace XFG_KNS
}  // namespace xfg
