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

#include <cuda.h>

#include "xfg_mixed.cuh"
#include "xfg_ops.h"

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
constexpr int RAWW = 40;                   // TMA box of the state: 40 columns (an even start),
constexpr int RAWN = RH * RAWW;            // the 13 region rows,
constexpr int RAW_BYTES = 5 * RAWN * 8;    // the 5 components, FP64
static_assert(TX == 32, "one warp per tile row");
static_assert(THREADS == 8 * 32 && TY + 1 == 8, "x face rows + 1 warp, y face rows = warps");
}  // namespace fz

// Shared memory of one tile (80.3 KB): SoA per quantity, region index (r + 3) * RW + (c + 3) for
// tile row r in [-3, TY + 3) and column c in [-3, TX + 3).
struct FusedTile {
    float uh[5][fz::RC], ul[5][fz::RC];       // U = uh + ul
    float sr[fz::RC];                         // sqrt(rho)
    float vx[fz::RC], vy[fz::RC], vz[fz::RC]; // velocity
    float hh[fz::RC], pr[fz::RC], cs[fz::RC]; // total enthalpy, pressure, sound speed
    float fxh[5][fz::FXN], fxl[5][fz::FXN];   // x flux = fxh + fxl, index r * RW + (c + 3)
    float fyh[5][fz::FYN], fyl[5][fz::FYN];   // y flux, index (r + 3) * TX + c
    float2 phx[5][fz::NXF];                   // x face flux as an exact float pair, r * (TX + 1) + c
    float2 phy[5][fz::NYF];                   // y face flux as an exact float pair, r * TX + c
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
// FP64 -> float pair by the bit patterns, integer operations and two FP32 operations (no FP64
// pipe work): h keeps the sign, the exponent and the top 24 significand bits of x (truncated), l the
// next 23 bits, so h + l equals x to 2^-47 relative. |x| below 2^-126 (zeros included) gives a
// signed zero, |x| of 2^128 and above (inf, NaN included) a NaN, which the state checks report.
__device__ __forceinline__ fp2 split_d(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned ex = (hw >> 20) & 0x7ffu, sg = hw & 0x80000000u;
    const bool normal = ex - 897u < 254u;  // biased FP32 exponent ex - 896 in [1, 254]
    const unsigned hb = sg | ((ex - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
    // the low 29 bits: their top 23 as an exact float (magic-number conversion), scaled by
    // 2^(ex - 1023 - 52 + 6); below 2^-80 the scale leaves the FP32 range and l is dropped
    const float m = __uint_as_float(0x4b000000u | ((lw & 0x1fffffffu) >> 6)) - 8388608.0f;
    const float sc = __uint_as_float(ex >= 943u ? (ex - 942u) << 23 : 0u);
    const unsigned lb = __float_as_uint(m * sc) | sg;
    return {__uint_as_float(normal ? hb : (ex > 1150u ? 0x7fc00000u : sg)), __uint_as_float(normal ? lb : sg)};
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

// Packed FP32 pairs (FFMA2 / FADD2 / FMUL2: two lanes of arithmetic per instruction).
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// a - b = s + e exactly (TwoSum of a and -b) on packed pairs; fma(x, -1, y) is y - x correctly
// rounded.
__device__ __forceinline__ float2 two_diff2(float2 a, float2 b, float2 &e) {
    const float2 m1 = bc2(-1.f);
    const float2 sd = fma2(b, m1, a);   // a - b
    const float2 bv = fma2(a, m1, sd);  // s - a
    const float2 av = fma2(bv, m1, sd); // s - bv
    e = fma2(add2(b, bv), m1, fma2(av, m1, a));
    return sd;
}

// WENO5-JS of two sides (.x and .y: the plus and the minus side of a face, independent stencils
// with the same operations) on doubled inputs v = 2 (f +- a u), about the centre value v3: returns the
// weighted sum num of the candidate offsets and the weight sum den, so that the side's WENO value
// is v3 / 2 + num / den (weno5old_BODY, WENO5s_schemes.hpp:12-69: indicators 13 a^2 + 3 b^2 + 1e-6,
// here over 13 with the epsilon scaled by 4 for the doubled input; candidates q_k = v3 + r_k with
// r_1 = a_1/12 + b_1/4, r_2 = a_2/12 - b_2/4, r_3 = a_3/12 - b_3/4, halved for the doubled input).
// The weights d_k / s_k^2 are formed against the smallest indicator, d_k (s_min / s_k)^2, so that
// they lie in [0, d_k] and their sum in [0.1, 1] whatever the scale of the data.
__device__ __forceinline__ void fz_side2(float2 v1, float2 v2, float2 v3, float2 v4, float2 v5, float2 &num,
                                         float2 &den) {
    const float2 m2 = bc2(-2.f), p3 = bc2(3.f), m4 = bc2(-4.f), m1 = bc2(-1.f);
    const float2 kW = bc2(3.0f / 13.0f), kEps = bc2(4.0e-6f / 13.0f), kA = bc2(1.0f / 24.0f);
    const float2 kB = bc2(1.0f / 8.0f), kNB = bc2(-1.0f / 8.0f);
    const float2 a1 = add2(fma2(m2, v2, v1), v3);
    const float2 b1 = fma2(p3, v3, fma2(m4, v2, v1));
    const float2 s1 = fma2(a1, a1, fma2(mul2(kW, b1), b1, kEps));
    const float2 a2 = add2(fma2(m2, v3, v2), v4);
    const float2 b2 = fma2(m1, v4, v2);
    const float2 s2 = fma2(a2, a2, fma2(mul2(kW, b2), b2, kEps));
    const float2 a3 = add2(fma2(m2, v4, v3), v5);
    const float2 b3 = fma2(p3, v3, fma2(m4, v4, v5));
    const float2 s3 = fma2(a3, a3, fma2(mul2(kW, b3), b3, kEps));
    const float2 r1 = fma2(kA, a1, mul2(kB, b1)), r2 = fma2(kA, a2, mul2(kNB, b2)), r3 = fma2(kA, a3, mul2(kNB, b3));
    const float2 sm = make_float2(fminf(s1.x, fminf(s2.x, s3.x)), fminf(s1.y, fminf(s2.y, s3.y)));
    const float2 i1 = mul2(sm, make_float2(frcp_a(s1.x), frcp_a(s1.y)));
    const float2 i2 = mul2(sm, make_float2(frcp_a(s2.x), frcp_a(s2.y)));
    const float2 i3 = mul2(sm, make_float2(frcp_a(s3.x), frcp_a(s3.y)));
    const float2 w1 = mul2(mul2(bc2(0.1f), i1), i1), w2 = mul2(mul2(bc2(0.6f), i2), i2), w3 = mul2(mul2(bc2(0.3f), i3), i3);
    den = add2(add2(w1, w2), w3);
    num = fma2(w3, r3, fma2(w2, r2, mul2(w1, r1)));
}
// Face value of one characteristic field: V[k] = (plus side at offset k - 2, minus side at offset
// 3 - k) for k = 0..4, the doubled split values; the plus side reads offsets -2..2, the minus side
// offsets 3..-1 (weno5old_GPU :71-95).
__device__ __forceinline__ float fz_weno5_2(const float2 *V) {
    float2 num, den;
    fz_side2(V[0], V[1], V[2], V[3], V[4], num, den);
    return fmaf(0.5f, V[2].x + V[2].y, fmaf(num.x, den.y, num.y * den.x) * frcp_a(den.x * den.y));
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
    const float va = vel[ka - 1], vb = vel[kb - 1];
    // Stencil points in pairs (m, 5 - m), m = 0..2 (offsets m - 2 and 3 - m), every operation on
    // both points at once. A split pair (a u + f, -a u + f) of the pair gives (P_m, M_{5-m}), the
    // WENO input pair k = m; (-a u + f, a u + f) gives (M_m, P_{5-m}), swapped into the pair
    // k = 5 - m (offset 0 is not read by the minus side, offset 3 not by the plus side).
    // Shear rows are taken without their sign s (x_k - v_k x0 for s (x_k - v_k x0)): WENO is odd,
    // so the field's flux is s times the unsigned one, and s^2 = 1 in the right eigenvectors.
    float2 V0[5], V1[5], V4[5], VA[5], VB[5];
    {
        float2 uhL[5], fhL[5];
#pragma unroll
        for (int n = 0; n < 5; n++) uhL[n] = bc2(-s.uh[n][rcL]), fhL[n] = bc2(-Fh[n * FN + fL]);
        const float2 NU = bc2(-_u), NV = bc2(-_v), NW = bc2(-_w), NUN = bc2(-un), HB2 = bc2(hb2), HB1 = bc2(hb1);
        const float2 HC1 = bc2(hc1), NENT = bc2(-ent0), NVA = bc2(-va), NVB = bc2(-vb), M1 = bc2(-1.f);
        const float2 A0 = make_float2(a0, -a0), A1 = make_float2(a1, -a1), A4 = make_float2(a4, -a4);
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const int rca = rcL + (m - 2) * SU, rcb = rcL + (3 - m) * SU;
            const int fia = fL + (m - 2) * SF, fib = fL + (3 - m) * SF;
            float2 x[5], y[5];
#pragma unroll
            for (int n = 0; n < 5; n++) {
                x[n] = add2(add2(make_float2(s.uh[n][rca], s.uh[n][rcb]), uhL[n]), make_float2(s.ul[n][rca], s.ul[n][rcb]));
                y[n] = add2(add2(make_float2(Fh[n * FN + fia], Fh[n * FN + fib]), fhL[n]),
                            make_float2(Fl[n * FN + fia], Fl[n * FN + fib]));
            }
            // projections of U (0) and F (1): with mt = x4 - (u x1 + v x2 + w x3) = -T.x,
            // A = b2/2 x0 + b1/2 mt, B' = (x_{D+1} - un x0) / (2c): acoustic rows A - B', A + B';
            // the entropy row negated (mt - ent0 x0, its flux enters R with the sign folded back)
            float2 r0[2], r1[2], r4[2], ra[2], rb[2];
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const float2 *X = a == 0 ? x : y;
                const float2 mt = fma2(NU, X[1], fma2(NV, X[2], fma2(NW, X[3], X[4])));
                const float2 av = fma2(HB1, mt, mul2(HB2, X[0]));
                const float2 bv = mul2(HC1, fma2(NUN, X[0], X[D + 1]));
                r0[a] = fma2(M1, bv, av);
                r4[a] = add2(av, bv);
                r1[a] = fma2(NENT, X[0], mt);
                ra[a] = fma2(NVA, X[0], X[ka]);
                rb[a] = fma2(NVB, X[0], X[kb]);
            }
            V0[m] = fma2(A0, r0[0], r0[1]);
            V1[m] = fma2(A1, r1[0], r1[1]);
            V4[m] = fma2(A4, r4[0], r4[1]);
            VA[m] = fma2(A1, ra[0], ra[1]);
            VB[m] = fma2(A1, rb[0], rb[1]);
            if (m > 0) {
                const float2 q0 = fma2(mul2(M1, A0), r0[0], r0[1]), q1 = fma2(mul2(M1, A1), r1[0], r1[1]);
                const float2 q4 = fma2(mul2(M1, A4), r4[0], r4[1]), qa = fma2(mul2(M1, A1), ra[0], ra[1]);
                const float2 qb = fma2(mul2(M1, A1), rb[0], rb[1]);
                V0[5 - m] = make_float2(q0.y, q0.x), V1[5 - m] = make_float2(q1.y, q1.x);
                V4[5 - m] = make_float2(q4.y, q4.x), VA[5 - m] = make_float2(qa.y, qa.x);
                VB[5 - m] = make_float2(qb.y, qb.x);
            }
        }
    }
    const float fl0 = fz_weno5_2(V0), nfl1 = fz_weno5_2(V1), fl4 = fz_weno5_2(V4);  // nfl1 = -fl1
    const float fla = fz_weno5_2(VA), flb = fz_weno5_2(VB);  // unsigned shear fluxes
    // right eigenvectors (RoeAverageRight_x/y) in the factored form: S = fl0 + fl4,
    // Sb = S + b1 fl1, Dc = c (fl4 - fl0)
    const float S = fl0 + fl4;
    const float Sb = fmaf(-b1, nfl1, S);
    const float Dc = _c * (fl4 - fl0);
    out[0] = Sb;
#pragma unroll
    for (int c = 1; c <= 3; c++) {
        if (c == D + 1) out[c] = fmaf(vel[c - 1], Sb, Dc);
        else if (c == ka) out[c] = vel[c - 1] * Sb + fla;
        else out[c] = vel[c - 1] * Sb + flb;
    }
    out[4] = fmaf(_H, Sb, fmaf(un, Dc, fmaf(va, fla, fmaf(vb, flb, nfl1))));
}

// One RK stage of a 2D single-gas block, mixed form (see the file comment). UI: the stage's input
// state (ghost cells filled); Uprev: U of the step (stages 2 and 3); Uout: the stage's output
// (a buffer other than UI: the halo of a tile is another tile's output). flag 1:
// Uout = UI + dt LU; 2: Uout = 3/4 Uprev + 1/4 UI + 1/4 dt LU; 3: Uout = (Uprev + 2 UI + 2 dt LU)/3.
// store_lu keeps LU; want_lam adds the GetDt maxima of the inner cells (GlobalDt_block.hpp:31-66)
// and writes their FP32 primitives (the last UpdateFluidStates a caller can read).
// The tile (bx, by) of the block, run by one CTA of fz::THREADS threads with a FusedTile of
// dynamic shared memory; dt the stage's time step (used when do_rk). RAW: phase A reads the state
// from the shared-memory box `raw` (fz::RAWW cells per row, the tile's region starting at column
// ox, written by a TMA copy) instead of UI; after_a() is called by every thread once phase A's
// reads of it are done (the persistent kernel's next copy starts there).
struct NoHook {
    __device__ void operator()() const {}
};
template <bool LLF, bool RAW = false, class AfterA = NoHook>
__device__ __forceinline__ void fused_stage_tile(const Geo &g, const DevFields &f, const FusedK &k,
                                                 const double *__restrict__ UI, const double *__restrict__ Uprev,
                                                 double *__restrict__ Uout, int flag, double dt, int do_rk, int store_lu,
                                                 int want_lam, int bx, int by, const double *raw = nullptr, int ox = 0,
                                                 AfterA after_a = AfterA()) {
    extern __shared__ float4 fz_smem[];
    FusedTile &s = *reinterpret_cast<FusedTile *>(fz_smem);
    __shared__ float red[2][fz::THREADS / 32];
    const int x0 = bx * fz::TX, y0 = by * fz::TY;
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
        double u5[5];
        if constexpr (RAW) {
            const int q = (r + fz::HW) * fz::RAWW + (c + fz::HW + ox);
#pragma unroll
            for (int n = 0; n < 5; n++) u5[n] = raw[n * fz::RAWN + q];
        } else {
#pragma unroll
            for (int n = 0; n < 5; n++) u5[n] = UI[n * P + id];
        }
        const fp2 rho = split_d(u5[0]), mx = split_d(u5[1]), my = split_d(u5[2]);
        const fp2 mz = split_d(u5[3]), en = split_d(u5[4]);
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
    after_a();
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
                const int fL = r * fz::RW + (c + fz::HW) - 1;
                fused_face<0, LLF>(s, (r + fz::HW) * fz::RW + (c + fz::HW) - 1, fL, k, out);
#pragma unroll
                for (int n = 0; n < 5; n++) {  // the face flux fxh_L + deviation, exactly as a pair
                    float e;
                    const float h = two_sum(s.fxh[n][fL], out[n], e);
                    s.phx[n][r * (fz::TX + 1) + c] = make_float2(h, e);
                }
            }
        } else {
            r = task - fz::TY, c = lane;  // face row r: between rows r - 1 and r
            if (x0 + c < g.Xi && y0 + r <= g.Yi) {
                float out[5];
                const int fL = (r - 1 + fz::HW) * fz::TX + c;
                fused_face<1, LLF>(s, (r - 1 + fz::HW) * fz::RW + (c + fz::HW), fL, k, out);
#pragma unroll
                for (int n = 0; n < 5; n++) {
                    float e;
                    const float h = two_sum(s.fyh[n][fL], out[n], e);
                    s.phy[n][r * fz::TX + c] = make_float2(h, e);
                }
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
            const int dx_ = r * (fz::TX + 1) + c, dy_ = r * fz::TX + c;
            const float2 IH = make_float2(g.idh[0], g.idh[1]), IL = make_float2(g.idl[0], g.idl[1]);
            int code = 0;
#pragma unroll
            for (int n = 0; n < 5; n++) {
                // (Phi_{i-1/2} - Phi_{i+1/2}) / dx + (Phi_{j-1/2} - Phi_{j+1/2}) / dy, x and y packed:
                // the high difference exact (TwoSum), the low parts and its error beside it, the
                // products with 1/dx, 1/dy as float pairs; a face flux enters its two cells with
                // equal and opposite weight, so the sum over cells telescopes
                const float2 fL = s.phx[n][dx_], fR = s.phx[n][dx_ + 1];
                const float2 fB = s.phy[n][dy_], fT = s.phy[n][dy_ + fz::TX];
                float2 e;
                const float2 d = two_diff2(make_float2(fL.x, fB.x), make_float2(fR.x, fT.x), e);
                const float2 t = add2(fma2(make_float2(fR.y, fT.y), bc2(-1.f), make_float2(fL.y, fB.y)), e);
                const float2 pr = mul2(d, IH);
                const float2 pl = fma2(d, IL, fma2(t, IH, fma2(d, IH, mul2(pr, bc2(-1.f)))));
                float e2;
                const float sa = two_sum(pr.x, pr.y, e2);
                const float ca = e2 + (pl.x + pl.y);
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

template <bool LLF>
__global__ void __launch_bounds__(fz::THREADS, 2)
    k_fused_stage(Geo g, DevFields f, FusedK k, const double *__restrict__ UI, const double *__restrict__ Uprev,
                  double *__restrict__ Uout, int flag, double dt_arg, const double *__restrict__ dt_dev, int do_rk,
                  int store_lu, int want_lam, int guard) {
    if (guard && step_done(f)) return;
    fused_stage_tile<LLF>(g, f, k, UI, Uprev, Uout, flag, dt_dev ? dt_dev[0] : dt_arg, do_rk, store_lu, want_lam,
                          blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------------------------------------
// Persistent form with the state staged by TMA. Each CTA loops over tiles (t = blockIdx.x,
// + gridDim.x, ...); the FP64 state of a tile's region arrives in shared memory through one
// cp.async.bulk.tensor.3d copy (a 40 x 13 x 5 box of the handle's SoA state: x from an even
// column, y, component), signalled on an mbarrier, and the copy of the next tile starts as soon as
// phase A of the current one has read the box, so it overlaps the face sweeps and the RK stage.
// Waits are bounded: a copy that does not arrive sets the error word ERR_TMA and the CTA returns.
// ---------------------------------------------------------------------------------------------
static_assert(fz::RAWW == FUSED_BOX_X && fz::RH == FUSED_BOX_Y, "TMA box of the host-side tensor maps");

__host__ __device__ constexpr size_t fused_raw_offset() { return (sizeof(FusedTile) + 127) / 128 * 128; }
// dynamic shared memory of the TMA form: the tile, 128 bytes of slack to align the box, the box,
// the mbarrier
__host__ __device__ constexpr size_t fused_tma_smem() { return fused_raw_offset() + 128 + fz::RAW_BYTES + 16; }

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// the region of tile (bx, by) starts at column Bx + 32 bx - 3; the box at that column rounded
// down to even (16-byte aligned x coordinate), ox the offset of the region in the box
__device__ __forceinline__ int fused_box_x(const Geo &g, int bx) { return (g.Bx + bx * fz::TX - fz::HW) & ~1; }

template <bool LLF>
__global__ void __launch_bounds__(fz::THREADS, 2)
    k_fused_stage_tma(Geo g, DevFields f, FusedK k, const __grid_constant__ CUtensorMap tmap,
                      const double *__restrict__ UI, const double *__restrict__ Uprev, double *__restrict__ Uout,
                      int flag, double dt_arg, const double *__restrict__ dt_dev, int do_rk, int store_lu, int want_lam,
                      int guard, int ntx, int ntiles) {
    if (guard && step_done(f)) return;
    extern __shared__ float4 fz_smem[];
    const unsigned base = smem_u32(fz_smem);
    const unsigned box = (base + (unsigned)fused_raw_offset() + 127u) & ~127u;
    const unsigned bar = box + fz::RAW_BYTES;
    const double *raw = reinterpret_cast<const double *>(reinterpret_cast<const char *>(fz_smem) + (box - base));
    const double dt = dt_dev ? dt_dev[0] : dt_arg;
    auto issue = [&](int t) {
        const int bx = t % ntx, by = t / ntx;
        mbar_expect_tx(bar, fz::RAW_BYTES);
        tma_load_3d(box, &tmap, fused_box_x(g, bx), g.By + by * fz::TY - fz::HW, 0, bar);
    };
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the barrier, seen by the copy engine
        if ((int)blockIdx.x < ntiles) issue(blockIdx.x);
    }
    __syncthreads();
    unsigned parity = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        bool ok = false;
        for (int it = 0; it < (1 << 22) && !ok; it++) ok = mbar_try_wait(bar, parity);
        parity ^= 1u;
        if (__syncthreads_or(!ok)) {  // the same decision in every thread of the CTA
            if (threadIdx.x == 0) atomicOr(&f.err[ERR_TMA], 1);
            return;
        }
        const int bx = t % ntx, by = t / ntx, tn = t + (int)gridDim.x;
        auto next = [&]() {  // phase A has read the box: the next tile's copy may overwrite it
            if (threadIdx.x == 0 && tn < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(tn);
            }
        };
        fused_stage_tile<LLF, true>(g, f, k, UI, Uprev, Uout, flag, dt, do_rk, store_lu, want_lam, bx, by, raw,
                                    g.Bx + bx * fz::TX - fz::HW - fused_box_x(g, bx), next);
        __syncthreads();  // phase C's reads of the tile arrays before the next phase A writes them
    }
}

// Ghost cells of a 2D block: 2 By rows of Xmax cells and 2 Bx columns of the Yi inner rows.
__host__ __device__ inline long long fused_ghost_cells(const Geo &g) { return 2LL * g.By * g.Xmax + 2LL * g.Bx * g.Yi; }

// GetDt maxima and FP32 primitives of ghost cell t of a 2D block (the stage-3 fused kernel covers
// the inner cells), the FP32 recovery of k_states_mixed; every thread of the block calls it.
__device__ __forceinline__ void fused_ghost_lam_body(const Geo &g, const DevFields &f, float gamma,
                                                     const double *__restrict__ UI, long long t) {
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
static __global__ void __launch_bounds__(kThreads) k_fused_ghost_lam(Geo g, DevFields f, float gamma,
                                                                     const double *__restrict__ UI, int guard) {
    if (guard && step_done(f)) return;
    fused_ghost_lam_body(g, f, gamma, UI, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace XFG_KNS
}  // namespace xfg
