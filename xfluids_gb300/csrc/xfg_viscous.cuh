// xfg_viscous.cuh - fourth-order viscous, heat-conduction and diffusion fluxes of a mixture
// (Visc / Visc_Heat / Visc_Diffu), subtracted from the face fluxes after the convective sweeps
// (and the positivity limiter), as ConVenction_block.hpp:419-566 does:
//   k_vderiv        GetInnerCellCenterDerivativeKernel (Fourth_Order/Visc_Order_kernels.hpp:16-72)
//   k_vderiv_bc<D>  CenterDerivativeBCKernel{X,Y,Z} (viscosity/Visc_kernels.hpp:7-204)
//   k_transport     Gettransport_coeff_aver (Visc_kernels.hpp:226-245, Visc_device.h)
//   k_visc<D>       GetWallViscousFlux{X,Y,Z} (Fourth_Order/Visc_Order_kernels.hpp:74-342)
// Mass diffusion: a single block's diffusion limiter is Dim_max = 0 (ConVenction_block.hpp:457-503
// reduces only the mass-fraction range; the Dkm range is reset to 1 by the MPI build alone), so
// the clamped diffusion flux Dim_Yil and with it every diffusion term is zero; the kernels take
// the viscous stress and heat conduction and leave the diffusion terms out.
#pragma once

#include "xfg_kernels.cuh"

namespace xfg {
namespace XFG_KNS {

enum { V_DUCX, V_DVCX, V_DWCX, V_DUCY, V_DVCY, V_DWCY, V_DUCZ, V_DVCZ, V_DWCZ };
constexpr double kVTwle = 1.0 / 12.0, kVTwfr = 1.0 / 24.0, kVSxtn = 1.0 / 16.0;

// Each kernel below is a device body (one thread's work, t its index in the launch) and a
// single-grid wrapper; the ensemble engine runs the same bodies per member (xfg_ensemble.cuh).

// device transport table (doubles): visc[NS*4], therm[NS*4], wa[NS*NS] = (W_j/W_k)^0.25,
// wb[NS*NS] = (1 + W_k/W_j)^-0.5, sid[NS]; offsets for a given NS
struct TrView {
    const double *visc, *therm, *wa, *wb, *sid;
    __device__ TrView(const double *t, int ns)
        : visc(t), therm(t + 4 * ns), wa(t + 8 * ns), wb(t + 8 * ns + ns * ns), sid(t + 8 * ns + 2 * ns * ns) {}
};

// one thread per cell of [B-2, inner+B+2) in every active direction
__device__ __forceinline__ void vderiv_body(const Geo &g, const DevFields &f, long long t) {
    const int r0[3] = {g.dimx ? g.Bx - 2 : 0, g.dimy ? g.By - 2 : 0, g.dimz ? g.Bz - 2 : 0};
    const int nx = g.dimx ? g.Xi + 4 : 1, ny = g.dimy ? g.Yi + 4 : 1, nz = g.dimz ? g.Zi + 4 : 1;
    if (t >= (long long)nx * ny * nz) return;
    const int i = (int)(t % nx) + r0[0];
    const long long r = t / nx;
    const int j = (int)(r % ny) + r0[1], k = (int)(r / ny) + r0[2];
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long st[3] = {1, (long long)g.Xmax, (long long)g.Xmax * g.Ymax};
    const int dims[3] = {g.dimx, g.dimy, g.dimz};
    const double inv[3] = {g._dx, g._dy, g._dz};
    const double dt[3] = {(double)g.dimx, (double)g.dimy, (double)g.dimz};
    const double *vel[3] = {f.u, f.v, f.w};
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double val = 0.0;
            if (dims[d]) {
                const double *q = vel[c];
                val = (8.0 * (q[id + st[d]] - q[id - st[d]]) - (q[id + 2 * st[d]] - q[id - 2 * st[d]])) * inv[d] * kVTwle *
                      dt[d];
                if (c != d) val = val * dt[c];
            }
            f.vde[(3 * d + c) * P + id] = val;
        }
}
static __global__ void __launch_bounds__(kThreads) k_vderiv(Geo g, DevFields f, int guard) {
    if (guard && step_done(f)) return;
    vderiv_body(g, f, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// The mixed form's derivatives: the same fourth-order differences in FP32 from the form's FP32
// velocities (primf components 1..3), written as FP32.
__device__ __forceinline__ void vderiv_f32_body(const Geo &g, const DevFields &f, long long t) {
    const int r0[3] = {g.dimx ? g.Bx - 2 : 0, g.dimy ? g.By - 2 : 0, g.dimz ? g.Bz - 2 : 0};
    const int nx = g.dimx ? g.Xi + 4 : 1, ny = g.dimy ? g.Yi + 4 : 1, nz = g.dimz ? g.Zi + 4 : 1;
    if (t >= (long long)nx * ny * nz) return;
    const int i = (int)(t % nx) + r0[0];
    const long long r = t / nx;
    const int j = (int)(r % ny) + r0[1], k = (int)(r / ny) + r0[2];
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long st[3] = {1, (long long)g.Xmax, (long long)g.Xmax * g.Ymax};
    const int dims[3] = {g.dimx, g.dimy, g.dimz};
    const float inv[3] = {(float)(g._dx * kVTwle), (float)(g._dy * kVTwle), (float)(g._dz * kVTwle)};
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float val = 0.f;
            if (dims[d] && (c == d || dims[c])) {
                const float *q = f.primf + (1 + c) * P;
                val = (8.f * (q[id + st[d]] - q[id - st[d]]) - (q[id + 2 * st[d]] - q[id - 2 * st[d]])) * inv[d];
            }
            f.vdef[(3 * d + c) * P + id] = val;
        }
}
static __global__ void __launch_bounds__(kThreads) k_vderiv_f32(Geo g, DevFields f, int guard) {
    if (guard && step_done(f)) return;
    vderiv_f32_body(g, f, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ghost layers of direction D: the four derivative components its flux reads
template <int D, class VT>
__device__ __forceinline__ void vderiv_bc_body(const Geo &g, const DevFields &f, VT *__restrict__ vde, long long t) {
    const int bw = D == 0 ? g.Bx : (D == 1 ? g.By : g.Bz);
    const int inner = D == 0 ? g.Xi : (D == 1 ? g.Yi : g.Zi);
    const int nmax = D == 0 ? g.Xmax : (D == 1 ? g.Ymax : g.Zmax);
    const int ta = D == 0 ? g.Ymax : g.Xmax, tb = D == 2 ? g.Ymax : g.Zmax;
    if (t >= (long long)bw * ta * tb) return;
    const int gl = (int)(t % bw);
    const long long r = t / bw;
    const int a = (int)(r % ta), b = (int)(r / ta);
    const long long P = g.pitch;
    constexpr int c0 = D == 0 ? V_DUCY : (D == 1 ? V_DVCX : V_DWCX);
    constexpr int c1 = D == 0 ? V_DUCZ : (D == 1 ? V_DVCZ : V_DWCY);
    constexpr int c2 = D == 0 ? V_DVCY : V_DUCX;
    constexpr int c3 = D == 2 ? V_DVCY : V_DWCZ;
    const int comps[4] = {c0, c1, c2, c3};
    auto cell = [&](int cn) {
        const int i = D == 0 ? cn : a, j = D == 0 ? a : (D == 1 ? cn : b), k = D == 2 ? cn : b;
        return (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    };
    for (int side = 0; side < 2; side++) {
        const int BC = g.bc[2 * D + side];
        const int cn = side == 0 ? gl : gl + nmax - bw;
        const int mirror_offset = side == 0 ? 0 : inner;
        const int index_inner = side == 0 ? bw : nmax - bw - 1;
        const int sign = side == 0 ? 1 : -1;
        const long long id = cell(cn);
        long long src = -1;
        bool neg = false;
        switch (BC) {
        case XFG_SYMMETRY: src = cell(2 * (bw + mirror_offset) - 1 - cn); break;
        case XFG_PERIODIC: src = cell(cn + sign * inner); break;
        case XFG_OUTFLOW: src = cell(index_inner); break;
        case XFG_NSLIPWALL:  // the mirror of X and Y (the reference's Z case indexes outside the array)
            src = cell(2 * (bw + mirror_offset) - 1 - cn), neg = true;
            break;
        case XFG_INFLOW:
#pragma unroll
            for (int m = 0; m < 4; m++) vde[comps[m] * P + id] = VT(0);
            break;
        default: break;
        }
        if (src >= 0)
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const VT v = vde[comps[m] * P + src];
                vde[comps[m] * P + id] = neg ? -v : v;
            }
    }
}
template <int D, class VT>
__global__ void __launch_bounds__(kThreads) k_vderiv_bc(Geo g, DevFields f, VT *__restrict__ vde, int guard) {
    if (guard && step_done(f)) return;
    vderiv_bc_body<D, VT>(g, f, vde, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// mixture viscosity (Wilke) and thermal conductivity on the cells k_visc reads: [B-2, inner+B+2)
// in every active direction. Per cell one ln T, NS viscosity fits, and the Wilke weights
// PHI_ki = W_ki^a (mu_k / mu_i)^(1/2) ... (Visc_device.h:30-38) with (mu_k / mu_i)^(1/2) formed as
// sqrt(mu_k) * (1 / sqrt(mu_i)): NS square roots and reciprocals instead of NS^2 pow calls, a
// difference of a few ulp (the fits themselves go through exp and log).
template <int NS>
__device__ __forceinline__ void transport_body(const Geo &g, const DevFields &f, const DevThermo &th, int heat,
                                               long long t) {
    const int nx = g.dimx ? g.Xi + 4 : 1, ny = g.dimy ? g.Yi + 4 : 1, nz = g.dimz ? g.Zi + 4 : 1;
    if (t >= (long long)nx * ny * nz) return;
    const int i0 = (int)(t % nx) + (g.dimx ? g.Bx - 2 : 0);
    const long long r = t / nx;
    const int j0 = (int)(r % ny) + (g.dimy ? g.By - 2 : 0), k0 = (int)(r / ny) + (g.dimz ? g.Bz - 2 : 0);
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k0 + (long long)g.Xmax * j0 + i0;
    const TrView tv(f.tr, NS);
    const double T = f.T[id], rho = f.rho[id];
    const double lT = log(T);
    double X[NS], mk[NS], sq[NS], isq[NS];
    double C_total = 0.0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
        X[i] = f.y[i * P + id] * th._Wi[i] * 1e-3 * rho;
        C_total = C_total + X[i];
    }
    const double _C = 1.0 / C_total;
#pragma unroll
    for (int i = 0; i < NS; i++) X[i] = X[i] * _C;
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const double *c = tv.visc + 4 * (int)tv.sid[k];
        mk[k] = exp(((c[3] * lT + c[2]) * lT + c[1]) * lT + c[0]);
        sq[k] = sqrt(mk[k]);
        isq[k] = 1.0 / sq[k];
    }
    const double s2 = sqrt(2.0);
    double mu = 0.0, kap = 0.0;
#pragma unroll
    for (int k = 0; k < NS; k++) {
        double den = 0.0;
#pragma unroll
        for (int i = 0; i < NS; i++) {
            double phi = tv.wa[k * NS + i] * (sq[k] * isq[i]);
            phi = (phi + 1.0) * (phi + 1.0) * 0.5 / s2;
            phi = phi * tv.wb[k * NS + i];
            den = den + X[i] * phi;
        }
        const double _den = 1.0 / den;
        mu = mu + X[k] * mk[k] * _den;
        if (heat) {
            const double *c = tv.therm + 4 * (int)tv.sid[k];
            kap = kap + X[k] * exp(((c[3] * lT + c[2]) * lT + c[1]) * lT + c[0]) * _den;
        }
    }
    f.mu[id] = mu;
    if (heat) f.kappa[id] = kap;
}
template <int NS>
__global__ void __launch_bounds__(kThreads) k_transport(Geo g, DevFields f, DevThermo th, int heat, int guard) {
    if (guard && step_done(f)) return;
    transport_body<NS>(g, f, th, heat, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// The mixed form's transport: the same sums in FP32 (mu and kappa to ~1e-6 relative; the fits lose
// about one decade to cancellation), from the FP32 table trf (species resolved, PHI's constant
// 0.5 / sqrt(2) folded into wb), written as FP32 for k_visc_f32.
template <int NS>
__device__ __forceinline__ void transport_f32_body(const Geo &g, const DevFields &f, const DevThermo &th, int heat,
                                                   long long t) {
    const int nx = g.dimx ? g.Xi + 4 : 1, ny = g.dimy ? g.Yi + 4 : 1, nz = g.dimz ? g.Zi + 4 : 1;
    if (t >= (long long)nx * ny * nz) return;
    const int i0 = (int)(t % nx) + (g.dimx ? g.Bx - 2 : 0);
    const long long r = t / nx;
    const int j0 = (int)(r % ny) + (g.dimy ? g.By - 2 : 0), k0 = (int)(r / ny) + (g.dimz ? g.Bz - 2 : 0);
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k0 + (long long)g.Xmax * j0 + i0;
    const float *visc = f.trf, *therm = f.trf + 4 * NS, *wa = f.trf + 8 * NS, *wb = f.trf + 8 * NS + NS * NS;
    const float lT = logf((float)f.T[id]);
    const double rho = f.rho[id];
    float X[NS], mk[NS], sq[NS], isq[NS];
    float C_total = 0.0f;
#pragma unroll
    for (int i = 0; i < NS; i++) {
        X[i] = (float)(f.y[i * P + id] * rho) * (float)(th._Wi[i] * 1e-3);
        C_total += X[i];
    }
    const float _C = 1.0f / C_total;
#pragma unroll
    for (int i = 0; i < NS; i++) X[i] *= _C;
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const float *c = visc + 4 * k;
        mk[k] = expf(((c[3] * lT + c[2]) * lT + c[1]) * lT + c[0]);
        sq[k] = sqrtf(mk[k]);
        isq[k] = 1.0f / sq[k];
    }
    float mu = 0.0f, kap = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; k++) {
        float den = 0.0f;
#pragma unroll
        for (int i = 0; i < NS; i++) {
            const float q = wa[k * NS + i] * (sq[k] * isq[i]) + 1.0f;
            den += X[i] * (q * q * wb[k * NS + i]);
        }
        const float _den = 1.0f / den;
        mu += X[k] * mk[k] * _den;
        if (heat) {
            const float *c = therm + 4 * k;
            kap += X[k] * expf(((c[3] * lT + c[2]) * lT + c[1]) * lT + c[0]) * _den;
        }
    }
    f.muf[id] = mu;
    if (heat) f.kappaf[id] = kap;
}
template <int NS>
__global__ void __launch_bounds__(kThreads) k_transport_f32(Geo g, DevFields f, DevThermo th, int heat, int guard) {
    if (guard && step_done(f)) return;
    transport_f32_body<NS>(g, f, th, heat, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// viscous stress and heat-conduction flux at the faces i+1/2 of direction D, subtracted from the
// FP64 face fluxes (the mixed form runs k_visc_f32)
template <int D, int E, class FT>
__device__ __forceinline__ void visc_body(const Geo &g, const DevFields &f, FT *__restrict__ Fw, int heat, long long t) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    if (t >= (long long)nfx * nfy * nfz) return;
    const int i = (int)(t % nfx) + g.Bx - (D == 0 ? 1 : 0);
    const long long r = t / nfx;
    const int j = (int)(r % nfy) + g.By - (D == 1 ? 1 : 0), k = (int)(r / nfy) + g.Bz - (D == 2 ? 1 : 0);
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long st = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long m1 = id - st, p1 = id + st, p2 = id + 2 * st;
    const double _dl = D == 0 ? g._dx : (D == 1 ? g._dy : g._dz);
    const double dt[3] = {(double)g.dimx, (double)g.dimy, (double)g.dimz};
    const double *vel[3] = {f.u, f.v, f.w};
    auto half = [&](const double *a) { return (9.0 * (a[p1] + a[id]) - (a[p2] + a[m1])) * kVSxtn; };
    auto b27 = [&](const double *a) { return 27.0 * (a[p1] - a[id]) - (a[p2] - a[m1]); };
    auto vd = [&](int c, long long q) { return f.vde[c * P + q]; };
    const double mue = half(f.mu);
    const double lamada = -2.0 * kOT * mue;
    double fv[3], hv[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c == D) {
            const int oa = c == 0 ? V_DVCY : V_DUCX, ob = c == 2 ? V_DVCY : V_DWCZ;
            fv[c] = (2.0 * mue + lamada) * b27(vel[c]) * _dl * kVTwfr;
            fv[c] += lamada *
                     (9.0 * (vd(oa, p1) + vd(oa, id)) - (vd(oa, p2) + vd(oa, m1)) + 9.0 * (vd(ob, p1) + vd(ob, id)) -
                      (vd(ob, p2) + vd(ob, m1))) *
                     kVSxtn;
            hv[c] = half(vel[c]);
        } else {
            const int cr = 3 * c + D;  // derivative of u_D along x_c
            fv[c] = mue * b27(vel[c]) * _dl * kVTwfr * dt[c];
            fv[c] += mue * (9.0 * (vd(cr, p1) + vd(cr, id)) - (vd(cr, p2) + vd(cr, m1))) * kVSxtn * dt[c];
            hv[c] = half(vel[c]) * dt[c];
        }
    }
    double F4 = fv[0] * hv[0] + fv[1] * hv[1] + fv[2] * hv[2];
    if (heat) {
        double kk = half(f.kappa);
        kk *= b27(f.T) * _dl * kVTwfr;
        F4 += kk;
    }
    Fw[1 * P + id] = (FT)((double)Fw[1 * P + id] - fv[0]);
    Fw[2 * P + id] = (FT)((double)Fw[2 * P + id] - fv[1]);
    Fw[3 * P + id] = (FT)((double)Fw[3 * P + id] - fv[2]);
    Fw[4 * P + id] = (FT)((double)Fw[4 * P + id] - F4);
    // component 0 and the species: minus zero (the reference subtracts 0.0 and the zero diffusion)
}
template <int D, int E, class FT>
__global__ void __launch_bounds__(kThreads) k_visc(Geo g, DevFields f, FT *__restrict__ Fw, int heat, int guard) {
    if (guard && step_done(f)) return;
    visc_body<D, E, FT>(g, f, Fw, heat, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// The mixed form's viscous and heat-conduction face flux: k_visc's terms in FP32 from the form's
// FP32 velocities (primf), derivatives, mu, kappa and T, subtracted from the FP32 face fluxes.
// FP32 rounding of u (~6e-8 |u|) moves the stress by far less than the FP32 convective flux's own
// rounding.
template <int D, int E>
__device__ __forceinline__ void visc_f32_body(const Geo &g, const DevFields &f, int heat, long long t) {
    const int nfx = g.Xi + (D == 0 ? 1 : 0), nfy = g.Yi + (D == 1 ? 1 : 0), nfz = g.Zi + (D == 2 ? 1 : 0);
    if (t >= (long long)nfx * nfy * nfz) return;
    const int i = (int)(t % nfx) + g.Bx - (D == 0 ? 1 : 0);
    const long long r = t / nfx;
    const int j = (int)(r % nfy) + g.By - (D == 1 ? 1 : 0), k = (int)(r / nfy) + g.Bz - (D == 2 ? 1 : 0);
    const long long P = g.pitch, id = (long long)g.Xmax * g.Ymax * k + (long long)g.Xmax * j + i;
    const long long st = D == 0 ? 1 : (D == 1 ? (long long)g.Xmax : (long long)g.Xmax * g.Ymax);
    const long long m1 = id - st, p1 = id + st, p2 = id + 2 * st;
    const float _dl24 = (float)((D == 0 ? g._dx : (D == 1 ? g._dy : g._dz)) * kVTwfr);
    const float dt[3] = {(float)g.dimx, (float)g.dimy, (float)g.dimz};
    const float *vel[3] = {f.primf + P, f.primf + 2 * P, f.primf + 3 * P};
    constexpr float s16 = (float)kVSxtn;
    auto half = [&](const float *a) { return (9.f * (a[p1] + a[id]) - (a[p2] + a[m1])) * s16; };
    auto b27 = [&](const float *a) { return 27.f * (a[p1] - a[id]) - (a[p2] - a[m1]); };
    auto vh = [&](int c) {  // 16 x the face value of derivative component c
        const float *a = f.vdef + c * P;
        return 9.f * (a[p1] + a[id]) - (a[p2] + a[m1]);
    };
    const float mue = half(f.muf);
    const float lamada = -2.f * (float)kOT * mue;
    float fv[3], hv[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c == D) {
            const int oa = c == 0 ? V_DVCY : V_DUCX, ob = c == 2 ? V_DVCY : V_DWCZ;
            fv[c] = (2.f * mue + lamada) * b27(vel[c]) * _dl24 + lamada * (vh(oa) + vh(ob)) * s16;
            hv[c] = half(vel[c]);
        } else {
            const int cr = 3 * c + D;  // derivative of u_D along x_c
            fv[c] = (mue * b27(vel[c]) * _dl24 + mue * vh(cr) * s16) * dt[c];
            hv[c] = half(vel[c]) * dt[c];
        }
    }
    float F4 = fv[0] * hv[0] + fv[1] * hv[1] + fv[2] * hv[2];
    if (heat) F4 += half(f.kappaf) * b27(f.Tf) * _dl24;
    float *Fw = f.Fwf[D];
    Fw[1 * P + id] -= fv[0];
    Fw[2 * P + id] -= fv[1];
    Fw[3 * P + id] -= fv[2];
    Fw[4 * P + id] -= F4;
}
template <int D, int E>
__global__ void __launch_bounds__(kThreads) k_visc_f32(Geo g, DevFields f, int heat, int guard) {
    if (guard && step_done(f)) return;
    visc_f32_body<D, E>(g, f, heat, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace XFG_KNS
}  // namespace xfg
