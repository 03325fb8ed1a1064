// xfg_ensemble.cuh - member table and batched kernels of the ensemble engine (xfg_ensemble.cu).
//
// One step of every active member is one sequence of batched launches: each launch covers the
// blocks of all members of that phase, a block finds its member through a prefix table of block
// offsets and runs the same device bodies as the single-grid kernels (xfg_kernels.cuh /
// xfg_mixed.cuh) on that member's arrays. The kernels are templates on the gas model (single gas or
// an NS-species mixture) and the arithmetic form; each instantiation unit compiles the forms of
// its gas model with the contraction flags of the single-grid units (mixture states, boundary
// fill and divergence without FMA contraction, their face sweeps with it) and registers their
// launchers, which the host side of the engine (xfg_ensemble.cu) looks up by (gas model, form).
#pragma once

#include "xfg_fused.cuh"
#include "xfg_kernels.cuh"
#include "xfg_mixed.cuh"
#include "xfg_ops.h"
#include "xfg_viscous.cuh"

namespace xfg {

// Device descriptor of one member.
struct EnsMember {
    Geo g;
    DevFields f;
    double cfl;
    int bc[6];
    int active;
    int ltx;    // face tile of this member: 2^ltx faces along x by kThreads >> ltx across
    int fused;  // 2D single-gas member of a mixed WENO5 LLF / Roe ensemble: its stages run as fused tiles
    int visc;   // xfg_scheme.viscous of a mixture member (0: inviscid)
    unsigned long long *glf;  // GLF running maxima (9 words in the member's small-word area)
};

// phases with a block table; PH_FALL holds three entries per member (x, y, z face sweeps of the
// fused face launch), the others one. PH_FUSED: the 32 x 7 tiles of the fused mixed stage
// (xfg_fused.cuh) of the fused members, PH_GLAM: their ghost cells' dt maxima. Viscous members:
// PH_VCELL the cells of the velocity derivatives and the transport coefficients ([B-2, inner+B+2)
// in every active direction), PH_VBC0..2 the derivatives' ghost layers, PH_VF0..2 the faces of the
// viscous fluxes.
enum {
    PH_BC0, PH_BC1, PH_BC2, PH_STATES, PH_F0, PH_F1, PH_F2, PH_DIV, PH_FALL, PH_FUSED, PH_GLAM,
    PH_VCELL, PH_VBC0, PH_VBC1, PH_VBC2, PH_VF0, PH_VF1, PH_VF2, PH_N
};

// Launchers of the per-member phases of one (gas model, form). Every launcher covers `nblk`
// blocks of the phase's table `tab` over the n members of `M` (n3 = 3 n entries for faces_all).
struct EnsOps {
    int cop, ns, precision;
    void (*bc)(const EnsMember *M, const int *tab, unsigned nblk, int n, int d, int flag, cudaStream_t st);
    void (*states)(const EnsMember *M, const int *tab, unsigned nblk, int n, const DevThermo &th, int ghost, int flag,
                   int want_lam, cudaStream_t st);
    void (*faces)(const EnsMember *M, const int *tab, unsigned nblk, int n, const DevThermo &th, int d, int order,
                  int flag, int art, cudaStream_t st);
    void (*faces_all)(const EnsMember *M, const int *tab, unsigned nblk, int n3, const DevThermo &th, int order,
                      int flag, int art, cudaStream_t st);
    void (*glf)(const EnsMember *M, const int *tab, unsigned nblk, int n, cudaStream_t st);
    void (*pp)(const EnsMember *M, const int *tab, unsigned nblk, int n, int flag, cudaStream_t st);
    void (*div_rk)(const EnsMember *M, const int *tab, unsigned nblk, int n, int flag, cudaStream_t st);
    // viscous mixtures (null for a single gas): ConVenction_block.hpp:419-566 over the members
    void (*vderiv)(const EnsMember *M, const int *tab, unsigned nblk, int n, cudaStream_t st);
    void (*vderiv_bc)(const EnsMember *M, const int *tab, unsigned nblk, int n, int d, cudaStream_t st);
    void (*transport)(const EnsMember *M, const int *tab, unsigned nblk, int n, const DevThermo &th, int heat,
                      cudaStream_t st);
    void (*visc)(const EnsMember *M, const int *tab, unsigned nblk, int n, int d, int heat, cudaStream_t st);
};

// Registry (xfg_ensemble.cu): tables per (cop, ns, precision); a face override replaces the face
// launchers of a table registered by another unit (other contraction flags).
void register_ens_ops(const EnsOps *ops);
void register_ens_faces(int cop, int ns, int precision, decltype(EnsOps::faces) faces,
                        decltype(EnsOps::faces_all) faces_all);
const EnsOps *find_ens_ops(int cop, int ns, int precision);

namespace XFG_KNS {

__device__ __forceinline__ int member_of_block(const int *__restrict__ off, int n, int b) {
    int lo = 0, hi = n;  // off[0] = 0 <= b < off[n]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool member_done(const EnsMember &m) { return m.f.dtbuf[4] != 0.0; }

// the stage input of a member: U (flag 1, or 0 before the first step), U1; a fused member's
// second stage reads U2, the first stage's output
__device__ __forceinline__ double *member_input(const EnsMember &m, int flag) {
    return flag == 1 || flag == 0 ? m.f.U : (flag == 2 && m.fused ? m.f.U2 : m.f.U1);
}

template <int D, int E>
__global__ void __launch_bounds__(kThreads) kb_bc(const EnsMember *__restrict__ M, const int *__restrict__ off, int n,
                                                  int flag) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    bc_body<D, E>(m.g, member_input(m, flag), m.bc[2 * D], m.bc[2 * D + 1], t);
}

template <bool COP, int NS, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_states(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                      int n, DevThermo th, int ghost, int flag, int want_lam) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long id = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    double *UI = member_input(m, flag);
    if constexpr (MIXED) {
        float lx = 0.f, ly = 0.f, lz = 0.f;
        states_mixed_body<COP, NS>(m.g, m.f, th, UI, ghost, want_lam, id, lx, ly, lz);
        if (want_lam) lam_block_reduce_f(m.g, m.f, lx, ly, lz);
    } else {
        double lx = 0.0, ly = 0.0, lz = 0.0;
        states_body<COP, NS>(m.g, m.f, th, UI, ghost, want_lam, id, lx, ly, lz);
        if (want_lam) lam_block_reduce(m.g, m.f, lx, ly, lz);
    }
}

template <int D, int ORDER, bool COP, int NS, bool MIXED>
__device__ __forceinline__ void member_face(const EnsMember &m, int lb, const DevThermo &th, int flag, int artificial) {
    const dim3 gd = face_grid_tile<D>(m.g, m.ltx);
    const int bx = lb % gd.x, by = (lb / gd.x) % gd.y, bz = lb / (gd.x * gd.y);
    int i, j, k;
    if (!face_of_tile<D>(m.g, bx, by, bz, m.ltx, i, j, k)) return;
    const double *glf = artificial == XFG_GLF ? (const double *)m.glf + 3 * D : nullptr;
    if constexpr (MIXED)
        faces_mixed_body<D, COP, NS, ORDER>(m.g, m.f, th, artificial, glf, i, j, k);
    else
        faces_body<D, COP, NS, ORDER>(m.g, m.f, th, member_input(m, flag), artificial, glf, i, j, k);
}

// one face sweep (direction D) of every member
template <int D, int ORDER, bool COP, int NS, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_faces(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                     int n, DevThermo th, int flag, int artificial) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    member_face<D, ORDER, COP, NS, MIXED>(m, blockIdx.x - off[mi], th, flag, artificial);
}

// all face sweeps of every member in one launch (entries 3 q + D of the table)
template <int ORDER, bool COP, int NS, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_faces_all(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                         int n3, DevThermo th, int flag, int artificial) {
    const int e = member_of_block(off, n3, blockIdx.x);
    const EnsMember &m = M[e / 3];
    if (member_done(m)) return;
    const int lb = blockIdx.x - off[e];
    switch (e % 3) {
    case 0: member_face<0, ORDER, COP, NS, MIXED>(m, lb, th, flag, artificial); break;
    case 1: member_face<1, ORDER, COP, NS, MIXED>(m, lb, th, flag, artificial); break;
    default: member_face<2, ORDER, COP, NS, MIXED>(m, lb, th, flag, artificial); break;
    }
}

// The single-gas mixed WENO5 face sweeps with registers fitted to XFG_FACES_MIXED_MINB resident
// blocks per SM, as k_faces_mixed_w5 of the single-grid path (the other forms stay unbounded).
template <int D>
__global__ void __launch_bounds__(kThreads, XFG_FACES_MIXED_MINB)
    kb_faces_m5(const EnsMember *__restrict__ M, const int *__restrict__ off, int n, DevThermo th, int flag,
                int artificial) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    member_face<D, 5, false, 1, true>(m, blockIdx.x - off[mi], th, flag, artificial);
}
template <int UNUSED>
__global__ void __launch_bounds__(kThreads, XFG_FACES_MIXED_MINB)
    kb_faces_all_m5(const EnsMember *__restrict__ M, const int *__restrict__ off, int n3, DevThermo th, int flag,
                    int artificial) {
    const int e = member_of_block(off, n3, blockIdx.x);
    const EnsMember &m = M[e / 3];
    if (member_done(m)) return;
    const int lb = blockIdx.x - off[e];
    switch (e % 3) {
    case 0: member_face<0, 5, false, 1, true>(m, lb, th, flag, artificial); break;
    case 1: member_face<1, 5, false, 1, true>(m, lb, th, flag, artificial); break;
    default: member_face<2, 5, false, 1, true>(m, lb, th, flag, artificial); break;
    }
}

template <int E, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_div_rk(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                      int n, int flag) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    if constexpr (MIXED)
        div_rk_mixed_body<E>(m.g, m.f, flag, m.f.dtbuf[0], 1, 0, t);
    else
        div_rk_body<E>(m.g, m.f, flag, m.f.dtbuf[0], 1, 0, t);
}

// positivity-preserving flux limiter (PositivityPreserving_kernels.hpp:5-76) on the face fluxes of
// every active direction of every member, with the member's wave-speed maxima of this step
// (written by kb_dt into dtbuf[5..7]); one thread per inner cell, as the divergence phase
template <bool COP, int NS, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_pp(const EnsMember *__restrict__ M, const int *__restrict__ off, int n,
                                                  int flag) {
    using S = Sys<COP, NS>;
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    const double *UI = member_input(m, flag);
    const int dims[3] = {m.g.dimx, m.g.dimy, m.g.dimz};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (!dims[d]) continue;
        const double l0 = m.f.dtbuf[5 + d];
        if constexpr (MIXED) {
            if (d == 0) pp_body<0, S::E, S::NCOP, float>(m.g, UI, m.f.Ff[0], m.f.Fwf[0], l0, m.cfl / l0, t);
            else if (d == 1) pp_body<1, S::E, S::NCOP, float>(m.g, UI, m.f.Ff[1], m.f.Fwf[1], l0, m.cfl / l0, t);
            else pp_body<2, S::E, S::NCOP, float>(m.g, UI, m.f.Ff[2], m.f.Fwf[2], l0, m.cfl / l0, t);
        } else {
            if (d == 0) pp_body<0, S::E, S::NCOP, double>(m.g, UI, m.f.F[0], m.f.Fw[0], l0, m.cfl / l0, t);
            else if (d == 1) pp_body<1, S::E, S::NCOP, double>(m.g, UI, m.f.F[1], m.f.Fw[1], l0, m.cfl / l0, t);
            else pp_body<2, S::E, S::NCOP, double>(m.g, UI, m.f.F[2], m.f.Fw[2], l0, m.cfl / l0, t);
        }
    }
}

// GLF maxima (ConVenction_block.hpp:115-215) of every member, folded into its running maxima as
// k_glf / k_glf_mixed do for a single grid: |u_d - c|, |u_d|, |u_d + c| over all cells, from the
// FP32 primitives of the single-gas mixed form (PRIMF) or the FP64 primitives
template <bool PRIMF>
__global__ void __launch_bounds__(kThreads) kb_glf(const EnsMember *__restrict__ M, const int *__restrict__ off, int n) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long id = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    const long long N = m.g.ncell(), P = m.g.pitch;
    double mx[9];
    for (int q = 0; q < 9; q++) mx[q] = 0.0;
    if (id < N) {
        const double c = PRIMF ? (double)m.f.primf[6 * P + id] : m.f.c[id];
        for (int d = 0; d < 3; d++) {
            const double v = PRIMF ? (double)m.f.primf[(1 + d) * P + id] : (d == 0 ? m.f.u[id] : (d == 1 ? m.f.v[id] : m.f.w[id]));
            mx[3 * d + 0] = fabs(v - c);
            mx[3 * d + 1] = fabs(v);
            mx[3 * d + 2] = fabs(v + c);
        }
    }
    // a block belongs to one member, so a warp's maxima are one member's
    for (int q = 0; q < 9; q++) {
        double x = mx[q];
        for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&m.glf[q], x);
    }
}

// Launchers of one (gas model, form); the table registered by Registrar, or the face launchers
// alone by FacesRegistrar.
// Viscous stress and heat conduction of the mixture members (xfg_viscous.cuh bodies, FP64 or the
// mixed form's FP32), in the single grid's order: derivatives, their ghost layers, transport
// coefficients, face fluxes.
template <bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_vderiv(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                      int n) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    if constexpr (MIXED) vderiv_f32_body(m.g, m.f, t);
    else vderiv_body(m.g, m.f, t);
}
template <int D, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_vderiv_bc(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                         int n) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    if constexpr (MIXED) vderiv_bc_body<D, float>(m.g, m.f, m.f.vdef, t);
    else vderiv_bc_body<D, double>(m.g, m.f, m.f.vde, t);
}
template <int NS, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_transport(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                         int n, DevThermo th, int heat) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    if constexpr (MIXED) transport_f32_body<NS>(m.g, m.f, th, heat, t);
    else transport_body<NS>(m.g, m.f, th, heat, t);
}
template <int D, int E, bool MIXED>
__global__ void __launch_bounds__(kThreads) kb_visc(const EnsMember *__restrict__ M, const int *__restrict__ off,
                                                    int n, int heat) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const EnsMember &m = M[mi];
    if (member_done(m)) return;
    const long long t = (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x;
    if constexpr (MIXED) visc_f32_body<D, E>(m.g, m.f, heat, t);
    else visc_body<D, E, double>(m.g, m.f, m.f.Fw[D], heat, t);
}

template <bool COP, int NS, bool MIXED>
struct EnsInst {
    static constexpr int E = Sys<COP, NS>::E;
    static void bc(const EnsMember *M, const int *tab, unsigned nb, int n, int d, int flag, cudaStream_t st) {
        if (d == 0) kb_bc<0, E><<<nb, kThreads, 0, st>>>(M, tab, n, flag);
        else if (d == 1) kb_bc<1, E><<<nb, kThreads, 0, st>>>(M, tab, n, flag);
        else kb_bc<2, E><<<nb, kThreads, 0, st>>>(M, tab, n, flag);
    }
    static void states(const EnsMember *M, const int *tab, unsigned nb, int n, const DevThermo &th, int ghost, int flag,
                       int want_lam, cudaStream_t st) {
        kb_states<COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, th, ghost, flag, want_lam);
    }
    template <int D, int ORDER>
    static void face(const EnsMember *M, const int *tab, unsigned nb, int n, const DevThermo &th, int flag, int art,
                     cudaStream_t st) {
        if constexpr (MIXED && !COP && ORDER == 5)
            kb_faces_m5<D><<<nb, kThreads, 0, st>>>(M, tab, n, th, flag, art);
        else
            kb_faces<D, ORDER, COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, th, flag, art);
    }
    template <int D>
    static void face_o(const EnsMember *M, const int *tab, unsigned nb, int n, const DevThermo &th, int order, int flag,
                       int art, cudaStream_t st) {
        if (order == 5) face<D, 5>(M, tab, nb, n, th, flag, art, st);
        else if (order == 6) face<D, 6>(M, tab, nb, n, th, flag, art, st);
        else face<D, 7>(M, tab, nb, n, th, flag, art, st);
    }
    static void faces(const EnsMember *M, const int *tab, unsigned nb, int n, const DevThermo &th, int d, int order,
                      int flag, int art, cudaStream_t st) {
        if (d == 0) face_o<0>(M, tab, nb, n, th, order, flag, art, st);
        else if (d == 1) face_o<1>(M, tab, nb, n, th, order, flag, art, st);
        else face_o<2>(M, tab, nb, n, th, order, flag, art, st);
    }
    static void faces_all(const EnsMember *M, const int *tab, unsigned nb, int n3, const DevThermo &th, int order,
                          int flag, int art, cudaStream_t st) {
        if constexpr (MIXED && !COP) {
            if (order == 5) {
                kb_faces_all_m5<0><<<nb, kThreads, 0, st>>>(M, tab, n3, th, flag, art);
                return;
            }
        }
        if (order == 5) kb_faces_all<5, COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n3, th, flag, art);
        else if (order == 6) kb_faces_all<6, COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n3, th, flag, art);
        else kb_faces_all<7, COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n3, th, flag, art);
    }
    static void glf(const EnsMember *M, const int *tab, unsigned nb, int n, cudaStream_t st) {
        kb_glf<MIXED && !COP><<<nb, kThreads, 0, st>>>(M, tab, n);
    }
    static void pp(const EnsMember *M, const int *tab, unsigned nb, int n, int flag, cudaStream_t st) {
        kb_pp<COP, NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, flag);
    }
    static void div_rk(const EnsMember *M, const int *tab, unsigned nb, int n, int flag, cudaStream_t st) {
        kb_div_rk<E, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, flag);
    }
    static void vderiv(const EnsMember *M, const int *tab, unsigned nb, int n, cudaStream_t st) {
        kb_vderiv<MIXED><<<nb, kThreads, 0, st>>>(M, tab, n);
    }
    static void vderiv_bc(const EnsMember *M, const int *tab, unsigned nb, int n, int d, cudaStream_t st) {
        if (d == 0) kb_vderiv_bc<0, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n);
        else if (d == 1) kb_vderiv_bc<1, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n);
        else kb_vderiv_bc<2, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n);
    }
    static void transport(const EnsMember *M, const int *tab, unsigned nb, int n, const DevThermo &th, int heat,
                          cudaStream_t st) {
        kb_transport<NS, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, th, heat);
    }
    static void visc(const EnsMember *M, const int *tab, unsigned nb, int n, int d, int heat, cudaStream_t st) {
        if (d == 0) kb_visc<0, E, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, heat);
        else if (d == 1) kb_visc<1, E, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, heat);
        else kb_visc<2, E, MIXED><<<nb, kThreads, 0, st>>>(M, tab, n, heat);
    }
    static const EnsOps *table(int prec) {
        static EnsOps t[3];
        if constexpr (COP)
            t[prec] = EnsOps{1, NS, prec, bc, states, faces, faces_all, glf, pp, div_rk, vderiv, vderiv_bc, transport, visc};
        else
            t[prec] = EnsOps{0, NS, prec, bc, states, faces, faces_all, glf, pp, div_rk, nullptr, nullptr, nullptr, nullptr};
        return &t[prec];
    }
};

template <bool COP, int NS, bool MIXED>
struct EnsRegistrar {
    explicit EnsRegistrar(int prec) { register_ens_ops(EnsInst<COP, NS, MIXED>::table(prec)); }
};
template <bool COP, int NS, bool MIXED>
struct EnsFacesRegistrar {
    explicit EnsFacesRegistrar(int prec) {
        register_ens_faces(COP ? 1 : 0, NS, prec, &EnsInst<COP, NS, MIXED>::faces, &EnsInst<COP, NS, MIXED>::faces_all);
    }
};

}  // namespace XFG_KNS
}  // namespace xfg
