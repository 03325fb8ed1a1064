// xfg_inst.cuh - launchers of the kernels for one (COP, NS, arithmetic form); included by the
// instantiation units. Each unit defines XFG_KNS (its own kernel namespace) before the include and
// registers the tables it compiles:
//   xfg_inst_ncop.cu          single gas, FP64 with FMA contraction + mixed form
//   xfg_inst_ncop_strict.cu   single gas, FP64 without contraction (--fmad=false)
//   xfg_inst_cop<N>.cu        N-species mixture, FP64 without contraction (--fmad=false)
//   xfg_inst_cop<N>_mixed.cu  N-species mixture, mixed form
#pragma once

#include "xfg_fused.cuh"
#include "xfg_kernels.cuh"
#include "xfg_mixed.cuh"
#include "xfg_ops.h"
#include "xfg_viscous.cuh"

namespace xfg {
namespace XFG_KNS {

template <bool COP, int NS, bool MIXED>
struct Inst {
    static constexpr int E = Sys<COP, NS>::E;

    static void bc(const LaunchCtx &c, double *U, const double *guard) {
        const Geo &g = c.g;
        if (g.dimx) {
            long long n = (long long)g.Bx * g.Ymax * g.Zmax;
            k_bc<0, E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, U, c.bc[0], c.bc[1], guard);
        }
        if (g.dimy) {
            long long n = (long long)g.By * g.Xmax * g.Zmax;
            k_bc<1, E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, U, c.bc[2], c.bc[3], guard);
        }
        if (g.dimz) {
            long long n = (long long)g.Bz * g.Xmax * g.Ymax;
            k_bc<2, E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, U, c.bc[4], c.bc[5], guard);
        }
    }
    static void states(const LaunchCtx &c, double *UI, int want_lam, int guard) {
        const long long n = c.g.ncell();
        if (MIXED)
            k_states_mixed<COP, NS><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, c.f, c.th, UI, c.ghost, want_lam, guard);
        else
            k_states<COP, NS><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, c.f, c.th, UI, c.ghost, want_lam, guard);
    }
    template <int D, int ORDER>
    static void faces_d(const LaunchCtx &c, const double *UI, int guard) {
        const Geo &g = c.g;
        long long n = (long long)(g.Xi + (D == 0)) * (g.Yi + (D == 1)) * (g.Zi + (D == 2));
        const double *glf = c.glf ? c.glf + 3 * D : nullptr;
        (void)n;
        const dim3 grid = face_grid<D>(g), block(32, 4, 1);
        if constexpr (MIXED && !COP && ORDER == 5)
            k_faces_mixed_w5<D><<<grid, block, 0, c.st>>>(g, c.f, c.th, c.artificial, glf, guard);
        else if constexpr (MIXED)
            k_faces_mixed<D, COP, NS, ORDER><<<grid, block, 0, c.st>>>(g, c.f, c.th, c.artificial, glf, guard);
        else
            k_faces<D, COP, NS, ORDER><<<grid, block, 0, c.st>>>(g, c.f, c.th, UI, c.artificial, glf, guard);
    }
    template <int ORDER>
    static void faces(const LaunchCtx &c, int d, const double *UI, int guard) {
        if (d == 0) faces_d<0, ORDER>(c, UI, guard);
        else if (d == 1) faces_d<1, ORDER>(c, UI, guard);
        else faces_d<2, ORDER>(c, UI, guard);
    }
    static void div_rk(const LaunchCtx &c, int flag, double dt, const double *dt_dev, int do_rk, int store_lu, int guard) {
        const Geo &g = c.g;
        long long n = (long long)g.Xi * g.Yi * g.Zi;
        if (MIXED)
            k_div_rk_mixed<E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, c.f, flag, dt, dt_dev, do_rk, store_lu, guard);
        else
            k_div_rk<E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, c.f, flag, dt, dt_dev, do_rk, store_lu, guard);
    }
    static void glf(const LaunchCtx &c, unsigned long long *out, int guard) {
        // running maxima over the whole run (zeroed once when the handle is created), as the
        // reference's reductions fold in the previous eigen_block values
        if (MIXED && !COP)  // the single-gas mixed form keeps its primitives in FP32 only
            k_glf_mixed<<<grid_for(c.g.ncell(), kThreads), kThreads, 0, c.st>>>(c.g, c.f, out, guard);
        else
            k_glf<<<grid_for(c.g.ncell(), kThreads), kThreads, 0, c.st>>>(c.g, c.f, out, guard);
    }
    static void rk(const LaunchCtx &c, int flag, double dt) {
        long long n = (long long)c.g.Xi * c.g.Yi * c.g.Zi;
        k_rk<E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, c.f, flag, dt);
    }
    static void estimate_nan(const LaunchCtx &c, const double *UI, int *pos) {
        long long n = (long long)c.g.Xi * c.g.Yi * c.g.Zi;
        k_estimate_nan<E><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, UI, c.f.LU, pos);
    }

    template <int D>
    static void pp_d(const LaunchCtx &c, const double *UI, const double *lam0, int guard) {
        const long long n = (long long)c.g.Xi * c.g.Yi * c.g.Zi;
        if (MIXED)
            k_pp_mixed<D, COP, NS><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, c.f, UI, lam0, c.cfl, guard);
        else
            k_pp<D, COP, NS><<<grid_for(n, kThreads), kThreads, 0, c.st>>>(c.g, c.f, UI, lam0, c.cfl, guard);
    }
    static void pp(const LaunchCtx &c, int d, const double *UI, const double *lam0, int guard) {
        if (d == 0) pp_d<0>(c, UI, lam0, guard);
        else if (d == 1) pp_d<1>(c, UI, lam0, guard);
        else pp_d<2>(c, UI, lam0, guard);
    }

    static void visc(const LaunchCtx &c, int guard) {
        if constexpr (COP) {
            const Geo &g = c.g;
            const int heat = (c.viscous & 2) ? 1 : 0;
            const long long nd = (long long)(g.dimx ? g.Xi + 4 : 1) * (g.dimy ? g.Yi + 4 : 1) * (g.dimz ? g.Zi + 4 : 1);
            const long long nb[3] = {(long long)g.Bx * g.Ymax * g.Zmax, (long long)g.By * g.Xmax * g.Zmax,
                                     (long long)g.Bz * g.Xmax * g.Ymax};
            if constexpr (MIXED) {  // FP32 derivatives, transport and fluxes
                k_vderiv_f32<<<grid_for(nd, kThreads), kThreads, 0, c.st>>>(g, c.f, guard);
                if (g.dimx) k_vderiv_bc<0, float><<<grid_for(nb[0], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vdef, guard);
                if (g.dimy) k_vderiv_bc<1, float><<<grid_for(nb[1], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vdef, guard);
                if (g.dimz) k_vderiv_bc<2, float><<<grid_for(nb[2], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vdef, guard);
                k_transport_f32<NS><<<grid_for(nd, kThreads), kThreads, 0, c.st>>>(g, c.f, c.th, heat, guard);
            } else {
                k_vderiv<<<grid_for(nd, kThreads), kThreads, 0, c.st>>>(g, c.f, guard);
                if (g.dimx) k_vderiv_bc<0, double><<<grid_for(nb[0], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vde, guard);
                if (g.dimy) k_vderiv_bc<1, double><<<grid_for(nb[1], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vde, guard);
                if (g.dimz) k_vderiv_bc<2, double><<<grid_for(nb[2], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.vde, guard);
                k_transport<NS><<<grid_for(nd, kThreads), kThreads, 0, c.st>>>(g, c.f, c.th, heat, guard);
            }
            const long long nf[3] = {(long long)(g.Xi + 1) * g.Yi * g.Zi, (long long)g.Xi * (g.Yi + 1) * g.Zi,
                                     (long long)g.Xi * g.Yi * (g.Zi + 1)};
            if constexpr (MIXED) {
                if (g.dimx) k_visc_f32<0, E><<<grid_for(nf[0], kThreads), kThreads, 0, c.st>>>(g, c.f, heat, guard);
                if (g.dimy) k_visc_f32<1, E><<<grid_for(nf[1], kThreads), kThreads, 0, c.st>>>(g, c.f, heat, guard);
                if (g.dimz) k_visc_f32<2, E><<<grid_for(nf[2], kThreads), kThreads, 0, c.st>>>(g, c.f, heat, guard);
            } else {
                if (g.dimx) k_visc<0, E, double><<<grid_for(nf[0], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.Fw[0], heat, guard);
                if (g.dimy) k_visc<1, E, double><<<grid_for(nf[1], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.Fw[1], heat, guard);
                if (g.dimz) k_visc<2, E, double><<<grid_for(nf[2], kThreads), kThreads, 0, c.st>>>(g, c.f, c.f.Fw[2], heat, guard);
            }
        }
    }

    // the fused mixed stage (2D single gas, WENO5; fused_applies decides)
    static FusedK fused_consts(const LaunchCtx &c) {
        const double gm1 = c.th.ncop_gamma - 1.0;
        FusedK k;
        k.gamma = (float)c.th.ncop_gamma;
        k.gm1h = (float)gm1;
        k.gm1l = (float)(gm1 - (double)k.gm1h);
        k.igm1 = (float)(1.0 / gm1);
        return k;
    }
    static void fused(const LaunchCtx &c, int flag, const double *UI, const double *Uprev, double *Uout,
                      const double *dt_dev, int do_rk, int store_lu, int want_lam, int guard) {
        if constexpr (MIXED && !COP) {
            const Geo &g = c.g;
            const dim3 grid((g.Xi + fz::TX - 1) / fz::TX, (g.Yi + fz::TY - 1) / fz::TY, 1);
            const int which = UI == c.f.U ? 0 : (UI == c.f.U1 ? 1 : (UI == c.f.U2 ? 2 : -1));
            const CUtensorMap *tm = which >= 0 ? static_cast<const CUtensorMap *>(c.tmap[which]) : nullptr;
            if (tm && c.nsm > 0) {  // persistent CTAs, the state staged by TMA
                const int ntiles = (int)(grid.x * grid.y);
                const int nb = ntiles < 2 * c.nsm ? ntiles : 2 * c.nsm;
                const size_t sm = fused_tma_smem();
                if (c.artificial == XFG_LLF)
                    k_fused_stage_tma<true><<<nb, fz::THREADS, sm, c.st>>>(g, c.f, fused_consts(c), *tm, UI, Uprev, Uout,
                                                                          flag, 0.0, dt_dev, do_rk, store_lu, want_lam,
                                                                          guard, (int)grid.x, ntiles);
                else
                    k_fused_stage_tma<false><<<nb, fz::THREADS, sm, c.st>>>(g, c.f, fused_consts(c), *tm, UI, Uprev, Uout,
                                                                           flag, 0.0, dt_dev, do_rk, store_lu, want_lam,
                                                                           guard, (int)grid.x, ntiles);
                return;
            }
            const size_t smem = sizeof(FusedTile);
            if (c.artificial == XFG_LLF)
                k_fused_stage<true><<<grid, fz::THREADS, smem, c.st>>>(g, c.f, fused_consts(c), UI, Uprev, Uout, flag,
                                                                        0.0, dt_dev, do_rk, store_lu, want_lam, guard);
            else
                k_fused_stage<false><<<grid, fz::THREADS, smem, c.st>>>(g, c.f, fused_consts(c), UI, Uprev, Uout, flag,
                                                                         0.0, dt_dev, do_rk, store_lu, want_lam, guard);
        }
    }
    static int fused_prepare() {
        if constexpr (MIXED && !COP) {
            const int smem = (int)sizeof(FusedTile);
            const int smt = (int)fused_tma_smem();
            cudaError_t e = cudaFuncSetAttribute(k_fused_stage<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_fused_stage<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_fused_stage_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smt);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_fused_stage_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smt);
            return (int)e;
        }
        return 0;
    }
    static void fused_ghost_lam(const LaunchCtx &c, const double *UI, int guard) {
        if constexpr (MIXED && !COP) {
            const Geo &g = c.g;
            const long long n = fused_ghost_cells(g);
            k_fused_ghost_lam<<<grid_for(n, kThreads), kThreads, 0, c.st>>>(g, c.f, (float)c.th.ncop_gamma, UI, guard);
        }
    }

    // tables for scheme orders 5 (WENO5-JS), 6 (WENO-CU6) and 7 (WENO7), registered under
    // precision id `prec`
    static const Ops *table(int order, int prec) {
        static Ops t[3][3];
        Ops &o = t[order - 5][prec];
        const bool has_fused = MIXED && !COP && order == 5;
        o = Ops{COP ? 1 : 0, NS, order, prec, bc, states, order == 7 ? faces<7> : (order == 6 ? faces<6> : faces<5>),
                div_rk, glf, rk, estimate_nan, pp, visc, has_fused ? fused : nullptr,
                has_fused ? fused_ghost_lam : nullptr, has_fused ? fused_prepare : nullptr};
        return &o;
    }
};

// Registers, at load time, the tables of one (COP, NS, form) under the given precision ids.
template <bool COP, int NS, bool MIXED>
struct Registrar {
    explicit Registrar(std::initializer_list<int> precisions) {
        for (int prec : precisions) {
            for (int order = 5; order <= 7; order++) register_ops(Inst<COP, NS, MIXED>::table(order, prec));
        }
    }
};

// Registers only the face-sweep launchers of one mixture size under the given precision ids,
// replacing those of the tables another unit registered (this unit's compile flags apply to the
// face kernels alone).
template <bool COP, int NS>
struct FacesRegistrar {
    explicit FacesRegistrar(std::initializer_list<int> precisions) {
        using I = Inst<COP, NS, false>;
        for (int prec : precisions) {
            register_faces_override(COP ? 1 : 0, NS, 5, prec, &I::template faces<5>);
            register_faces_override(COP ? 1 : 0, NS, 6, prec, &I::template faces<6>);
            register_faces_override(COP ? 1 : 0, NS, 7, prec, &I::template faces<7>);
        }
    }
};

}  // namespace XFG_KNS
}  // namespace xfg
