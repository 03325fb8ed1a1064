// xfg_ops.h - host-side table of kernel launchers, one table per compiled (COP, NS, order).
// The API (xfg_api.cu) picks the table for a handle at creation; each instantiation unit
// (xfg_inst_*.cu) fills the tables of its species count.
#pragma once

#include <cuda_runtime.h>

#include <initializer_list>
#include <vector>

#include "xfg_device.cuh"

namespace xfg {

// box of the fused stage's TMA copy of the state (columns, rows; all 5 components)
constexpr int FUSED_BOX_X = 40, FUSED_BOX_Y = 13;

struct LaunchCtx {
    Geo g;
    DevFields f;
    DevThermo th;
    cudaStream_t st;
    int artificial;                    // Artificial_type
    int ghost;                         // GhostSpecies
    int bc[6];
    const double *glf;                 // GLF maxima per direction (9 doubles) or nullptr
    int precision;                     // xfg_precision
    double cfl;                        // CFLnumber (positivity limiter)
    int viscous;                       // xfg_scheme.viscous
    // fused mixed stage staged by TMA: host copies of the CUtensorMap of the state buffers U, U1,
    // U2 (null when the block's row pitch does not allow a tensor map), and the SM count
    const void *tmap[3];
    int nsm;
};

struct Ops {
    int cop, ns, order;
    int precision;                     // xfg_precision the table serves
    void (*bc)(const LaunchCtx &, double *U, const double *guard);
    void (*states)(const LaunchCtx &, double *UI, int want_lam, int guard);
    void (*faces)(const LaunchCtx &, int d, const double *UI, int guard);
    void (*div_rk)(const LaunchCtx &, int flag, double dt, const double *dt_dev, int do_rk, int store_lu, int guard);
    void (*glf)(const LaunchCtx &, unsigned long long *out, int guard);
    void (*rk)(const LaunchCtx &, int flag, double dt);
    void (*estimate_nan)(const LaunchCtx &, const double *UI, int *pos);
    void (*pp)(const LaunchCtx &, int d, const double *UI, const double *lam0, int guard);
    void (*visc)(const LaunchCtx &, int guard);   // viscous and heat-conduction fluxes (mixtures)
    // Fused RK stage of a 2D single-gas block in the mixed form (xfg_fused.cuh): states, face
    // fluxes, divergence and the stage combination in one launch; null in the other tables.
    void (*fused)(const LaunchCtx &, int flag, const double *UI, const double *Uprev, double *Uout,
                  const double *dt_dev, int do_rk, int store_lu, int want_lam, int guard);
    // GetDt maxima (and FP32 primitives) of the ghost cells, beside the stage-3 fused launch.
    void (*fused_ghost_lam)(const LaunchCtx &, const double *UI, int guard);
    // Shared-memory attribute of the fused kernels (called once at handle creation, outside any
    // stream capture); returns a CUDA error code.
    int (*fused_prepare)();
};

// Whether a handle of this block and scheme runs the fused mixed stage: two active directions
// x and y, single gas, WENO5, LLF or Roe, no positivity limiter.
inline bool fused_applies(const xfg_block &b, const xfg_scheme &s, const Ops *ops) {
    return ops && ops->fused && b.DimX && b.DimY && !b.DimZ && !s.cop && s.precision == XFG_MIXED &&
           s.scheme_order == 5 && (s.artificial_type == XFG_LLF || s.artificial_type == XFG_ROE) && !s.positivity &&
           !s.viscous;
}

// Message returned by xfg_last_error() on this host thread.
void set_last_error(const char *msg);

// Checks of a block, scheme and thermal set that every entry point taking them shares: scheme
// switches in range, Bwidth against the scheme's stencil, consistent sizes, the face launches'
// grid limits. Returns 0 or -1 with the message set.
int validate_block_scheme(const xfg_block *b, const xfg_scheme *s, const xfg_thermal *t);

// Device transport tables of a viscous mixture from the caller's fits (xfg_transport), shared by
// xfg_set_transport and xfg_ensemble_set_transport: FP64 t = visc[4 ns], therm[4 ns],
// wa[ns ns] = (W_i / W_k)^0.25, wb[ns ns] = (1 + W_k / W_i)^-0.5, sid[ns]; FP32 tf = the same with
// the species resolved through sid and wb scaled by 0.5 / sqrt(2). Returns 0, or -1 with the error
// text set.
int pack_transport(const xfg_transport *tr, int ns, std::vector<double> &t, std::vector<float> &tf);

// Registry filled by the instantiation units.
const Ops *find_ops(int cop, int ns, int order, int precision);
void register_ops(const Ops *ops);
// Face-sweep launcher from another instantiation unit (other compile flags) that replaces the
// `faces` entry of the table registered under the same key.
using FacesFn = void (*)(const LaunchCtx &, int d, const double *UI, int guard);
void register_faces_override(int cop, int ns, int order, int precision, FacesFn faces);

inline unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace xfg
