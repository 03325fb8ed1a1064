// Batched kernels of 5-species mixture ensembles, FP64 form, compiled without floating-point
// contraction (as the single-grid mixture units): boundary fill, primitive recovery with the
// temperature Newton iteration, the positivity limiter and the divergence + RK stage, and the
// face sweeps of the strict arithmetic (also used, as in the single-grid path, when the positivity
// limiter is on). The contracted face sweeps of the FP64 form are in xfg_ensemble_cop5_fma.cu.
#define XFG_KNS ens_cop5
#include "xfg_ensemble.cuh"
static xfg::ens_cop5::EnsRegistrar<true, 5, false> reg_fp64(XFG_FP64);
static xfg::ens_cop5::EnsRegistrar<true, 5, false> reg_strict(XFG_FP64_STRICT);
