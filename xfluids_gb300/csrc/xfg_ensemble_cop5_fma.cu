// Batched kernels of 5-species mixture ensembles compiled with floating-point contraction: the
// face sweeps of the FP64 form (registered over the table of xfg_ensemble_cop5.cu, as the
// single-grid path contracts its mixture face sweeps) and every kernel of the mixed form.
#define XFG_KNS ens_cop5_fma
#include "xfg_ensemble.cuh"
static xfg::ens_cop5_fma::EnsFacesRegistrar<true, 5, false> reg_fp64_faces(XFG_FP64);
static xfg::ens_cop5_fma::EnsRegistrar<true, 5, true> reg_mixed(XFG_MIXED);
