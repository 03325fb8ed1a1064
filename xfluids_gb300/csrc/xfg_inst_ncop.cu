// Kernel instantiation: single gas (Emax = 5), WENO5 and WENO7; FP64 with FMA contraction and the
// mixed form.
#define XFG_KNS ncop_fast
#include "xfg_inst.cuh"
static xfg::ncop_fast::Registrar<false, 1, false> reg_fp64({XFG_FP64});
static xfg::ncop_fast::Registrar<false, 1, true> reg_mixed({XFG_MIXED});
