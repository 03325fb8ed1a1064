// Kernel instantiation: single gas (Emax = 5), WENO5 and WENO7, FP64 compiled without contraction
// (--fmad=false), the operation sequence of the reference's CPU build.
#define XFG_KNS ncop_strict
#include "xfg_inst.cuh"
static xfg::ncop_strict::Registrar<false, 1, false> reg_strict({XFG_FP64_STRICT});
