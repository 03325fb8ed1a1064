// Kernel instantiation: mixture of 6 species (Emax = 10), WENO5 and WENO7, FP64 compiled without
// contraction (--fmad=false); serves both FP64 precision ids.
#define XFG_KNS cop6_strict
#include "xfg_inst.cuh"
static xfg::cop6_strict::Registrar<true, 6, false> reg_fp64({XFG_FP64, XFG_FP64_STRICT});
