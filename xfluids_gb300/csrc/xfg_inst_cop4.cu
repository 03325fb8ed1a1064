// Kernel instantiation: mixture of 4 species (Emax = 8), WENO5 and WENO7, FP64 compiled without
// contraction (--fmad=false); serves both FP64 precision ids.
#define XFG_KNS cop4_strict
#include "xfg_inst.cuh"
static xfg::cop4_strict::Registrar<true, 4, false> reg_fp64({XFG_FP64, XFG_FP64_STRICT});
