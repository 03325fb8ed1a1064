// Kernel instantiation: mixture of 3 species (Emax = 7), WENO5 and WENO7, FP64 compiled without
// contraction (--fmad=false); serves both FP64 precision ids.
#define XFG_KNS cop3_strict
#include "xfg_inst.cuh"
static xfg::cop3_strict::Registrar<true, 3, false> reg_fp64({XFG_FP64, XFG_FP64_STRICT});
