// Kernel instantiation: mixture of 2 species (Emax = 6), WENO5 and WENO7, FP64 compiled without
// contraction (--fmad=false); serves both FP64 precision ids.
#define XFG_KNS cop2_strict
#include "xfg_inst.cuh"
static xfg::cop2_strict::Registrar<true, 2, false> reg_fp64({XFG_FP64, XFG_FP64_STRICT});
