// Kernel instantiation: mixture of 5 species (Emax = 9), WENO5 and WENO7, FP64 compiled without
// contraction (--fmad=false); serves both FP64 precision ids.
#define XFG_KNS cop5_strict
#include "xfg_inst.cuh"
static xfg::cop5_strict::Registrar<true, 5, false> reg_fp64({XFG_FP64, XFG_FP64_STRICT});
