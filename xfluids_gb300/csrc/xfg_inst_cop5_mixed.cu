// Kernel instantiation: mixture of 5 species (Emax = 9), WENO5 and WENO7, mixed form.
#define XFG_KNS cop5_mixed
#include "xfg_inst.cuh"
static xfg::cop5_mixed::Registrar<true, 5, true> reg_mixed({XFG_MIXED});
