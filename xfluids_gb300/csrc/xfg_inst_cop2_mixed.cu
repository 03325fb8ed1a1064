// Kernel instantiation: mixture of 2 species (Emax = 6), WENO5 and WENO7, mixed form.
#define XFG_KNS cop2_mixed
#include "xfg_inst.cuh"
static xfg::cop2_mixed::Registrar<true, 2, true> reg_mixed({XFG_MIXED});
