// Kernel instantiation: mixture of 3 species (Emax = 7), WENO5 and WENO7, mixed form.
#define XFG_KNS cop3_mixed
#include "xfg_inst.cuh"
static xfg::cop3_mixed::Registrar<true, 3, true> reg_mixed({XFG_MIXED});
