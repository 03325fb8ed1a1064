// Kernel instantiation: mixture of 4 species (Emax = 8), WENO5 and WENO7, mixed form.
#define XFG_KNS cop4_mixed
#include "xfg_inst.cuh"
static xfg::cop4_mixed::Registrar<true, 4, true> reg_mixed({XFG_MIXED});
