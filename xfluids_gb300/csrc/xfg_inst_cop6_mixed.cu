// Kernel instantiation: mixture of 6 species (Emax = 10), WENO5 and WENO7, mixed form.
#define XFG_KNS cop6_mixed
#include "xfg_inst.cuh"
static xfg::cop6_mixed::Registrar<true, 6, true> reg_mixed({XFG_MIXED});
