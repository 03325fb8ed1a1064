// Kernel instantiation: multi-component mixture of 4 species, Emax = 8, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<true, 4> reg_cop4;
