// Kernel instantiation: multi-component mixture of 2 species, Emax = 6, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<true, 2> reg_cop2;
