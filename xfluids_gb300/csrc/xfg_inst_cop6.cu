// Kernel instantiation: multi-component mixture of 6 species, Emax = 10, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<true, 6> reg_cop6;
