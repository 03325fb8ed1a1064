// Kernel instantiation: multi-component mixture of 3 species, Emax = 7, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<true, 3> reg_cop3;
