// Kernel instantiation: multi-component mixture of 5 species, Emax = 9, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<true, 5> reg_cop5;
