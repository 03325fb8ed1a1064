// Kernel instantiation: single gas (no COP), Emax = 5, WENO5 and WENO7.
#include "xfg_inst.cuh"
static xfg::Registrar<false, 1> reg_ncop;
