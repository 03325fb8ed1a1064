// Kernel instantiation: the FP64 face sweeps of a 5-species mixture compiled with FMA contraction.
// They replace the face launchers of the no-contraction unit for XFG_FP64; primitive recovery
// (the temperature Newton iteration, whose stopping test |dT| <= 1e-6 makes T sensitive to the
// rounding of every operation) and all other kernels stay in that unit, and XFG_FP64_STRICT keeps
// its no-contraction faces.
#define XFG_KNS cop5_faces
#include "xfg_inst.cuh"
static xfg::cop5_faces::FacesRegistrar<true, 5> reg_faces({XFG_FP64});
