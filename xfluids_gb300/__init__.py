"""GB300-native convective right-hand side of XFluids (WENO5/7 + LLF, flux divergence, SSP-RK3,
primitive recovery with the multi-component temperature Newton iteration, CFL dt).

The compute path is the CUDA library xfluids_gb300/_build/libxfluids_gb300.so behind the C ABI of
include/xfluids_gb300.h; `Fluid` mirrors the reference's class Fluid over that ABI.
"""
from .abi import Block, Scheme, Thermal, INFLOW, OUTFLOW, SYMMETRY, PERIODIC, ROE, LLF, GLF, FP64, MIXED
from .mesh import make_block, make_scheme, empty_thermal

__all__ = ["Block", "Scheme", "Thermal", "make_block", "make_scheme", "empty_thermal",
           "INFLOW", "OUTFLOW", "SYMMETRY", "PERIODIC", "ROE", "LLF", "GLF", "FP64", "MIXED"]


def Fluid(*args, **kwargs):  # noqa: N802 - the reference's class name
    from .fluid import Fluid as _F
    return _F(*args, **kwargs)
