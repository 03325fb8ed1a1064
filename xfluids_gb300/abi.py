"""ctypes mirror of include/xfluids_gb300.h and the loader of the CUDA library.

The structures here are byte-for-byte the C structs of the ABI. The library is the in-tree
``xfluids_gb300/_build/libxfluids_gb300.so`` produced by ``__graft_entry__.build()``; loading fails
loudly when it is missing, there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

MAX_SPECIES = 9
MAX_EQ = MAX_SPECIES + 4

# enum xfg_bc, reference src/include/global_setup.h:96-105
INFLOW, OUTFLOW, SYMMETRY, PERIODIC, NSLIPWALL, VISCWALL, SLIPWALL, INNERBLOCK = range(8)
# enum xfg_artificial (Artificial_type)
ROE, LLF, GLF = 1, 2, 3
# enum xfg_precision
FP64, MIXED, FP64_STRICT = 0, 1, 2

# enum xfg_array
ARRAYS = {
    "U": 0, "U1": 1, "LU": 2, "rho": 3, "p": 4, "u": 5, "v": 6, "w": 7, "c": 8, "H": 9,
    "T": 10, "gamma": 11, "e": 12, "Cp": 13, "R": 14, "y": 15, "Fwx": 16, "Fwy": 17, "Fwz": 18,
}
AOS_E = {"U", "U1", "LU", "Fwx", "Fwy", "Fwz"}


class Block(C.Structure):
    """xfg_block: the fields of the reference Block/MeshSize the path reads."""
    _fields_ = [
        ("Xmax", C.c_int), ("Ymax", C.c_int), ("Zmax", C.c_int),
        ("X_inner", C.c_int), ("Y_inner", C.c_int), ("Z_inner", C.c_int),
        ("Bwidth_X", C.c_int), ("Bwidth_Y", C.c_int), ("Bwidth_Z", C.c_int),
        ("DimX", C.c_int), ("DimY", C.c_int), ("DimZ", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("_dx", C.c_double), ("_dy", C.c_double), ("_dz", C.c_double),
        ("CFLnumber", C.c_double),
        ("Boundarys", C.c_int * 6),
    ]

    @property
    def ncell(self) -> int:
        return self.Xmax * self.Ymax * self.Zmax

    @property
    def inner_cells(self) -> int:
        return self.X_inner * self.Y_inner * self.Z_inner

    @property
    def shape(self):
        """(Zmax, Ymax, Xmax): numpy shape of a SoA field (x fastest)."""
        return (self.Zmax, self.Ymax, self.Xmax)

    def inner_slices(self):
        return (slice(self.Bwidth_Z, self.Bwidth_Z + self.Z_inner),
                slice(self.Bwidth_Y, self.Bwidth_Y + self.Y_inner),
                slice(self.Bwidth_X, self.Bwidth_X + self.X_inner))


class Thermal(C.Structure):
    """xfg_thermal: Setup::ReadThermal output (src/read_ini/src/thermal.cpp:36-178)."""
    _fields_ = [
        ("num_species", C.c_int),
        ("Wi", C.c_double * MAX_SPECIES),
        ("_Wi", C.c_double * MAX_SPECIES),
        ("Ri", C.c_double * MAX_SPECIES),
        ("Hia", C.c_double * (MAX_SPECIES * 21)),
        ("Hib", C.c_double * (MAX_SPECIES * 6)),
    ]


class Scheme(C.Structure):
    """xfg_scheme: the reference's compile-time scheme switches as run-time values."""
    _fields_ = [
        ("cop", C.c_int), ("num_species", C.c_int), ("scheme_order", C.c_int),
        ("artificial_type", C.c_int), ("thermo", C.c_int), ("ghost_species", C.c_int),
        ("ncop_gamma", C.c_double), ("precision", C.c_int), ("positivity", C.c_int), ("viscous", C.c_int),
    ]

    @property
    def Emax(self) -> int:
        return self.num_species + 4 if self.cop else 5


FIT_ORDER, SPCH = 4, 9
VISC, VISC_HEAT, VISC_DIFFU = 1, 2, 4


class Transport(C.Structure):
    """xfg_transport: fitted transport coefficients and species characteristics."""
    _fields_ = [
        ("num_species", C.c_int),
        ("visc", C.c_double * (MAX_SPECIES * FIT_ORDER)),
        ("therm", C.c_double * (MAX_SPECIES * FIT_ORDER)),
        ("dkj", C.c_double * (MAX_SPECIES * MAX_SPECIES * FIT_ORDER)),
        ("species_chara", C.c_double * (MAX_SPECIES * SPCH)),
        ("yil_limiter", C.c_double), ("dim_limiter", C.c_double),
    ]


_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libxfluids_gb300.so")
_lib = None


class XfgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"xfluids_gb300 status {status}: {msg}")
        self.status = status


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA library not built: {LIB_PATH} is missing (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    pd = C.POINTER(C.c_double)
    pi = C.POINTER(C.c_int)
    L.xfg_last_error.restype = C.c_char_p
    L.xfg_build_info.restype = C.c_char_p
    sig = {
        "xfg_create": [C.POINTER(Block), C.POINTER(Scheme), C.POINTER(Thermal), I, C.POINTER(P)],
        "xfg_destroy": [P],
        "xfg_set_state": [P, P, P],
        "xfg_get_array": [P, I, P],
        "xfg_set_array": [P, I, P],
        "xfg_boundary": [P, I],
        "xfg_update_states": [P, I, pi, C.POINTER(C.c_float)],
        "xfg_compute_lu": [P, I, C.POINTER(C.c_float)],
        "xfg_update_rk3": [P, I, D],
        "xfg_get_dt": [P, pd],
        "xfg_estimate_nan": [P, I, pi, pi],
        "xfg_step": [P, D, pd, pd],
        "xfg_advance": [P, I, D, pd, pi],
        "xfg_set_time": [P, D],
        "xfg_get_time": [P, pd],
        "xfg_synchronize": [P],
        "xfg_device_array": [P, I, C.POINTER(P), C.POINTER(C.c_size_t)],
        "xfg_measure_pipe_peaks": [I, pd],
        "xfg_time_phases": [P, D, C.POINTER(C.c_float)],
        "xfg_advance_timed": [P, I, D, pd, pi, C.POINTER(C.c_float)],
        "xfg_launches_per_step": [P, pi],
        "xfg_pinned_alloc": [C.c_size_t, C.POINTER(P)],
        "xfg_pinned_free": [P],
        "xfg_compute_lu_noalloc": [C.POINTER(Block), C.POINTER(Scheme), C.POINTER(Thermal), P, P, P, P],
    }
    sig.update({
        "xfg_ensemble_create": [I, C.c_size_t, C.POINTER(Scheme), C.POINTER(Thermal), I, C.POINTER(P)],
        "xfg_ensemble_destroy": [P],
        "xfg_ensemble_add": [P, C.POINTER(Block), P, D, pi],
        "xfg_ensemble_add_t": [P, C.POINTER(Block), P, P, D, pi],
        "xfg_ensemble_remove": [P, I],
        "xfg_ensemble_advance": [P, I, I, C.POINTER(C.c_float)],
        "xfg_ensemble_status": [P, I, pd, pi, pi],
        "xfg_ensemble_get_state": [P, I, P],
        "xfg_ensemble_set_option": [P, I, I],
        "xfg_ensemble_checkpoint_write": [P, I, C.c_char_p, C.c_float, P],
        "xfg_ensemble_add_checkpoint": [P, C.POINTER(Block), C.c_char_p, D, P, pi],
        "xfg_checkpoint_write": [P, C.c_char_p, I, D, C.c_float],
        "xfg_set_transport": [P, C.POINTER(Transport)],
        "xfg_ensemble_set_transport": [P, C.POINTER(Transport)],
        "xfg_checkpoint_read": [P, C.c_char_p, pi, pd, C.POINTER(C.c_float)],
        "xfg_ensemble_get_option": [P, I, pi],
        "xfg_ensemble_active": [P],
    })
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.xfg_ensemble_member_bytes.argtypes = [C.POINTER(Block), I]
    L.xfg_ensemble_member_bytes.restype = C.c_size_t
    L.xfg_ensemble_member_bytes_for.argtypes = [C.POINTER(Block), C.POINTER(Scheme)]
    L.xfg_ensemble_member_bytes_for.restype = C.c_size_t
    L.xfg_ensemble_free_bytes.argtypes = [P]
    L.xfg_ensemble_free_bytes.restype = C.c_size_t
    _lib = L
    return L


def check(status: int) -> int:
    if status < 0:
        raise XfgError(status, lib().xfg_last_error().decode())
    return status


def ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))
