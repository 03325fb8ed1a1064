"""ctypes wrapper of the CPU oracle (test infrastructure, see xfo_core.hpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU arms may import this module. It builds
oracle/_build/libxfo.so on first use when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from xfluids_gb300.abi import Block, Scheme, Thermal, Transport, ARRAYS, AOS_E

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libxfo.so")
SOURCES = ["xfo_capi.cpp", "xfo_core.hpp", "xfo_count.hpp"]


def build(force=False):
    """Compile the oracle (g++ -O3, OpenMP, no FMA contraction: the same bits on x86-64 and aarch64)."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(os.path.join(HERE, s)) for s in SOURCES)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           os.path.join(HERE, "xfo_capi.cpp"), "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I, D = C.c_void_p, C.c_int, C.c_double
        L.xfo_create.restype = P
        L.xfo_create.argtypes = [C.POINTER(Block), C.POINTER(Scheme), C.POINTER(Thermal)]
        L.xfo_destroy.argtypes = [P]
        L.xfo_destroy.restype = None
        for name, args in {
            "xfo_set_threads": [I], "xfo_set_state": [P, P, P], "xfo_boundary": [P, I],
            "xfo_update_states": [P, I], "xfo_compute_lu": [P, I], "xfo_update_rk3": [P, I, D],
            "xfo_get_dt": [P, C.POINTER(D)], "xfo_step": [P, D, C.POINTER(D), C.POINTER(D)],
            "xfo_set_time": [P, D], "xfo_get_array": [P, I, P], "xfo_set_transport": [P, C.POINTER(Transport)],
            "xfo_count_flops": [C.POINTER(Block), C.POINTER(Scheme), C.POINTER(Thermal), P, P, I,
                                C.POINTER(C.c_uint64)],
        }.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = I
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().xfo_set_threads(n)


class Oracle:
    """One fluid block on the CPU, stage-by-stage like class Fluid."""

    def __init__(self, block: Block, scheme: Scheme, thermal: Thermal, U: np.ndarray, T=None, transport=None):
        self.block, self.scheme, self.thermal = block, scheme, thermal
        self.E = scheme.Emax
        self.h = lib().xfo_create(C.byref(block), C.byref(scheme), C.byref(thermal))
        if not self.h:
            raise MemoryError("oracle allocation failed")
        if transport is not None:
            self.transport = transport
            lib().xfo_set_transport(self.h, C.byref(transport))
        self.set_state(U, T)

    def __del__(self):
        if getattr(self, "h", None):
            lib().xfo_destroy(self.h)
            self.h = None

    def set_state(self, U, T=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.size == self.block.ncell * self.E
        Tp = None
        if T is not None:
            T = np.ascontiguousarray(T, dtype=np.float64)
            Tp = T.ctypes.data_as(C.c_void_p)
        lib().xfo_set_state(self.h, U.ctypes.data_as(C.c_void_p), Tp)

    def boundary(self, flag):
        lib().xfo_boundary(self.h, flag)

    def update_states(self, flag):
        lib().xfo_update_states(self.h, flag)

    def compute_lu(self, flag):
        lib().xfo_compute_lu(self.h, flag)

    def update_rk3(self, flag, dt):
        lib().xfo_update_rk3(self.h, flag, dt)

    def get_dt(self):
        d = C.c_double()
        lib().xfo_get_dt(self.h, C.byref(d))
        return d.value

    def initialize(self):
        """main.cpp:45-47: BoundaryCondition + UpdateStates on U before the first step."""
        self.boundary(0)
        self.update_states(0)

    def stage(self, flag, dt):
        UI = 0 if flag == 1 else 1
        self.boundary(UI)
        self.update_states(UI)
        self.compute_lu(UI)
        self.update_rk3(flag, dt)

    def step(self, target_t=1e300):
        t, dt = C.c_double(), C.c_double()
        lib().xfo_step(self.h, target_t, C.byref(t), C.byref(dt))
        return t.value, dt.value

    def set_time(self, t):
        lib().xfo_set_time(self.h, t)

    def get(self, name):
        n = self.block.ncell
        size = n * self.E if name in AOS_E else (n * self.scheme.num_species if name == "y" else n)
        out = np.empty(size, dtype=np.float64)
        lib().xfo_get_array(self.h, ARRAYS[name], out.ctypes.data_as(C.c_void_p))
        return out


def count_flops(block, scheme, thermal, U, T=None, nsteps=1):
    """Algorithmic flops of nsteps steps; returns a dict per phase."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    Tp = None
    if T is not None:
        T = np.ascontiguousarray(T, dtype=np.float64)
        Tp = T.ctypes.data_as(C.c_void_p)
    out = (C.c_uint64 * 9)()
    lib().xfo_count_flops(C.byref(block), C.byref(scheme), C.byref(thermal),
                          U.ctypes.data_as(C.c_void_p), Tp, nsteps, out)
    names = ["boundary", "update_states", "local_eigen", "faces_x", "faces_y", "faces_z",
             "divergence", "rk", "dt"]
    return {k: int(v) for k, v in zip(names, out)}
