"""Host-side mirror of the reference's class Fluid (src/global_class.h:14-55) over the C ABI.

Method names, flags and return values follow the reference:
  BoundaryCondition(flag)      flag 0 -> U, else U1            (src/Fluids.cpp:922-933)
  UpdateFluidStates(flag)      -> (error captured, 4 timers)    (src/Fluids.cpp:935-944)
  ComputeFluidLU(flag)         -> 23 timers                     (src/Fluids.cpp:951-961)
  UpdateFluidURK3(flag, dt)    flag 1..3                         (src/Fluids.cpp:946-949)
  GetFluidDt()                 -> dt                             (src/Fluids.cpp:897-920)
  EstimateFluidNAN(flag)       -> error captured                 (src/Fluids.cpp:963-1040)
plus the fused forms step() and advance() that run XFLUIDS::Evolution's loop body on the device.
Every call goes to the CUDA library; there is no host fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import Block, Scheme, Thermal, ARRAYS, AOS_E, check, lib


class Fluid:
    def __init__(self, block: Block, scheme: Scheme, thermal: Thermal, device: int = 0):
        self.block, self.scheme, self.thermal = block, scheme, thermal
        self.E = scheme.Emax
        self.NS = scheme.num_species
        self._h = C.c_void_p()
        check(lib().xfg_create(C.byref(block), C.byref(scheme), C.byref(thermal), device, C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().xfg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------------------------
    def InitialU(self, U: np.ndarray, T: np.ndarray | None = None):
        """Load U (AoS, Emax per cell) and the Newton warm-start T; U1 = U."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.size != self.block.ncell * self.E:
            raise ValueError(f"U has {U.size} values, expected {self.block.ncell * self.E}")
        Tp = None
        if T is not None:
            T = np.ascontiguousarray(T, dtype=np.float64)
            if T.size != self.block.ncell:
                raise ValueError("T size mismatch")
            Tp = T.ctypes.data_as(C.c_void_p)
        check(lib().xfg_set_state(self._h, U.ctypes.data_as(C.c_void_p), Tp))

    set_state = InitialU

    def set_transport(self, transport):
        """Fitted transport data of a viscous scheme (xfg_transport, thermo.transport_from_arrays)."""
        check(lib().xfg_set_transport(self._h, C.byref(transport)))

    # -- checkpoints (XFLUIDS::Output_Ubak / Read_Ubak, src/XFLUIDS.cpp:658-724) -------------------
    def write_checkpoint(self, path: str, step: int, time: float, duration: float = 0.0):
        check(lib().xfg_checkpoint_write(self._h, str(path).encode(), int(step), float(time), float(duration)))

    def read_checkpoint(self, path: str):
        """Load U from a checkpoint file; returns (step, time, duration). Run initialize() next."""
        st, t, dur = C.c_int(), C.c_double(), C.c_float()
        check(lib().xfg_checkpoint_read(self._h, str(path).encode(), C.byref(st), C.byref(t), C.byref(dur)))
        return st.value, t.value, dur.value

    def get(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """Array `name` in the reference layout; into `out` when given (e.g. a PinnedArray's
        array, so that the device-to-host copy runs at the link's speed)."""
        n = self.block.ncell
        size = n * self.E if name in AOS_E else (n * self.NS if name == "y" else n)
        if out is None:
            out = np.empty(size, dtype=np.float64)
        elif out.size != size or out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a contiguous float64 array of {size} values")
        check(lib().xfg_get_array(self._h, ARRAYS[name], out.ctypes.data_as(C.c_void_p)))
        return out

    def set(self, name: str, arr: np.ndarray):
        """Write U, U1 (reference AoS layout, ghosts included) or T into the handle."""
        n = self.block.ncell
        size = n * self.E if name in ("U", "U1") else n
        if name not in ("U", "U1", "T"):
            raise ValueError("set() takes U, U1 or T")
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        if a.size != size:
            raise ValueError(f"{name} needs {size} values")
        check(lib().xfg_set_array(self._h, ARRAYS[name], a.ctypes.data_as(C.c_void_p)))

    # -- the reference's stage methods -------------------------------------------------------
    def BoundaryCondition(self, flag: int = 0):
        check(lib().xfg_boundary(self._h, flag))

    def UpdateFluidStates(self, flag: int = 0):
        err = C.c_int()
        tm = (C.c_float * 4)()
        check(lib().xfg_update_states(self._h, flag, C.byref(err), tm))
        return bool(err.value), list(tm)

    def ComputeFluidLU(self, flag: int = 0):
        tm = (C.c_float * 23)()
        check(lib().xfg_compute_lu(self._h, flag, tm))
        return list(tm)

    def UpdateFluidURK3(self, flag: int, dt: float):
        check(lib().xfg_update_rk3(self._h, flag, dt))

    def GetFluidDt(self) -> float:
        d = C.c_double()
        check(lib().xfg_get_dt(self._h, C.byref(d)))
        return d.value

    def EstimateFluidNAN(self, flag: int):
        err = C.c_int()
        pos = (C.c_int * (self.E + 4))()
        check(lib().xfg_estimate_nan(self._h, flag, C.byref(err), pos))
        return bool(err.value), list(pos)

    # -- XFLUIDS::Evolution loop body --------------------------------------------------------
    def initialize(self):
        """main.cpp:45-47: BoundaryCondition(U) then UpdateStates(U) before the first step."""
        self.BoundaryCondition(0)
        err, _ = self.UpdateFluidStates(0)
        return err

    def stage(self, flag: int, dt: float):
        """One RK stage as XFLUIDS::RungeKuttaSP3rd runs it (src/XFLUIDS.cpp:441-525)."""
        UI = 0 if flag == 1 else 1
        self.BoundaryCondition(UI)
        err, _ = self.UpdateFluidStates(UI)
        self.ComputeFluidLU(UI)
        self.UpdateFluidURK3(flag, dt)
        return err

    def step(self, target_t: float = 1e300):
        """One fused step: returns (status, t, dt). status 0 ok, >0 numerical error code."""
        t, dt = C.c_double(), C.c_double()
        st = check(lib().xfg_step(self._h, target_t, C.byref(t), C.byref(dt)))
        return st, t.value, dt.value

    def advance(self, nsteps: int, target_t: float = 1e300):
        """Up to nsteps fused steps from a replayed CUDA graph: returns (status, t, steps)."""
        t, n = C.c_double(), C.c_int()
        st = check(lib().xfg_advance(self._h, nsteps, target_t, C.byref(t), C.byref(n)))
        return st, t.value, n.value

    def advance_timed(self, nsteps: int, target_t: float = 1e300):
        """advance() plus the device time (ms, CUDA events on the handle's stream)."""
        t, n, ms = C.c_double(), C.c_int(), C.c_float()
        st = check(lib().xfg_advance_timed(self._h, nsteps, target_t, C.byref(t), C.byref(n), C.byref(ms)))
        return st, t.value, n.value, ms.value

    @property
    def launches_per_step(self) -> int:
        n = C.c_int()
        check(lib().xfg_launches_per_step(self._h, C.byref(n)))
        return n.value

    def time_phases(self, target_t: float = 1e300):
        """One fused step with per-phase device times (ms): dt, boundary, states, faces x/y/z, rk."""
        ms = (C.c_float * 7)()
        check(lib().xfg_time_phases(self._h, target_t, ms))
        return dict(zip(["dt", "boundary", "states", "faces_x", "faces_y", "faces_z", "div_rk"], list(ms)))

    @property
    def time(self) -> float:
        t = C.c_double()
        check(lib().xfg_get_time(self._h, C.byref(t)))
        return t.value

    @time.setter
    def time(self, t: float):
        check(lib().xfg_set_time(self._h, t))

    def synchronize(self):
        check(lib().xfg_synchronize(self._h))


def measure_pipe_peaks(device: int = 0):
    """Measured FP64 / FP32 FMA throughput of the GPU in FLOP/s (FMA = 2)."""
    out = (C.c_double * 3)()
    check(lib().xfg_measure_pipe_peaks(device, out))
    return {"fp64_flops": out[0], "fp32_flops": out[1], "sm_clock_mhz": out[2]}


class PinnedArray:
    """A numpy view of page-locked host memory (xfg_pinned_alloc)."""

    def __init__(self, n: int, dtype=np.float64):
        self.nbytes = int(n) * np.dtype(dtype).itemsize
        self._p = C.c_void_p()
        check(lib().xfg_pinned_alloc(self.nbytes, C.byref(self._p)))
        buf = (C.c_char * self.nbytes).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(n))

    def close(self):
        if self._p.value:
            self.array = None
            lib().xfg_pinned_free(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_info() -> str:
    return lib().xfg_build_info().decode()


__all__ = ["Fluid", "measure_pipe_peaks", "build_info", "abi"]
