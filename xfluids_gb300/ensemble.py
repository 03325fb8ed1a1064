"""Batched ensemble of independent grids (single gas, or 5-species mixtures) over the C ABI
(xfg_ensemble_*).

Each member is one XFLUIDS run of the same scheme with its own size, state, dt and target time;
all members share one device pool and one sequence of batched kernels per step, replayed from a
CUDA graph. Used by the ensemble benchmark and by the request server (xfluids_gb300/serve.py).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import Block, Scheme, Thermal, check, lib
from .mesh import empty_thermal

NO_SLOT, NO_MEMORY = 1, 2
# launch-schedule options (xfg_ensemble_set_option)
LARGEST_FIRST, FUSED_FACES, GRAPH_STEPS, TILE_1D, TILE_2D_SMALL, TILE_2D_LARGE, TILE_3D = range(7)
OPTIONS = {"largest_first": LARGEST_FIRST, "fused_faces": FUSED_FACES, "graph_steps": GRAPH_STEPS,
           "tile_1d": TILE_1D, "tile_2d_small": TILE_2D_SMALL, "tile_2d_large": TILE_2D_LARGE, "tile_3d": TILE_3D}


class Ensemble:
    def __init__(self, scheme: Scheme, capacity: int, pool_bytes: int, device: int = 0, thermal: Thermal = None):
        self.scheme = scheme
        self.pool_bytes = int(pool_bytes)
        self.thermal = thermal or empty_thermal()
        self._e = C.c_void_p()
        check(lib().xfg_ensemble_create(capacity, int(pool_bytes), C.byref(scheme), C.byref(self.thermal), device,
                                        C.byref(self._e)))
        self.blocks = {}

    def close(self):
        if getattr(self, "_e", None) and self._e.value:
            lib().xfg_ensemble_destroy(self._e)
            self._e = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_transport(self, transport):
        """Fitted transport data shared by the members of a viscous mixture ensemble (xfg_transport,
        thermo.transport_from_arrays / transport.fit_transport); needed before the first advance."""
        check(lib().xfg_ensemble_set_transport(self._e, C.byref(transport)))

    @staticmethod
    def member_bytes(block: Block, precision, scheme: Scheme = None) -> int:
        """Pool bytes of one member: a single gas of this precision, or a member under `scheme`."""
        if scheme is not None:
            return lib().xfg_ensemble_member_bytes_for(C.byref(block), C.byref(scheme))
        return lib().xfg_ensemble_member_bytes(C.byref(block), precision)

    def add(self, block: Block, U: np.ndarray, target_t: float, T: np.ndarray = None):
        """Admit a member (T: the temperature that warm-starts a mixture's Newton iteration);
        returns its slot, or None when no slot or no pool memory is free."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        Tp = None
        if T is not None:
            T = np.ascontiguousarray(T, dtype=np.float64)
            Tp = T.ctypes.data_as(C.c_void_p)
        slot = C.c_int(-1)
        rc = check(lib().xfg_ensemble_add_t(self._e, C.byref(block), U.ctypes.data_as(C.c_void_p), Tp,
                                            float(target_t), C.byref(slot)))
        if rc in (NO_SLOT, NO_MEMORY):
            return None
        self.blocks[slot.value] = block
        return slot.value

    def remove(self, slot: int):
        check(lib().xfg_ensemble_remove(self._e, slot))
        self.blocks.pop(slot, None)

    def advance(self, nsteps: int = 1, use_graph: bool = True):
        """nsteps steps of every active member; returns (status, device ms)."""
        ms = C.c_float()
        st = check(lib().xfg_ensemble_advance(self._e, nsteps, 1 if use_graph else 0, C.byref(ms)))
        return st, ms.value

    def status(self, slot: int):
        t, n, done = C.c_double(), C.c_int(), C.c_int()
        err = check(lib().xfg_ensemble_status(self._e, slot, C.byref(t), C.byref(n), C.byref(done)))
        return {"t": t.value, "steps": n.value, "done": bool(done.value), "error": err}

    def get_state(self, slot: int) -> np.ndarray:
        b = self.blocks[slot]
        out = np.empty(b.ncell * self.scheme.Emax, dtype=np.float64)
        check(lib().xfg_ensemble_get_state(self._e, slot, out.ctypes.data_as(C.c_void_p)))
        return out

    def write_checkpoint(self, slot: int, path: str, duration: float = 0.0):
        """The member as a checkpoint file of the reference's format (step count, time, U).
        Returns the GetDt maxima its next step would use (for add_checkpoint's lam)."""
        lam = np.zeros(3)
        check(lib().xfg_ensemble_checkpoint_write(self._e, slot, str(path).encode(), float(duration),
                                                  lam.ctypes.data_as(C.c_void_p)))
        return [float(x) for x in lam]

    def add_checkpoint(self, block: Block, path: str, target_t: float, lam=None):
        """Admit a member from a checkpoint file (time and step count restored; with lam, also the
        dt of its next step); slot or None."""
        slot = C.c_int(-1)
        lam_p = None
        if lam is not None:
            lam_a = np.ascontiguousarray(lam, dtype=np.float64)
            lam_p = lam_a.ctypes.data_as(C.c_void_p)
        rc = check(lib().xfg_ensemble_add_checkpoint(self._e, C.byref(block), str(path).encode(), float(target_t),
                                                     lam_p, C.byref(slot)))
        if rc in (NO_SLOT, NO_MEMORY):
            return None
        self.blocks[slot.value] = block
        return slot.value

    def set_option(self, option, value: int):
        option = OPTIONS.get(option, option)
        check(lib().xfg_ensemble_set_option(self._e, int(option), int(value)))

    def get_option(self, option) -> int:
        option = OPTIONS.get(option, option)
        v = C.c_int()
        check(lib().xfg_ensemble_get_option(self._e, int(option), C.byref(v)))
        return v.value

    def schedule(self) -> dict:
        return {name: self.get_option(o) for name, o in OPTIONS.items()}

    def set_schedule(self, sched: dict):
        for name, v in sched.items():
            self.set_option(name, v)

    @property
    def free_bytes(self) -> int:
        return lib().xfg_ensemble_free_bytes(self._e)

    @property
    def active(self) -> int:
        return lib().xfg_ensemble_active(self._e)
