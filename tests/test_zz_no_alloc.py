"""xfg_compute_lu_noalloc: the right-hand side of a state for callers that cannot allocate device
memory (they pass device pointers in and out; the library's intermediates live in a fixed device
array). Checked against the allocating path (xfg_create + xfg_boundary + xfg_update_states +
xfg_compute_lu) on two calls in a row, and against the oracle's right-hand side of the same state.
Collected last on purpose (file name)."""
import ctypes as C
import ctypes.util
import glob
import os

import numpy as np
import pytest

import helpers as H
from xfluids_gb300 import cases

pytestmark = pytest.mark.gpu


def _cudart():
    cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*") + [ctypes.util.find_library("cudart") or ""]
    for c in cands:
        if c and os.path.exists(c):
            L = C.CDLL(c)
            L.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            L.cudaFree.argtypes = [C.c_void_p]
            L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            L.cudaDeviceSynchronize.argtypes = []
            L.cudaSetDevice.argtypes = [C.c_int]
            return L
    pytest.skip("libcudart not found")


class DevBuf:
    def __init__(self, rt, nbytes):
        self.rt, self.p = rt, C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.p), nbytes) == 0
        self.nbytes = nbytes

    def put(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert self.rt.cudaMemcpy(self.p, a.ctypes.data_as(C.c_void_p), a.nbytes, 1) == 0

    def get(self, n):
        out = np.empty(n, dtype=np.float64)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), self.p, out.nbytes, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.p)


def _oracle_lu(b, s, th, U, T):
    """The oracle's right-hand side of U and the dt of the same state."""
    from oracle.xfo import Oracle
    o = Oracle(b, s, th, U, T)
    o.boundary(0)
    o.update_states(0)
    o.compute_lu(0)
    return o.get("LU"), o.get_dt()


def _reference_lu(b, s, th, U, T):
    from xfluids_gb300.fluid import Fluid
    f = Fluid(b, s, th)
    f.InitialU(U, T)
    f.BoundaryCondition(0)
    f.UpdateFluidStates(0)
    f.ComputeFluidLU(0)
    lu = f.get("LU")
    f.close()
    return lu


@pytest.mark.parametrize("case", ["vortex48", "mixing5"])
def test_noalloc_matches_allocating_path_twice(case, cuda_lib):
    if case == "vortex48":
        b, s, th, U, T = cases.isentropic_vortex(48)
    else:
        b, s, th, U, T = H.mixing_small((16, 12, 8))
    E = s.Emax
    ref = _reference_lu(b, s, th, U, T)
    oracle, dt = _oracle_lu(b, s, th, U, T)
    rt = _cudart()
    rt.cudaSetDevice(0)
    dU = DevBuf(rt, U.size * 8)
    dLU = DevBuf(rt, U.size * 8)
    dT = DevBuf(rt, b.ncell * 8) if T is not None else None
    try:
        dU.put(U)
        if dT is not None:
            dT.put(T)
        for call in range(2):
            rc = cuda_lib.xfg_compute_lu_noalloc(C.byref(b), C.byref(s), C.byref(th), dU.p,
                                                 dT.p if dT is not None else None, dLU.p, None)
            assert rc == 0, cuda_lib.xfg_last_error().decode()
            assert rt.cudaDeviceSynchronize() == 0
            got = dLU.get(U.size)
            r = H.normwise(H.inner_aos(b, got, E), H.inner_aos(b, ref, E), E)
            assert np.all(r <= H.PARITY_TOL), f"call {call}: {r}"
            # against the oracle: per component for the single gas; for the mixture (whose FP64
            # face sweeps are contracted) through the stage increment max|dt dLU| / max|U|, as the
            # stage parity tests compare it
            g, o = H.inner_aos(b, got, E), H.inner_aos(b, oracle, E)
            if s.cop:
                ro = np.abs(dt * (g - o)).max(axis=0) / np.abs(H.inner_aos(b, U, E)).max(axis=0).clip(1e-300)
            else:
                ro = H.normwise(g, o, E)
            assert np.all(ro <= H.PARITY_TOL), f"call {call} against the oracle: {ro}"
            ghosts = got.reshape(b.Zmax, b.Ymax, b.Xmax, E).copy()
            ghosts[b.inner_slices()] = 0.0
            assert not ghosts.any()
    finally:
        dU.free(), dLU.free()
        if dT is not None:
            dT.free()


def test_noalloc_rejects_blocks_beyond_scratch(cuda_lib):
    b, s, th, U, T = cases.isentropic_vortex(1024)   # 50 arrays x 1.06 M cells: about 424 MB > 64 MiB
    rc = cuda_lib.xfg_compute_lu_noalloc(C.byref(b), C.byref(s), C.byref(th), C.c_void_p(16), None,
                                         C.c_void_p(16), None)
    assert rc < 0
    assert "too large" in cuda_lib.xfg_last_error().decode()
