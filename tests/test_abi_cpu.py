"""The C-ABI library loads, exports every declared entry point, and its structs match ctypes.
No compute calls (no GPU here)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from xfluids_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xfluids_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(xfg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(cuda_lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(cuda_lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (xfg_\w+)", out))
    assert set(syms) <= exported


def test_build_info_lists_kernels(cuda_lib):
    info = cuda_lib.xfg_build_info().decode()
    assert "sm_103a" in info and "ncop1/weno5" in info and "cop5/weno7" in info


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "xfluids_gb300.h"
int main(void) {
    printf("%zu %zu %zu\n", sizeof(xfg_block), sizeof(xfg_thermal), sizeof(xfg_scheme));
    printf("%zu %zu %zu\n", offsetof(xfg_block, dx), offsetof(xfg_block, CFLnumber), offsetof(xfg_block, Boundarys));
    printf("%zu %zu\n", offsetof(xfg_thermal, Hia), offsetof(xfg_thermal, Hib));
    printf("%zu %zu %zu\n", offsetof(xfg_scheme, ncop_gamma), offsetof(xfg_scheme, precision),
           offsetof(xfg_scheme, positivity));
    return 0;
}
"""


def test_struct_layouts_match_header():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(src, "w").write(PROBE)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    B, T, S = abi.Block, abi.Thermal, abi.Scheme
    expect = [C.sizeof(B), C.sizeof(T), C.sizeof(S), B.dx.offset, B.CFLnumber.offset, B.Boundarys.offset,
              T.Hia.offset, T.Hib.offset, S.ncop_gamma.offset, S.precision.offset, S.positivity.offset]
    assert vals == expect


def test_create_rejects_bad_arguments(cuda_lib):
    from xfluids_gb300 import cases
    b, s, th, U, T = cases.sod(32)
    s.scheme_order = 8
    h = C.c_void_p()
    rc = cuda_lib.xfg_create(C.byref(b), C.byref(s), C.byref(th), 0, C.byref(h))
    assert rc == -1 and not h.value
    assert "scheme_order" in cuda_lib.xfg_last_error().decode()
    s.scheme_order = 5
    b.Bwidth_X = 2
    rc = cuda_lib.xfg_create(C.byref(b), C.byref(s), C.byref(th), 0, C.byref(h))
    assert rc == -1 and "Bwidth" in cuda_lib.xfg_last_error().decode()
    from xfluids_gb300.abi import OUTFLOW
    from xfluids_gb300.mesh import make_block
    long3d = make_block((8, 70000, 8), (1.0, 1.0, 1.0), [OUTFLOW] * 6)
    rc = cuda_lib.xfg_create(C.byref(long3d), C.byref(s), C.byref(th), 0, C.byref(h))
    assert rc == -1 and "elongated" in cuda_lib.xfg_last_error().decode()


def test_ensemble_rejects_unsupported_schemes_before_touching_a_device(cuda_lib):
    """xfg_ensemble_create checks the scheme first (no device call is made for these)."""
    from xfluids_gb300.ensemble import Ensemble
    from xfluids_gb300.mesh import make_scheme
    for kw in (dict(cop=True, num_species=2), dict(precision=2), dict(scheme_order=8), dict(viscous=1)):
        visc = kw.pop("viscous", 0)
        sc = make_scheme(**{"scheme_order": 5, "artificial_type": abi.LLF, **kw})
        sc.viscous = visc
        with pytest.raises(abi.XfgError):
            Ensemble(sc, capacity=2, pool_bytes=1 << 20)


def test_checkpoint_format_is_the_references(tmp_path):
    """int32 Step, float64 Time, float32 duration, then U, packed (XFLUIDS.cpp:658-724)."""
    import numpy as np
    from xfluids_gb300 import checkpoint
    U = np.arange(40, dtype=np.float64) * 0.5
    p = tmp_path / "ck"
    checkpoint.write(p, 17, 0.125, 3.5, U)
    raw = p.read_bytes()
    assert len(raw) == 4 + 8 + 4 + 8 * 40
    assert raw[:4] == (17).to_bytes(4, "little")
    assert np.frombuffer(raw[4:12], "<f8")[0] == 0.125 and np.frombuffer(raw[12:16], "<f4")[0] == 3.5
    step, t, dur, V = checkpoint.read(p, 40)
    assert (step, t, dur) == (17, 0.125, 3.5) and np.array_equal(U, V)
    with pytest.raises(ValueError):
        checkpoint.read(p, 41)


def test_noalloc_rejects_bad_arguments_before_touching_a_device(cuda_lib):
    """xfg_compute_lu_noalloc checks its arguments and the block's scratch need against the fixed
    scratch size before any CUDA call; these calls return there (the state pointers are never
    dereferenced)."""
    from xfluids_gb300 import cases
    from xfluids_gb300.abi import MIXED
    fake = C.c_void_p(256)
    f = cuda_lib.xfg_compute_lu_noalloc

    def call(b, s, th, U=fake, LU=fake):
        return f(C.byref(b), C.byref(s), C.byref(th), U, None, LU, None)

    b, s, th, _, _ = cases.isentropic_vortex(32)
    assert call(b, s, th, U=None) == -1 and "null" in cuda_lib.xfg_last_error().decode()
    s.precision = MIXED
    assert call(b, s, th) == -1 and "FP64" in cuda_lib.xfg_last_error().decode()
    s.precision = 0
    s.positivity = 1
    assert call(b, s, th) == -1 and "positivity" in cuda_lib.xfg_last_error().decode()
    s.positivity = 0
    big, s2, th2, _, _ = cases.isentropic_vortex(512)
    assert call(big, s2, th2) == -2
    assert "XFG_NOALLOC_MAX_SCRATCH_BYTES" in cuda_lib.xfg_last_error().decode()
    # a z-only block of 70000 cells fits the scratch (37 arrays x 70 k cells) but not the face
    # launch's grid limit: rejected by the checks xfg_create makes, before any launch
    from xfluids_gb300.mesh import make_block, make_scheme, empty_thermal
    from xfluids_gb300.abi import PERIODIC
    zb = make_block((0, 0, 70000), (1.0, 1.0, 1.0), [PERIODIC] * 6, bwidth=3)
    assert call(zb, make_scheme(), empty_thermal()) == -1
    assert "elongated" in cuda_lib.xfg_last_error().decode()
    s.artificial_type = 7
    assert call(b, s, th) == -1 and "artificial_type" in cuda_lib.xfg_last_error().decode()
