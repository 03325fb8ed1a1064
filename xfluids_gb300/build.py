"""In-tree build of the CUDA library for sm_103a (nvcc, translation units compiled in parallel)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libxfluids_gb300.so")

# (unit, extra nvcc flags): FP64 mixture kernels and the strict single-gas kernels are compiled
# without floating-point contraction.
NOFMA = ["--fmad=false", "-DXFG_STRICT"]
UNITS = [("xfg_api.cu", []), ("xfg_noalloc.cu", []), ("xfg_inst_ncop.cu", []), ("xfg_inst_ncop_strict.cu", NOFMA),
         ("xfg_ensemble.cu", [])]
UNITS += [(f"xfg_inst_cop{n}.cu", NOFMA) for n in (2, 3, 4, 5, 6)]
UNITS += [(f"xfg_inst_cop{n}_mixed.cu", []) for n in (2, 3, 4, 5, 6)]
UNITS += [(f"xfg_inst_cop{n}_faces.cu", []) for n in (2, 3, 4, 5, 6)]
UNITS += [("xfg_ensemble_cop5.cu", NOFMA), ("xfg_ensemble_cop5_fma.cu", [])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _sources_mtime():
    m = 0.0
    for root in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(root):
            if f.endswith((".cu", ".cuh", ".h")):
                m = max(m, os.path.getmtime(os.path.join(root, f)))
    return m


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every unit (in parallel) and link libxfluids_gb300.so. Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    nvcc = _nvcc()

    def compile_one(item):
        unit, unit_flags = item
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        extra = os.environ.get("XFG_NVCC_EXTRA", "").split()
        cmd = [nvcc, *ARCH, *FLAGS, *unit_flags, *extra, "-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    workers = min(len(UNITS), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
