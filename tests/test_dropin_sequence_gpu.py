"""The reference's time-loop call sequence over the C ABI (tests/dropin_sequence.cpp): per step
CopyToUbak, GetFluidDt and RungeKuttaSP3rd's BoundaryCondition / UpdateStates / ComputeLU /
EstimateNAN / UpdateU for the three stages, with the C++ drop-in's copies into the reference-visible
buffers (the primitives after the third stage's UpdateStates, U after the step). Its state after the
steps equals the graph-replayed fused steps' (xfg_advance) to 1e-13, and its time per step is
printed beside theirs: at 4096^2 the overhead of the sequence (per-call synchronisation, the
primitive and U mirrors, the Ubak copy the reference itself makes) is bounded."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "dropin_sequence.cpp")


@pytest.fixture(scope="module")
def harness(cuda_lib, tmp_path_factory):
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    libdir = os.path.join(ROOT, "xfluids_gb300", "_build")
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_sequence")
    cmd = ["g++", "-O2", "-std=c++17", SRC, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           "-L", libdir, "-lxfluids_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, n, steps):
    r = subprocess.run([exe, str(n), str(steps)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    print(out)
    return out


def test_dropin_sequence_equals_fused_steps(harness):
    out = _run(harness, 256, 6)
    assert out["max_normwise_diff"] <= 1e-13, out


def test_dropin_sequence_overhead_at_4096(harness):
    out = _run(harness, 4096, 3)
    assert out["max_normwise_diff"] <= 1e-13, out
    assert out["dropin_over_advance"] <= 1.25, out
