"""Stage-by-stage parity against the oracle at the workloads' parity sizes, two SSP-RK3 steps:
every stage's U, U1, LU, the primitives and dt within the parity bound (test_parity_gpu.run_stagewise),
and the strict form bit for bit.

- the 2D isentropic vortex at 1024^2 (its x rows are 1032 cells with ghosts: past 2^10 per row and
  above a million cells, the sizes where a stride or index bug of the larger workloads shows);
- the 5-species JANAF WENO7 temporal mixing layer at 64 x 32 x 32 (the workload's own state at the
  parity size: 1 % noise, periodic x and z, outflow y);
- the member of the seeded 256-member Riemann ensemble closest to 128^2 (member 11, 129^2), with
  the ensemble's own quadrant states and CFL 0.45.

The oracle runs on all host threads (its reductions are order-independent, so the result is the
same on any thread count).
"""
import os

import numpy as np
import pytest

import helpers as H
from oracle import xfo
from test_parity_gpu import run_stagewise
from xfluids_gb300 import cases
from xfluids_gb300.abi import FP64, FP64_STRICT

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _all_threads():
    xfo.set_threads(os.cpu_count() or 1)
    yield


def _ensemble_member_near(n=128, count=256, seed=0):
    sizes, _ = cases.ensemble_sizes(count, seed)
    q = int(np.argmin(np.abs(sizes - n)))
    return q, int(sizes[q])


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
def test_vortex_1024_stagewise(precision, cuda_lib):
    worst = run_stagewise(cases.isentropic_vortex(1024), steps=2, precision=precision)
    print(f"vortex 1024^2: worst normwise relative difference {worst:.3e}")
    if precision == FP64_STRICT:
        assert worst == 0.0


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
def test_mixing_layer_64x32x32_stagewise(precision, cuda_lib):
    th = H.thermal(cases.MIXING_SPECIES, 0)
    worst = run_stagewise(cases.mixing_layer((64, 32, 32), thermal=th), steps=2, precision=precision)
    print(f"mixing layer 64x32x32: worst normwise relative difference {worst:.3e}")
    if precision == FP64_STRICT:
        assert worst == 0.0   # JANAF: no log, the strict form is the reference's operation sequence


@pytest.mark.parametrize("precision", [FP64, FP64_STRICT], ids=["fp64", "strict"])
def test_ensemble_member_stagewise(precision, cuda_lib):
    q, n = _ensemble_member_near(128)
    assert n <= 140
    worst = run_stagewise(H.riemann_member(q, n), steps=2, precision=precision)
    print(f"ensemble member {q} ({n}^2): worst normwise relative difference {worst:.3e}")
    if precision == FP64_STRICT:
        assert worst == 0.0
