"""Continuous-batching server (xfluids_gb300/serve.py): every request served in the mix, with
others arriving, running and leaving around it, gives the same result as the same solve run
alone through the single-grid path (Fluid.advance to its end time)."""
import pytest

from helpers import PARITY_TOL, normwise
from xfluids_gb300.ensemble import Ensemble
from xfluids_gb300.fluid import Fluid
from xfluids_gb300.mesh import empty_thermal
from xfluids_gb300.serve import Server, poisson_trace, serving_scheme, summary

pytestmark = pytest.mark.gpu

# mixed-precision results against the mixed single-grid run: FP32 rounding of differently
# contracted expressions, accumulated over the steps of a solve (normwise, per component)
MIXED_TOL = 1e-4


def solve_alone(r, scheme):
    """(U, t, steps, status) of the request run alone until its end time or its first error."""
    f = Fluid(r.block, scheme, empty_thermal())
    try:
        f.InitialU(r.U)
        f.initialize()
        while True:
            st, t, steps = f.advance(64, r.t_end)
            if st != 0 or t >= r.t_end:
                return f.get("U").reshape(-1), t, steps, st
    finally:
        f.close()


def small_trace(count=10, seed=7):
    return poisson_trace(count, rate=200.0, seed=seed, lo=5.0, hi=7.0, t_lo=0.02, t_hi=0.05)


@pytest.mark.parametrize("prec", [0, 1])
def test_each_result_is_the_same_alone_and_in_the_mix(cuda_lib, prec):
    trace = small_trace()
    scheme = serving_scheme(prec)
    # three slots and a pool for about three of the larger requests: requests queue, join while
    # others run, and reuse freed slots and memory
    biggest = max(Ensemble.member_bytes(r.block, prec) for r in trace)
    srv = Server(prec, hbm_budget=3 * biggest + (1 << 20), capacity=3, chunk=2)
    try:
        srv.run(trace, realtime=False)
    finally:
        srv.close()
    assert srv.max_running == 3           # the slots fill up: requests share the device
    overlapped = sum(1 for a in trace for b in trace if a.rid < b.rid and b.admitted < a.done)
    assert overlapped > 0
    ok = 0
    for r in trace:
        ref, t_ref, steps_ref, st_ref = solve_alone(r, scheme)
        # random quadrant states: the unlimited scheme fails on some of them at the first step,
        # alone as in the mix (the oracle too); such a request leaves with the error code
        assert (r.error != 0) == (st_ref != 0), (r.rid, r.error, st_ref)
        if r.error:
            continue
        ok += 1
        assert r.t == pytest.approx(r.t_end, rel=1e-14)
        err = normwise(r.result, ref, 5).max()
        if prec == 0:
            assert r.steps == steps_ref
            assert err <= PARITY_TOL, (r.rid, r.kind, r.n, err)
        else:
            assert abs(r.steps - steps_ref) <= 1
            assert err <= MIXED_TOL, (r.rid, r.kind, r.n, err)
    assert ok >= len(trace) - 3
    s = summary(trace)
    assert s["errors"] == len(trace) - ok and s["p99_s"] >= s["p50_s"] > 0


def test_realtime_trace_reports_latency(cuda_lib):
    trace = small_trace(6, seed=11)
    srv = Server(1, hbm_budget=1 << 30, capacity=8, chunk=16, keep_results=False)
    try:
        srv.run(trace, realtime=True)
    finally:
        srv.close()
    s = summary(trace, device_ms=srv.device_ms)
    assert s["requests"] == 6 and s["errors"] == 0  # the seed-11 trace has no failing request
    assert all(r.done >= r.arrival for r in trace)
    assert s["cell_updates_per_s"] > 0 and s["device_s"] > 0
