"""Checkpoint files in the reference's format (XFLUIDS::Output_Ubak / Read_Ubak) written and read
by the C ABI, and the save / resume of resident serving state built on them."""
import numpy as np
import pytest

from helpers import riemann_small, sod_like
from xfluids_gb300 import cases, checkpoint
from xfluids_gb300.ensemble import Ensemble
from xfluids_gb300.fluid import Fluid
from xfluids_gb300.mesh import make_scheme
from xfluids_gb300.serve import Server, poisson_trace

pytestmark = pytest.mark.gpu


def test_handle_checkpoint_round_trip(cuda_lib, tmp_path):
    b, s, th, U, T = cases.isentropic_vortex(32)
    f = Fluid(b, s, th)
    f.InitialU(U, T)
    f.initialize()
    st, t, n = f.advance(3)
    U3 = f.get("U").reshape(-1)
    p = tmp_path / "vortex_CheckingPoint"
    f.write_checkpoint(p, n, t, 1.5)
    step, time, dur, V = checkpoint.read(p, b.ncell * 5)
    assert (step, time, dur) == (3, t, 1.5) and np.array_equal(V, U3)
    f.close()
    g = Fluid(b, s, th)
    assert g.read_checkpoint(p) == (3, t, 1.5)
    assert np.array_equal(g.get("U").reshape(-1), U3) and np.array_equal(g.get("U1").reshape(-1), U3)
    assert g.time == t
    g.close()
    # a file of another block is refused
    b2, s2, th2, U2, _ = cases.isentropic_vortex(16)
    h = Fluid(b2, s2, th2)
    with pytest.raises(Exception):
        h.read_checkpoint(p)
    h.close()


def _members():
    out = []
    for mk in (lambda: sod_like(96), lambda: riemann_small(40), lambda: cases.isentropic_vortex(24)):
        b, _, _, U, _ = mk()
        out.append((b, np.ascontiguousarray(U).reshape(-1)))
    return out


def test_ensemble_member_resumes_exactly(cuda_lib, tmp_path):
    scheme = make_scheme(cop=False, scheme_order=5)
    ms = _members()
    pool = sum(Ensemble.member_bytes(b, 0) for b, _ in ms) + (1 << 20)
    ref = Ensemble(scheme, capacity=4, pool_bytes=pool)
    e1 = Ensemble(scheme, capacity=4, pool_bytes=pool)
    e2 = Ensemble(scheme, capacity=4, pool_bytes=pool)
    try:
        sr = [ref.add(b, U, 1e300) for b, U in ms]
        s1 = [e1.add(b, U, 1e300) for b, U in ms]
        ref.advance(7)
        e1.advance(3)
        lams = [e1.write_checkpoint(q, tmp_path / f"m{q}.ckpt") for q in s1]
        s2 = [e2.add_checkpoint(b, tmp_path / f"m{q}.ckpt", 1e300, lam) for (b, _), q, lam in zip(ms, s1, lams)]
        assert [e2.status(q)["steps"] for q in s2] == [0, 0, 0]  # status is as of the last advance
        e2.advance(4)
        for a, c in zip(sr, s2):
            assert e2.status(c)["steps"] == ref.status(a)["steps"] == 7
            assert e2.status(c)["t"] == ref.status(a)["t"]
            assert np.array_equal(e2.get_state(c), ref.get_state(a))
    finally:
        ref.close(), e1.close(), e2.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_server_save_and_resume_gives_the_uninterrupted_results(cuda_lib, tmp_path, prec):
    trace = poisson_trace(8, seed=11, lo=5.0, hi=7.0, t_lo=0.02, t_hi=0.05)
    whole = Server(prec, hbm_budget=1 << 30, capacity=3, chunk=4)
    try:
        whole.run(trace, realtime=False)
    finally:
        whole.close()
    trace2 = poisson_trace(8, seed=11, lo=5.0, hi=7.0, t_lo=0.02, t_hi=0.05)
    first = Server(prec, hbm_budget=1 << 30, capacity=3, chunk=4)
    try:
        first.run(trace2, realtime=False, max_chunks=5)
        assert first.running and (first.pending or first.waiting)   # saved mid-run
        finished = {r.rid: r for r in trace2 if r.result is not None}
        first.save(tmp_path / "srv")
    finally:
        first.close()
    second = Server.resume(tmp_path / "srv")
    try:
        left = list(second.running.values()) + second.waiting + second.pending
        second.run(realtime=False)
    finally:
        second.close()
    for r in left:
        finished[r.rid] = r
    assert sorted(finished) == [r.rid for r in trace]
    for r in trace:
        q = finished[r.rid]
        assert q.steps == r.steps and q.t == r.t
        assert np.array_equal(q.result, r.result), r.rid
