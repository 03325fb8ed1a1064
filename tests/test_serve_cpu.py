"""Host logic of the request server (xfluids_gb300/serve.py) against a fake ensemble: requests join
in arrival order while slots are free, finished ones leave after their chunk, and a request whose
time stops advancing over a chunk (dt = 0) is retired with error STALLED instead of holding the
server forever. The bench's whole-ensemble solve loop (bench.bench_ensemble_solve) bounds itself
the same way."""
import numpy as np

from xfluids_gb300 import serve
from xfluids_gb300.mesh import make_block


class FakeEnsemble:
    """Every member advances by dt per step until its target; a member whose dt is 0 never moves."""

    pool_bytes = 1 << 40

    def __init__(self, capacity, dts):
        self.capacity, self.dts = capacity, dts  # dt of each request id
        self.slots = {}

    def add(self, block, U, t_end):
        if len(self.slots) >= self.capacity:
            return None
        slot = min(set(range(self.capacity)) - set(self.slots))
        self.slots[slot] = {"rid": int(U[0]), "t": 0.0, "t_end": t_end, "steps": 0}
        return slot

    def advance(self, n):
        for m in self.slots.values():
            for _ in range(n):
                if m["t"] >= m["t_end"]:
                    break
                m["t"] = min(m["t_end"], m["t"] + self.dts[m["rid"]])
                m["steps"] += 1
        return 0, 1.0

    def status(self, slot):
        m = self.slots[slot]
        return {"done": m["t"] >= m["t_end"], "error": 0, "t": m["t"], "steps": m["steps"]}

    def get_state(self, slot):
        return np.zeros(1)

    def remove(self, slot):
        del self.slots[slot]


def _server(capacity, dts):
    srv = object.__new__(serve.Server)
    srv.precision, srv.capacity, srv.chunk, srv.keep = 1, capacity, 4, True
    srv.scheme = serve.serving_scheme(1)
    srv.ens = FakeEnsemble(capacity, dts)
    srv.device_ms, srv.chunks, srv.max_running, srv.elapsed0 = 0.0, 0, 0, 0.0
    srv.pending, srv.waiting, srv.running = [], [], {}
    return srv


def _requests(n):
    b = make_block((16, 0, 0), (1.0, 1.0, 1.0), [2] * 6)
    return [serve.Request(rid=q, kind="1d", n=16, t_end=1.0, arrival=0.0, block=b, U=np.full(1, float(q)))
            for q in range(n)]


def test_requests_finish_in_admission_order_with_slot_limit():
    srv = _server(2, {0: 0.25, 1: 0.125, 2: 0.5})
    trace = _requests(3)
    srv.run(trace, realtime=False)
    assert all(r.error == 0 and r.t == 1.0 for r in trace)
    assert [r.steps for r in trace] == [4, 8, 2]
    assert srv.max_running == 2              # the third waited for a free slot
    assert trace[2].admitted >= trace[0].done


def test_a_request_whose_time_stops_is_retired_as_stalled():
    srv = _server(4, {0: 0.25, 1: 0.0, 2: 0.5})
    trace = _requests(3)
    srv.run(trace, realtime=False, max_chunks=50)
    assert not srv.running and not srv.waiting and not srv.pending
    assert trace[1].error == serve.STALLED and trace[1].t == 0.0
    assert trace[0].error == 0 and trace[2].error == 0 and trace[0].t == 1.0


def test_bench_whole_solve_reports_stalled_members(monkeypatch):
    import bench
    from xfluids_gb300 import ensemble

    class FakeEns(FakeEnsemble):
        def __init__(self, scheme, capacity, pool_bytes, device=0):
            super().__init__(capacity, {0: 0.125, 1: 0.0, 2: 0.25})

        @staticmethod
        def member_bytes(block, precision, scheme=None):
            return 1

        def close(self):
            pass

    monkeypatch.setattr(ensemble, "Ensemble", FakeEns)
    b = make_block((16, 16, 0), (1.0, 1.0, 1.0), [2] * 6)
    members = [(b, np.full(1, float(q))) for q in range(3)]
    out = bench.bench_ensemble_solve(0, members, serve.serving_scheme(1), 1, chunk=4, max_chunks=20)
    assert out["stalled_members"] == [1] and out["unfinished_members"] == [] and out["failed_members"] == []
    # the stalled member ran its first chunk (4 steps of dt = 0) before it was taken out
    assert out["cell_updates"] == 16 * 16 * (2 + 4 + 1) and out["chunks"] == 1
