"""Continuous-batching request server for independent solves.

A request is one XFLUIDS run of its own grid to its own end time (a 1D two-state or a 2D
four-quadrant Riemann problem, WENO5 LLF, SSP-RK3). Requests arrive on a seeded Poisson trace.
The server owns one Ensemble whose device pool is the HBM budget; the state of every admitted
request stays resident on the device until it finishes. The loop alternates

  1. admit: waiting requests, in arrival order, take a slot while a slot and pool memory are free
     (xfg_ensemble_add, which also runs the request's first BoundaryCondition + UpdateStates);
  2. run: `chunk` fused steps of every admitted request, one batched launch sequence per step,
     replayed from a CUDA graph (re-captured only when membership changed);
  3. retire: requests that reached their end time are copied out and leave, freeing their slot
     and memory for the queue.

Requests arriving while others run are admitted at the next chunk boundary, so their work
overlaps on the device with the requests already running. Time to solution = completion time -
arrival time (queueing + service), measured on the host wall clock from the trace start. In
replay mode (realtime=False, for tests) one request joins per chunk and its clock starts when it
joins.
"""
from __future__ import annotations

import argparse
import json
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import cases, checkpoint
from .abi import LLF, Block
from .ensemble import Ensemble
from .mesh import make_scheme


# error code of a request retired because its time stopped advancing (dt = 0)
STALLED = 30000


@dataclass
class Request:
    rid: int
    kind: str            # "1d" or "2d"
    n: int               # cells per side
    t_end: float
    arrival: float       # seconds after the trace start
    block: object = None
    U: np.ndarray = None
    # filled by the server
    start: float = float("nan")     # arrival on the server clock (the enqueue time in replay mode)
    admitted: float = float("nan")
    done: float = float("nan")
    steps: int = 0
    t: float = 0.0
    error: int = 0
    t_seen: float = -1.0            # the time reported after the previous chunk
    result: np.ndarray = field(default=None, repr=False)

    @property
    def cells(self) -> int:
        return self.n if self.kind == "1d" else self.n * self.n

    @property
    def tts(self) -> float:
        return self.done - self.start


def make_request(rid, kind, n, t_end, arrival, rng, precision=0) -> Request:
    """Build the grid and initial state of one request; states are drawn like the ensemble's
    (rho in U[0.1,2], u,v in U[-1,1], p in U[0.05,2])."""
    if kind == "1d":
        q = cases.riemann_states(rng)
        b, _, _, U, _ = cases.riemann1d(n, (q[0, 0], q[0, 1], q[0, 3]), (q[1, 0], q[1, 1], q[1, 3]),
                                        precision=precision)
    else:
        b, _, _, U, _ = cases.riemann2d(n, cases.riemann_states(rng), precision=precision)
    return Request(rid, kind, int(n), float(t_end), float(arrival), b, np.ascontiguousarray(U).reshape(-1))


def poisson_trace(count, rate=200.0, seed=0, lo=8.0, hi=11.0, frac_2d=0.5, t_lo=0.1, t_hi=0.3, n_max=None):
    """The first `count` requests of a seeded Poisson stream: exponential inter-arrival times of
    mean 1/rate, 1D or 2D with probability frac_2d, cells per side round(2^U[lo,hi]), end time
    U[t_lo,t_hi]. n_max caps the size (small test traces only)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        kind = "2d" if rng.uniform() < frac_2d else "1d"
        n = int(np.rint(2.0 ** rng.uniform(lo, hi)))
        if n_max:
            n = min(n, n_max)
        out.append(make_request(rid, kind, n, rng.uniform(t_lo, t_hi), t, rng))
    return out


def serving_scheme(precision=0):
    return make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=precision)


class Server:
    def __init__(self, precision=0, hbm_budget=32 << 30, capacity=64, chunk=16, device=0, keep_results=True):
        self.precision, self.hbm_budget, self.capacity, self.chunk, self.device = precision, int(hbm_budget), capacity, \
            chunk, device
        self.scheme = serving_scheme(precision)
        self.ens = Ensemble(self.scheme, capacity=capacity, pool_bytes=int(hbm_budget), device=device)
        self.keep = keep_results
        self.device_ms = 0.0
        self.chunks = 0
        self.max_running = 0
        self.pending, self.waiting, self.running = [], [], {}
        self.elapsed0 = 0.0   # server clock at the start of this process (non-zero after a resume)

    def close(self):
        self.ens.close()

    def run(self, trace=None, realtime=True, max_chunks=None, progress=None):
        """Serve the submitted requests (and `trace`, Requests sorted by arrival) until all are
        done, or for at most `max_chunks` chunks. realtime=False replays the arrivals in order
        without waiting for the wall clock (tests). progress(server) is called after each chunk."""
        if trace is not None:
            self.pending.extend(trace)
        pending, waiting, running = self.pending, self.waiting, self.running
        t0 = time.perf_counter() - self.elapsed0
        now = lambda: time.perf_counter() - t0
        self._now = now
        done_chunks = 0
        while pending or waiting or running:
            if max_chunks is not None and done_chunks >= max_chunks:
                break
            clock = now()
            while pending and (pending[0].arrival <= clock or not realtime):
                r = pending.pop(0)
                r.start = r.arrival if realtime else clock
                waiting.append(r)
                if not realtime:
                    break
            # admit in arrival order while slots and memory allow
            while waiting:
                r = waiting[0]
                if Ensemble.member_bytes(r.block, self.scheme.precision) > self.ens.pool_bytes:
                    raise ValueError(f"request {r.rid} ({r.kind} {r.n}) does not fit the HBM budget")
                slot = self.ens.add(r.block, r.U, r.t_end)
                if slot is None:
                    break
                r.admitted = now()
                running[slot] = waiting.pop(0)
            if not running:
                if pending and realtime:
                    time.sleep(max(0.0, pending[0].arrival - now()))
                continue
            self.max_running = max(self.max_running, len(running))
            _, ms = self.ens.advance(self.chunk)
            self.device_ms += ms
            self.chunks += 1
            done_chunks += 1
            clock = now()
            for slot in list(running):
                st = self.ens.status(slot)
                # a request whose time did not move over a whole chunk (dt = 0: an infinite wave
                # speed) would never finish: it is retired with error STALLED
                stalled = not (st["done"] or st["error"]) and st["t"] <= running[slot].t_seen
                running[slot].t_seen = st["t"]
                if st["done"] or st["error"] or stalled or st["t"] >= running[slot].t_end:
                    r = running.pop(slot)
                    r.done, r.steps, r.t, r.error = clock, st["steps"], st["t"], STALLED if stalled else st["error"]
                    if self.keep:
                        r.result = self.ens.get_state(slot)
                    self.ens.remove(slot)
            if progress is not None:
                progress(self)
        self.elapsed0 = now()
        return trace

    # -- save / resume the server's resident state ---------------------------------------------
    def save(self, directory):
        """Write every unfinished request to `directory`: the running ones as checkpoint files of
        the reference's format taken from the device (step count, time, state) with the dt maxima
        of their next step, the queued ones as their initial state; plus manifest.json."""
        os.makedirs(directory, exist_ok=True)
        reqs = []
        for slot, r in self.running.items():
            path = os.path.join(directory, f"req{r.rid}.ckpt")
            lam = self.ens.write_checkpoint(slot, path)
            reqs.append(_req_record(r, "running", path, lam))
        for state, queue in (("waiting", self.waiting), ("pending", self.pending)):
            for r in queue:
                path = os.path.join(directory, f"req{r.rid}.ckpt")
                checkpoint.write(path, 0, 0.0, 0.0, r.U)
                reqs.append(_req_record(r, state, path, None))
        manifest = {"precision": self.precision, "hbm_budget": self.hbm_budget, "capacity": self.capacity,
                    "chunk": self.chunk, "elapsed": self.elapsed0, "requests": reqs}
        with open(os.path.join(directory, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1)

    @classmethod
    def resume(cls, directory, device=0, keep_results=True):
        """A server holding the saved requests: running ones re-admitted from their checkpoints
        (the steps they take next are the ones the saved server would have taken), queued ones
        queued again. Continue with run()."""
        with open(os.path.join(directory, "manifest.json")) as f:
            m = json.load(f)
        srv = cls(m["precision"], m["hbm_budget"], m["capacity"], m["chunk"], device, keep_results)
        srv.elapsed0 = m["elapsed"]
        for rec in m["requests"]:
            b = Block()
            for k, v in rec["block"].items():
                if k == "Boundarys":
                    for q in range(6):
                        b.Boundarys[q] = v[q]
                else:
                    setattr(b, k, v)
            r = Request(rec["rid"], rec["kind"], rec["n"], rec["t_end"], rec["arrival"], b, None)
            r.start, r.admitted = rec["start"], rec["admitted"]
            if rec["state"] == "running":
                slot = srv.ens.add_checkpoint(b, rec["path"], r.t_end, rec["lam"])
                if slot is None:
                    raise RuntimeError("a saved running request does not fit the restored server")
                srv.running[slot] = r
            else:
                r.U = checkpoint.read(rec["path"], b.ncell * 5)[3]
                (srv.waiting if rec["state"] == "waiting" else srv.pending).append(r)
        return srv


def _req_record(r, state, path, lam):
    b = r.block
    block = {k: getattr(b, k) for k, _ in b._fields_ if k != "Boundarys"} | {"Boundarys": list(b.Boundarys)}
    return {"rid": r.rid, "kind": r.kind, "n": r.n, "t_end": r.t_end, "arrival": r.arrival, "start": r.start,
            "admitted": r.admitted, "state": state, "path": path, "lam": lam, "block": block}


def summary(trace, wall_s=None, device_ms=None):
    tts = np.array([r.tts for r in trace])
    work = float(sum(r.cells * r.steps for r in trace))
    span = max(r.done for r in trace) - min(r.start for r in trace)
    out = {"requests": len(trace), "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
           "max_s": float(tts.max()), "makespan_s": float(span), "cell_updates": work,
           "cell_updates_per_s": work / span, "errors": int(sum(1 for r in trace if r.error)),
           # arrival rate the server sustains at this throughput: throughput / mean work per request
           "sustainable_rate_req_s": (work / span) / (work / len(trace)) if work > 0 else 0.0}
    if device_ms is not None:
        out["device_s"] = device_ms * 1e-3
    return out


def main():
    ap = argparse.ArgumentParser(description="serve a seeded Poisson trace of Riemann solves")
    ap.add_argument("--requests", type=int, default=12)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--budget-gb", type=float, default=32.0)
    ap.add_argument("--chunk", type=int, default=16)
    a = ap.parse_args()
    prec = 1 if a.precision == "mixed" else 0
    trace = poisson_trace(a.requests, a.rate, a.seed)
    srv = Server(prec, hbm_budget=int(a.budget_gb * (1 << 30)), chunk=a.chunk, keep_results=False)
    try:
        srv.run(trace)
        s = summary(trace, device_ms=srv.device_ms)
    finally:
        srv.close()
    s.update({"precision": a.precision, "rate": a.rate, "seed": a.seed})
    print(json.dumps(s))


if __name__ == "__main__":
    main()
