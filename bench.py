#!/usr/bin/env python3
"""Benchmark of the convective right-hand side: cell-updates/s of the 2D isentropic Euler vortex
(periodic [0,10]^2, 4096^2 cells, WENO5-JS + LLF, SSP-RK3, CFL 0.5), plain FP64 path (the headline
`value`) and the mixed-precision form (FP32 reconstruction, FP64 state) beside it.

One step = one full SSP-RK3 time step (3 stages, dt included) of the whole grid; one cell-update =
one inner cell advanced one step. The state (670 MB) is larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--size 4096]

--impl reference times the reference algorithm's CPU implementation (the oracle restatement,
OpenMP over all host threads) on the same workload. Under torchrun every rank advances its own
replica of the grid (replicas only: no data exchange); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# Algorithmic flops of the vortex workload (WENO5-JS LLF, single gas), counted once by running the
# oracle restatement with a counting scalar (+,-,*,/,sqrt,exp,log = 1; max/abs/compare = 0) on the
# 64^2 vortex: per x face, and per cell-update over all kernels of one SSP-RK3 step.
# tests/test_bench_cpu.py recounts both on the oracle and checks them.
FLOPS_PER_FACE_X = 1378.0
FLOPS_PER_CELL_UPDATE = 8711.78271484375
FLOP_COUNT_SIZE = 64
# Thermodynamic tables of the mixture workloads (NASA-9 / JANAF coefficients)
THERMO_JSON = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "thermo_tables.json")
# Lennard-Jones data and collision integrals of runtime.dat for the transport fits of the mixture
TRANSPORT_TABLES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                "transport_tables.json")
# DRAM bytes per face of the FP64 x-face kernel: 674.2 MB read + 152.8 MB written in one ncu
# capture of the 2048^2 vortex (4.196 M faces); traffic grows with the faces of a launch
NCU_FACE_BYTES_FP64 = (674.218496e6 + 152.813568e6) / (2049 * 2048)
# Warp instructions per cell and stage of the fused mixed stage kernel: 2979 thread instructions
# per cell (sass__inst_executed_per_opcode summed) / 32, ncu capture of the 2048^2 vortex
NCU_FUSED_WARP_INSTR_PER_CELL = 2979.0 / 32.0


def issue_roofline(device, cells, launch_ms, sm_mhz):
    """The fused mixed stage against the bound it meets, instruction issue: its warp instructions
    per launch (the ncu count per cell times the cells) over the launch time, against one warp
    instruction per cycle on each of the 4 schedulers of every SM at the measured SM clock."""
    import torch
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    achieved = cells * NCU_FUSED_WARP_INSTR_PER_CELL / (launch_ms * 1e-3)
    peak = nsm * 4 * sm_mhz * 1e6
    return {"bound": "instruction issue", "kernel": "k_fused_stage", "achieved": achieved, "peak": peak,
            "unit": "warp instructions/s", "frac": achieved / peak, "warp_instructions_per_cell": NCU_FUSED_WARP_INSTR_PER_CELL,
            "sms": nsm, "sm_mhz": sm_mhz}


def hbm_context(traffic_bytes, launch_ms, peaks_path=os.path.join(ROOT, "MEASURED_PEAKS.json")):
    """DRAM throughput of one launch of the dominant kernel (ncu traffic per launch over its
    CUDA-event time) against the measured HBM copy bandwidth of this GPU model, else 6.8 TB/s."""
    if traffic_bytes is None or not launch_ms:
        return None
    try:
        with open(peaks_path) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError, TypeError):
        peak, src = 6800.0, "of fallback (6.8 TB/s)"
    gbs = traffic_bytes / (launch_ms * 1e-3) / 1e9
    return {"dram_gbs": gbs, "hbm_peak_gbs": peak, "frac": gbs / peak, "peak_source": src}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    """Barrier + max-over-ranks for torchrun launches (no data-path collective)."""

    def __init__(self, world, local):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as td
            cuda = torch.cuda.is_available()
            if cuda:
                torch.cuda.set_device(local)
            td.init_process_group("nccl" if cuda else "gloo")
            self.td, self.torch = td, torch
            self.device = "cuda" if cuda else "cpu"

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=self.device)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.world == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=self.device)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in self.rows for q in range(4) if len(r) > 5 + q and r[5 + q] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(size, threads, min_seconds=10.0):
    """Oracle (restatement) on the host cores: steps of the size^2 vortex until min_seconds."""
    from oracle import xfo
    from xfluids_gb300 import cases
    xfo.set_threads(threads)
    b, s, th, U, T = cases.isentropic_vortex(size)
    o = xfo.Oracle(b, s, th, U, T)
    o.initialize()
    o.step()  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        o.step()
        n += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return size * size * n / el, n, el


def run_reference_arm(args, world, rank):
    if rank != 0:
        return 0
    from oracle import xfo
    threads = os.cpu_count() or 1
    xfo.set_threads(threads)
    from xfluids_gb300 import cases
    # every step is one full step of the whole grid; a grid whose warmup + steps would take longer
    # than the time budget is refused (an unavailable line), never shrunk
    probe_n = 1024
    rate, _, _ = cpu_baseline(probe_n, threads, min_seconds=2.0)
    n = args.size
    projected = (args.steps + args.warmup) * n * n / rate
    if projected > REFERENCE_ARM_BUDGET_S:
        print(json.dumps({"impl": "reference", "unavailable": f"{args.steps + args.warmup} steps of the {n}^2 vortex "
                          f"on {threads} host threads would take about {projected:.0f} s, above the "
                          f"{REFERENCE_ARM_BUDGET_S:.0f} s budget of this arm"}), flush=True)
        return 0
    b, s, th, U, T = cases.isentropic_vortex(n)
    o = xfo.Oracle(b, s, th, U, T)
    o.initialize()
    for _ in range(args.warmup):
        o.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step()
    el = time.perf_counter() - t0
    value = n * n * args.steps / el
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": vortex_workload(n), "precision": "fp64", "cells": n * n,
                   "parallelism": f"host threads x{threads}", "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps of the {n}^2 vortex after {args.warmup} warm-up steps"},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


_T0 = time.perf_counter()


def progress(what):
    """One progress line on stderr (the JSON result stays the only line on stdout)."""
    sys.stderr.write(f"[bench {time.perf_counter() - _T0:8.1f} s] {what}\n")
    sys.stderr.flush()


def vortex_workload(n):
    """The config.workload string of both arms."""
    return f"2D isentropic Euler vortex {n}^2, periodic [0,10]^2, WENO5-JS LLF, SSP-RK3, CFL 0.5"


REFERENCE_ARM_BUDGET_S = 600.0
TUNE_PAD_STEPS = 12  # steps of the schedule search, padded (the full search has 11 trials)


def bench_ensemble(args, local, members, scheme, precision):
    """Batched ensemble (256 independent 2D four-quadrant Riemann problems, N per side
    round(2^U[7,10]), WENO5 LLF, CFL 0.45): warm-up steps (graph capture), then args.steps fused
    steps of all members timed with CUDA events on the ensemble's stream."""
    from xfluids_gb300 import autotune
    from xfluids_gb300.ensemble import Ensemble
    scheme.precision = precision
    pool = sum(Ensemble.member_bytes(b, precision) for b, _ in members) + 4096 * len(members)
    e = Ensemble(scheme, capacity=len(members), pool_bytes=pool, device=local)
    try:
        slots = [e.add(b, U, 0.25) for b, U in members]
        assert None not in slots
        e.advance(args.warmup)
        # schedule search on the live ensemble (bit-identical results under every schedule); the
        # FP64 search is shorter, its steps cost ~15x more
        space = None if precision else [("tile_2d_large", [5, 6, 7]), ("tile_2d_small", [5, 6, 4]),
                                         ("fused_faces", [0, 1])]
        sched, rep = autotune.tune(e, steps=1, space=space, use_cache=False)
        if len(rep["trials"]) < TUNE_PAD_STEPS:  # both precisions reach the same step count
            e.advance(TUNE_PAD_STEPS - len(rep["trials"]))
        before = [e.status(q)["steps"] for q in slots]
        st, ms = e.advance(args.steps)
        info = [e.status(q) for q in slots]
        states = [e.get_state(q) for q in slots]
    finally:
        e.close()
    # cell-updates actually performed: a member stopped by a numerical error (no positivity
    # limiter on these states) does no further steps
    work = sum(b.X_inner * b.Y_inner * (i["steps"] - s0) for (b, _), i, s0 in zip(members, info, before))
    failed = [q for q, i in enumerate(info) if i["error"]]
    return {"value": work / (ms * 1e-3), "ms": ms, "cell_updates": work, "status": st,
            "failed_members": failed, "schedule": sched, "tuning_trials": len(rep["trials"]),
            "tuned_ms_per_step": [round(t[1], 3) for t in rep["trials"]]}, states


def bench_ensemble_solve(local, members, scheme, precision, chunk=256, max_chunks=120):
    """Whole solve of the batched ensemble to its end time t = 0.25: every member advanced until it
    is done; members that finished (or stopped on a numerical error) leave the launch tables after
    each chunk of graph-replayed steps. Device time (CUDA events) and wall time of the solve,
    cell-updates performed, the members stopped by an error; bounded by max_chunks, with members
    whose time stopped moving (dt = 0) reported as stalled and those left as unfinished."""
    from xfluids_gb300.ensemble import Ensemble
    scheme.precision = precision
    pool = sum(Ensemble.member_bytes(b, precision) for b, _ in members) + 4096 * len(members)
    e = Ensemble(scheme, capacity=len(members), pool_bytes=pool, device=local)
    failed, stalled, work, dev_ms, chunks = [], [], 0, 0.0, 0
    try:
        live = {e.add(b, U, 0.25): q for q, (b, U) in enumerate(members)}
        assert None not in live
        t_prev = {slot: 0.0 for slot in live}
        t0 = time.perf_counter()
        while live and chunks < max_chunks:
            _, ms = e.advance(chunk)
            dev_ms += ms
            chunks += 1
            for slot in list(live):
                info = e.status(slot)
                # a member whose time did not move over a whole chunk (dt = 0) would never finish
                stuck = not info["done"] and info["t"] <= t_prev[slot]
                t_prev[slot] = info["t"]
                if info["done"] or stuck:
                    q = live.pop(slot)
                    work += members[q][0].X_inner * members[q][0].Y_inner * info["steps"]
                    if info["error"]:
                        failed.append(q)
                    if stuck:
                        stalled.append(q)
                    e.remove(slot)
        wall = time.perf_counter() - t0
    finally:
        e.close()
    return {"t_end": 0.25, "device_s": dev_ms * 1e-3, "wall_s": wall, "cell_updates": work,
            "cell_updates_per_s": work / (dev_ms * 1e-3), "failed_members": sorted(failed), "chunks": chunks,
            "steps_per_chunk": chunk, "stalled_members": sorted(stalled), "unfinished_members": sorted(live.values())}


def bench_serving(local, count, precision, fp64_check_work=3e8):
    """Continuous-batching server on the first `count` requests of the seeded Poisson trace
    (mean 200 req/s, 1D and 2D Riemann solves, N per side round(2^U[8,11]), t_end U[0.1,0.3]);
    the smaller results are re-solved alone in FP64 for the error of the served precision."""
    from xfluids_gb300.fluid import Fluid
    from xfluids_gb300.mesh import empty_thermal
    from xfluids_gb300.serve import Server, poisson_trace, serving_scheme, summary
    warm = poisson_trace(2, seed=99, lo=6.0, hi=7.0, t_lo=0.01, t_hi=0.02)
    trace = poisson_trace(count, seed=0)
    srv = Server(precision, hbm_budget=48 << 30, capacity=64, chunk=16, device=local)
    try:
        srv.run(warm, realtime=False)
        srv.device_ms = 0.0

        def report(sv):
            if sv.chunks % 100 == 0:
                progress(f"serving: chunk {sv.chunks}, {len(sv.running)} running, {len(sv.waiting)} waiting, "
                         f"{len(sv.pending)} pending, device {sv.device_ms * 1e-3:.1f} s")
        srv.run(trace, realtime=True, progress=report)
        out = summary(trace, device_ms=srv.device_ms)
    finally:
        srv.close()
    l1, fp64_errors = [], []
    sc = serving_scheme(0)
    for r in trace:
        # requests the server stopped on a numerical error (no positivity limiter on these random
        # states) have no served result to compare
        if r.error or r.cells * r.steps > fp64_check_work:
            continue
        f = Fluid(r.block, sc, empty_thermal(), device=local)
        f.InitialU(r.U)
        f.initialize()
        t, st = 0.0, 0
        while t < r.t_end and st == 0:
            st, t, _ = f.advance(256, r.t_end)
        if st == 0:
            ref = f.get("U").reshape(r.block.Zmax, r.block.Ymax, r.block.Xmax, 5)[r.block.inner_slices()]
            got = r.result.reshape(r.block.Zmax, r.block.Ymax, r.block.Xmax, 5)[r.block.inner_slices()]
            l1.append(float(np.abs(got - ref).mean()))
        else:
            fp64_errors.append(r.rid)
        f.close()
    out.update({"requests_checked_vs_fp64": len(l1), "l1_vs_fp64_max": max(l1) if l1 else None,
                "fp64_recheck_errors": fp64_errors,
                "trace": f"first {count} requests, Poisson mean 200 req/s, seed 0",
                "sizes": [f"{r.kind}:{r.n}" for r in trace]})
    return out


def bench_mixing_layer(args, local, steps):
    """3D inert temporal mixing layer (512 x 256 x 256, 5 species H2/O2/N2/H2O/AR, 7-coefficient
    thermo of the reference's runtime.dat, WENO7 LLF), FP64 and mixed from the same state: one
    warm-up step (graph capture), a reset, then `steps` timed steps; relative L1 / Linf of the
    mixed state against the FP64 state at the same step count; the strict form (no contraction,
    the reference's operation order) beside the FP64 form (contracted face sweeps). The FP64 and
    mixed runs with viscous stress,
    heat conduction and species diffusion (the reference's fitted transport data) give the share of
    a step those terms add."""
    from xfluids_gb300 import thermo
    from xfluids_gb300.abi import MIXED
    from xfluids_gb300.fluid import Fluid
    th = thermo.load_thermal(cases_mod().MIXING_SPECIES, 0, tables_json=THERMO_JSON)
    b, s, th, U, T = cases_mod().mixing_layer((512, 256, 256), thermal=th)
    res, states = {}, {}
    from xfluids_gb300 import transport
    tr = transport.fit_transport(cases_mod().MIXING_SPECIES, th, 0, tables_json=TRANSPORT_TABLES,
                                 inv_spacing=(b._dx, b._dy, b._dz))
    for prec, visc in ((0, 0), (MIXED, 0), (2, 0), (0, 7), (MIXED, 7)):
        s.precision, s.viscous = prec, visc
        f = Fluid(b, s, th, device=local)
        if visc:
            f.set_transport(tr)
        f.InitialU(U, T)
        f.initialize()
        f.advance(1)
        f.InitialU(U, T)
        f.initialize()
        f.time = 0.0
        st, t, k, ms = f.advance_timed(steps)
        cells = b.X_inner * b.Y_inner * b.Z_inner
        key = {0: "fp64", MIXED: "mixed", 2: "fp64_strict"}[prec] + ("_viscous" if visc else "")
        res[key] = {"value": cells * k / (ms * 1e-3), "ms_per_step": ms / k, "steps": k, "status": st, "t": t}
        if not visc and prec != 2:
            states[prec] = f.get("U").reshape(b.Zmax, b.Ymax, b.Xmax, 9)[b.inner_slices()].reshape(-1, 9)
        f.close()
    s.viscous = 0
    for p in ("fp64", "mixed"):  # share of a step the viscous, heat and diffusion terms add
        res[p + "_viscous"]["viscous_share_of_step"] = 1.0 - res[p]["ms_per_step"] / res[p + "_viscous"]["ms_per_step"]
    d = np.abs(states[MIXED] - states[0])
    scale = np.abs(states[0]).mean(axis=0)
    live = scale > 0  # the H2O density is zero in this mixing layer (no reaction)
    names = ["rho", "rho_u", "rho_v", "rho_w", "E", "rho_Y_H2", "rho_Y_O2", "rho_Y_N2", "rho_Y_H2O"]
    # momentum components against the mean magnitude of the momentum vector (the transverse
    # components carry only the 1% noise, so their own mean is not their scale)
    mom = np.sqrt((states[0][:, 1:4] ** 2).sum(axis=1)).mean()
    from xfluids_gb300.workloads import per_component
    per = per_component(states[MIXED], states[0], names)
    vec_scale = np.array([scale[0], mom, mom, mom, scale[4]] + [scale[0]] * 4)
    l1_state = float((d[:, live].mean(axis=0) / vec_scale[live]).max())
    d, states[0], scale = d[:, live], states[0][:, live], scale[live]
    res.update({"workload": "3D temporal mixing layer 512x256x256, 5 species, WENO7-JS LLF, SSP-RK3, CFL 0.5",
                "cells": b.X_inner * b.Y_inner * b.Z_inner,
                "mixed_speedup_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                "l1_rel_mixed_vs_fp64": float((d.mean(axis=0) / scale).max()),
                "l1_state_rel_mixed_vs_fp64": l1_state,
                "l1_note": "l1_rel: per component over its own mean |U|; l1_state_rel: momentum components over the "
                           "mean momentum magnitude, species over the mean density",
                "per_component": per,
                "linf_rel_mixed_vs_fp64": float((d.max(axis=0) / np.abs(states[0]).max(axis=0)).max())})
    return res


def mixing_members(count=16, seed=7):
    """Members of the batched mixing-layer ensemble: `count` temporal mixing layers (the 5-species
    case of bench_mixing_layer, WENO7 LLF) of seeded sizes 32 a x 16 b x 16 c, a, b, c uniform in
    [4, 8] (about 2.4 M cells a member on average)."""
    from xfluids_gb300 import thermo
    th = thermo.load_thermal(cases_mod().MIXING_SPECIES, 0, tables_json=THERMO_JSON)
    rng = np.random.default_rng(seed)
    out, s = [], None
    for q in range(count):
        a, b_, c = (int(v) for v in rng.integers(4, 9, size=3))
        b, s, th, U, T = cases_mod().mixing_layer((32 * a, 16 * b_, 16 * c), thermal=th, seed=1234 + q)
        out.append((b, U, T))
    return s, th, out


def bench_mixing_ensemble(local, steps, count=16):
    """Batched ensemble of 3D mixing layers (mixing_members), FP64 and mixed: all members admitted,
    one warm-up step (graph capture), then `steps` batched steps timed with CUDA events; per
    component L1 of the mixed states against the FP64 ones after the same steps."""
    from xfluids_gb300.abi import MIXED
    from xfluids_gb300.ensemble import Ensemble
    from xfluids_gb300.workloads import per_component
    s, th, ms = mixing_members(count)
    res, states = {}, {}
    for prec in (0, MIXED):
        s.precision = prec
        pool = sum(Ensemble.member_bytes(b, prec, scheme=s) for b, _, _ in ms) + 4096 * len(ms)
        e = Ensemble(s, capacity=len(ms), pool_bytes=pool, device=local, thermal=th)
        try:
            slots = [e.add(b, U, 1e300, T=T) for b, U, T in ms]
            assert None not in slots
            e.advance(1)
            before = [e.status(q)["steps"] for q in slots]
            st, dev_ms = e.advance(steps)
            info = [e.status(q) for q in slots]
            states[prec] = [e.get_state(q) for q in slots]
        finally:
            e.close()
        work = sum(b.X_inner * b.Y_inner * b.Z_inner * (i["steps"] - s0) for (b, _, _), i, s0 in zip(ms, info, before))
        res["mixed" if prec else "fp64"] = {"value": work / (dev_ms * 1e-3), "ms_per_step": dev_ms / steps,
                                            "cell_updates": work, "status": st,
                                            "failed_members": [q for q, i in enumerate(info) if i["error"]]}
    names = ["rho", "rho_u", "rho_v", "rho_w", "E", "rho_Y_H2", "rho_Y_O2", "rho_Y_N2", "rho_Y_H2O"]
    inner = lambda b, x: x.reshape(b.Zmax, b.Ymax, b.Xmax, -1)[b.inner_slices()].reshape(-1, x.size // (b.Zmax * b.Ymax * b.Xmax))
    got = np.concatenate([inner(b, x)[:, :9] for (b, _, _), x in zip(ms, states[MIXED])])
    ref = np.concatenate([inner(b, x)[:, :9] for (b, _, _), x in zip(ms, states[0])])
    res.update({"workload": f"{count} temporal mixing layers (5 species, WENO7-JS LLF, SSP-RK3, CFL 0.5) of sizes "
                            "32a x 16b x 16c, a, b, c ~ U[4, 8] (seed 7), one batched launch per phase, CUDA-graph replay",
                "cells": sum(b.X_inner * b.Y_inner * b.Z_inner for b, _, _ in ms), "steps": steps,
                "sizes": [f"{b.X_inner}x{b.Y_inner}x{b.Z_inner}" for b, _, _ in ms],
                "mixed_speedup_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                "per_component_mixed_vs_fp64": per_component(got, ref, names)})
    return res


def accuracy_gpu(local, n=192, t_end=0.5):
    """FP64 and mixed runs of the 2D vortex n^2 to t_end on the GPU, free running (no
    resynchronisation); the inner-cell states are compared in the CPU leg (accuracy_vs_oracle)."""
    from xfluids_gb300.abi import MIXED
    from xfluids_gb300.fluid import Fluid
    cs = cases_mod()
    b, s, th, U, T = cs.isentropic_vortex(n)
    sl = b.inner_slices()
    runs = {"n": n, "t_end": t_end}
    for name, prec in (("fp64", 0), ("mixed", MIXED)):
        s.precision = prec
        f = Fluid(b, s, th, device=local)
        f.InitialU(U, T)
        f.initialize()
        tg, k, st = 0.0, 0, 0
        while tg < t_end and st == 0:
            st, tg, kk = f.advance(64, t_end)
            k += kk
        if st:
            raise RuntimeError(f"accuracy run {name} stopped with status {st} at t = {tg}")
        runs[name] = (k, f.get("U").reshape(b.Zmax, b.Ymax, b.Xmax, 5)[sl].reshape(-1, 5))
        f.close()
    return runs


def accuracy_vs_oracle(runs, threads):
    """CPU leg, as the checker: the oracle advances the same vortex to the same time; returns the
    drift of each GPU run against it and the density error of each against the exact vortex."""
    from oracle import xfo
    cs = cases_mod()
    n, t_end = runs["n"], runs["t_end"]
    xfo.set_threads(threads)
    b, s, th, U, T = cs.isentropic_vortex(n)
    o = xfo.Oracle(b, s, th, U, T)
    o.initialize()
    t, n_o = 0.0, 0
    while t < t_end:
        t, _ = o.step(t_end)
        n_o += 1
    sl = b.inner_slices()
    ref = o.get("U").reshape(b.Zmax, b.Ymax, b.Xmax, 5)[sl].reshape(-1, 5)
    rho_ex = cs.isentropic_vortex_exact(b, t_end)[sl].reshape(-1)
    out = {"workload": f"2D isentropic vortex {n}^2 to t = {t_end}", "steps": n_o}
    for name in ("fp64", "mixed"):
        k, g = runs[name]
        d = np.abs(g - ref)
        out[name] = {"steps": k, "l1_vs_oracle": float(d.mean()),
                     "max_normwise_vs_oracle": float(max(d[:, q].max() / np.abs(ref[:, q]).max()
                                                         for q in range(5) if np.abs(ref[:, q]).max() > 0)),
                     "l1_rho_vs_exact": float(np.abs(g[:, 0] - rho_ex).mean()),
                     "linf_rho_vs_exact": float(np.abs(g[:, 0] - rho_ex).max())}
    out["oracle_l1_rho_vs_exact"] = float(np.abs(ref[:, 0] - rho_ex).mean())
    return out


def cpu_leg(threads, accuracy_runs=None, size=1024, min_seconds=10.0):
    """The CPU leg of the GPU arm (rank 0): the oracle restatement timed on the host cores
    (cpu_baseline: steps of the size^2 vortex for about min_seconds) and, when accuracy runs were
    made, the oracle as their checker."""
    val, steps, el = cpu_baseline(size, threads, min_seconds=min_seconds)
    acc = None if accuracy_runs is None else accuracy_vs_oracle(accuracy_runs, threads)
    return val, steps, el, acc


def cases_mod():
    from xfluids_gb300 import cases
    return cases


def run_gpu_arm(args, world, rank, local):
    from xfluids_gb300 import cases
    from xfluids_gb300.abi import MIXED
    from xfluids_gb300.fluid import Fluid, PinnedArray, measure_pipe_peaks, build_info
    d = Dist(world, local)
    n = args.size
    peaks = measure_pipe_peaks(local)
    fpf, flops_per_cu = FLOPS_PER_FACE_X, FLOPS_PER_CELL_UPDATE

    def setup(precision):
        b, s, th, U, T = cases.isentropic_vortex(n, precision=precision)
        f = Fluid(b, s, th, device=local)
        f.InitialU(U, T)
        f.initialize()
        return f, b, U

    def reset(fl, U):
        fl.InitialU(U)
        fl.initialize()
        fl.time = 0.0

    # ---- plain FP64 path: device-timed value --------------------------------------------------
    progress("plain FP64 vortex")
    f, b, U0 = setup(0)
    f.advance(args.warmup)          # warm-up (also captures the step graph)
    reset(f, U0)
    d.barrier()
    f.synchronize()
    with ClockSampler(local) as clk:
        st, t_end, k, ms = f.advance_timed(args.steps)
    d.barrier()
    ms = d.max(ms)
    cells_all = d.sum(n * n * k)
    value = cells_all / (ms * 1e-3)
    launches = f.launches_per_step * k
    phases = [f.time_phases() for _ in range(2)]
    ph = {key: float(np.mean([p[key] for p in phases])) for key in phases[0]}
    face_launch_ms = ph["faces_x"] / 3.0
    faces_per_launch = (n + 1) * n
    achieved = fpf * faces_per_launch / (face_launch_ms * 1e-3)
    U_fp64 = f.get("U")
    t_fp64 = f.time
    ms_total_fp64 = ms / k

    # ---- end to end through the public API with host buffers -----------------------------------
    progress("e2e through the C ABI")
    E = 5
    host = PinnedArray(U0.size)
    host.array[:] = U0.reshape(-1)
    e2e_steps = max(1, min(args.steps, 3))
    f2, _, _ = setup(0)
    f2.advance(1)
    # one untimed pass of the whole sequence: the first call of each kernel loads its module
    f2.InitialU(host.array)
    f2.initialize()
    f2.advance(1)
    f2.get("U", out=host.array)
    host.array[:] = U0.reshape(-1)
    f2.synchronize()
    d.barrier()
    parts = np.zeros(4)  # wall seconds of the four calls (each returns after its work is done)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        f2.InitialU(host.array)            # H2D of the step's input state
        tb = time.perf_counter()
        f2.initialize()
        tc = time.perf_counter()
        f2.advance(1)
        td = time.perf_counter()
        f2.get("U", out=host.array)         # D2H of the step's result into the pinned buffer
        it = (tb - ta, tc - tb, td - tc, time.perf_counter() - td)
        parts += it
        progress("e2e step: " + ", ".join(f"{1e3 * x:.1f}" for x in it) + " ms (set_state, states, advance, get)")
    el = time.perf_counter() - t0
    el = d.max(el)
    e2e_value = d.sum(n * n * e2e_steps) / el
    e2e_parts = parts
    bytes_state = U0.size * 8
    f2.close()
    host.close()

    # ---- mixed precision form, from the same initial state to the same final time ---------------
    progress("mixed vortex")
    fm, _, _ = setup(MIXED)
    fm.advance(args.warmup)
    reset(fm, U0)
    d.barrier()
    st_m, tm, km, ms_m = fm.advance_timed(args.steps + 16, t_fp64)
    ms_m = d.max(ms_m)
    value_mixed = d.sum(n * n * km) / (ms_m * 1e-3)
    Um = fm.get("U")
    Ui = U_fp64.reshape(b.Zmax, b.Ymax, b.Xmax, E)[b.inner_slices()]
    Umi = Um.reshape(b.Zmax, b.Ymax, b.Xmax, E)[b.inner_slices()]
    l1 = float(np.abs(Umi - Ui).mean())
    linf = float(np.abs(Umi - Ui).max())
    from xfluids_gb300.workloads import per_component
    mixed_components = per_component(Umi.reshape(-1, E), Ui.reshape(-1, E))
    phases_m = fm.time_phases()
    # the fused mixed stage kernel (one launch per stage) is reported in the faces_x phase
    mixed_face_ms = phases_m["faces_x"] / 3.0
    fm.close()
    f.close()

    # ---- batched ensemble, FP64 and mixed, and the serving trace -----------------------------
    ens = {}
    if args.ensemble:
        progress("batched ensemble")
        scheme_e, members = cases.riemann_ensemble(256, seed=0)
        e64, s64 = bench_ensemble(args, local, members, scheme_e, 0)
        emx, smx = bench_ensemble(args, local, members, scheme_e, MIXED)
        bad = set(e64["failed_members"]) | set(emx["failed_members"])
        diff = [np.abs(a - b_).reshape(members[q][0].Zmax, members[q][0].Ymax, members[q][0].Xmax, 5)[
                    members[q][0].inner_slices()].reshape(-1, 5)
                for q, (a, b_) in enumerate(zip(smx, s64)) if q not in bad]
        ncell_all = sum(x.shape[0] for x in diff)
        ens = {"workload": "256 independent 2D four-quadrant Riemann problems, N per side round(2^U[7,10]) (seed 0), "
                           "WENO5-JS LLF, SSP-RK3, CFL 0.45, one batched launch per phase, CUDA-graph replay",
               "cells": sum(b.X_inner * b.Y_inner for b, _ in members), "steps": args.steps,
               "fp64": e64, "mixed": emx, "members_compared": len(diff),
               "mixed_speedup_vs_fp64": emx["value"] / e64["value"],
               "mixed_speedup_vs_plain_fp64_vortex": emx["value"] / value,
               "l1_mixed_vs_fp64": float(sum(x.sum() for x in diff) / (ncell_all * 5)),
               "linf_mixed_vs_fp64": float(max(x.max() for x in diff))}
        del s64, smx, diff
        if args.ensemble_solve:
            progress("ensemble whole solve")
            ens["whole_solve_mixed"] = bench_ensemble_solve(local, members, scheme_e, MIXED)
    progress("serving trace")
    serving = bench_serving(local, args.serve_requests, MIXED) if args.serve_requests > 0 else None
    progress("mixing layer")
    mixing = bench_mixing_layer(args, local, args.mixing_steps) if args.mixing_steps > 0 else None
    if mixing is not None and args.mixing_ensemble > 0:
        progress("batched mixing-layer ensemble")
        mixing["batched_ensemble"] = bench_mixing_ensemble(local, args.mixing_steps, args.mixing_ensemble)
        for p in ("fp64", "mixed"):
            mixing["batched_ensemble"][p]["vs_single_grid"] = mixing["batched_ensemble"][p]["value"] / mixing[p]["value"]
    progress("accuracy runs")
    accuracy_runs = accuracy_gpu(local) if args.accuracy else None
    d.close()
    if rank != 0:
        return 0

    fp64_peak = peaks["fp64_flops"] / 1e12
    traffic = None if NCU_FACE_BYTES_FP64 is None else NCU_FACE_BYTES_FP64 * faces_per_launch
    cpu_threads = os.cpu_count() or 1
    progress("CPU leg")
    cpu_val, cpu_steps, cpu_el, accuracy = cpu_leg(cpu_threads, accuracy_runs)
    progress("done")
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": k, "warmup": args.warmup, "ms_per_step": ms_total_fp64, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": vortex_workload(n), "precision": "fp64 (plain path)", "cells": n * n, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (state 670 MB)"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": bytes_state,
                "d2h_bytes_per_step": bytes_state, "steps": e2e_steps,
                "path": "xfg_set_state(pinned host U) + BoundaryCondition + UpdateFluidStates + xfg_advance(1) + xfg_get_array(U)",
                "ms_per_step_by_call": {k: float(v) * 1e3 / e2e_steps for k, v in
                                        zip(("set_state", "boundary_and_states", "advance", "get_array"), e2e_parts)}},
        "gpu_launches": launches,
        "roofline": {"bound": "fp64", "kernel": "k_faces<x> (FP64 characteristic WENO5 face flux)",
                     "achieved": achieved / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": achieved / 1e12 / fp64_peak, "traffic": traffic,
                     "traffic_note": "DRAM bytes per launch, ncu capture of the 2048^2 vortex scaled by faces",
                     "algorithmic_flops_per_face": fpf, "faces_per_launch": faces_per_launch,
                     "launch_ms": face_launch_ms,
                     "hbm": hbm_context(traffic, face_launch_ms),
                     "peak_source": "measured FP64 FMA chain on this GPU (xfg_measure_pipe_peaks); MEASURED_PEAKS.json has no FP64 figure"},
        "phases_ms_per_step": ph,
        "mixed": {"value": value_mixed, "unit": "cell-updates/s", "speedup_vs_fp64": value_mixed / value,
                  "steps": km, "l1_vs_fp64": l1, "linf_vs_fp64": linf, "t": tm,
                  "per_component_vs_fp64": mixed_components,
                  "fused_stage_launch_ms": mixed_face_ms, "phases_ms_per_step": phases_m,
                  "roofline": {"bound": "fp32 (instruction issue)", "kernel": "k_fused_stage (2D mixed RK stage)",
                               "achieved": FLOPS_PER_CELL_UPDATE / 3.0 * n * n / (mixed_face_ms * 1e-3) / 1e12,
                               "peak": peaks["fp32_flops"] / 1e12, "unit": "TFLOP/s",
                               "frac": FLOPS_PER_CELL_UPDATE / 3.0 * n * n / (mixed_face_ms * 1e-3) / peaks["fp32_flops"],
                               "note": "algorithmic flops of one RK stage (the oracle's count, a third of a "
                                       "cell-update's) over the launch time; peak: measured scalar FP32 FMA chain"},
                  "fp32_peak_tflops": peaks["fp32_flops"] / 1e12,
                  "issue_roofline": issue_roofline(local, n * n, mixed_face_ms, peaks["sm_clock_mhz"])},
        "ensemble": ens or None,
        "serving": serving,
        "mixing_layer": mixing,
        "accuracy": accuracy,
        "cpu_baseline": {"value": cpu_val, "unit": "cell-updates/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"{cpu_steps} steps of the 1024^2 vortex ({cpu_el:.1f} s) on the oracle restatement"},
        "clocks": clk.summary(),
        "flops_per_cell_update": flops_per_cu,
        "build": build_info(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--ensemble", type=int, default=1, help="run the 256-member batched ensemble (0 = skip)")
    ap.add_argument("--ensemble-solve", type=int, default=1, help="whole mixed solve of the ensemble to t = 0.25 (0 = skip)")
    ap.add_argument("--serve-requests", type=int, default=100, help="requests of the serving trace (0 = skip)")
    ap.add_argument("--mixing-steps", type=int, default=2, help="timed steps of the 3D mixing layer (0 = skip)")
    ap.add_argument("--mixing-ensemble", type=int, default=16, help="members of the batched mixing-layer ensemble (0 = skip)")
    ap.add_argument("--accuracy", type=int, default=1, help="FP64 drift vs the oracle and error vs the exact vortex")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference_arm(args, world, rank)
    return run_gpu_arm(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
