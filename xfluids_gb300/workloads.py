"""Run one workload of the convective path on the GPU and print its rate (one JSON line).

    python -m xfluids_gb300.workloads vortex   --size 1024 --steps 10 [--precision mixed] [--positivity]
    python -m xfluids_gb300.workloads sod      --size 1024 --steps 100
    python -m xfluids_gb300.workloads mixing   --shape 256 128 64 --steps 2 [--precision mixed] [--viscous]
    python -m xfluids_gb300.workloads ensemble --members 32 --steps 4 [--precision mixed]
    python -m xfluids_gb300.workloads horizon  --size 1024 --periods 10

The horizon workload runs the 2D vortex for whole periods (t = 10 per period) in FP64 and in the
mixed form and reports the error of each against the exact vortex and of mixed against FP64.

Each run: initial state on the host, one warm-up step (captures the step graph), a reset to the
initial state, then the timed steps (CUDA events around the graph replays). The mixing layer reads
the thermo tables from a tables JSON (thermo.dump_tables), by default the one under tests/golden;
with --viscous it adds viscous stress, heat conduction and species diffusion with transport data
fitted by transport.fit_transport from a tables JSON, by default the one under tests/golden.
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np

from . import cases, thermo
from .abi import MIXED

_GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden")
DEFAULT_TABLES = os.path.join(_GOLDEN, "thermo_tables.json")
DEFAULT_TRANSPORT_TABLES = os.path.join(_GOLDEN, "transport_tables.json")


def single_grid(b, s, th, U, T, steps, device=0, transport=None):
    from .fluid import Fluid
    f = Fluid(b, s, th, device=device)
    try:
        if transport is not None:
            f.set_transport(transport)
        f.InitialU(U, T)
        f.initialize()
        f.advance(1)
        f.InitialU(U, T)
        f.initialize()
        f.time = 0.0
        st, t, k, ms = f.advance_timed(steps)
        phases = f.time_phases()  # device ms per phase of one more step, summed over its stages
    finally:
        f.close()
    cells = b.X_inner * b.Y_inner * b.Z_inner
    return {"status": st, "t": t, "steps": k, "ms": ms, "cells": cells, "cell_updates_per_s": cells * k / (ms * 1e-3),
            "phases_ms_per_step": phases}


def ensemble(members, steps, precision, device=0, tune=False):
    from . import autotune
    from .ensemble import Ensemble
    scheme, ms = cases.riemann_ensemble(members, seed=0, precision=precision)
    pool = sum(Ensemble.member_bytes(b, precision) for b, _ in ms) + 4096 * len(ms)
    e = Ensemble(scheme, capacity=len(ms), pool_bytes=pool, device=device)
    try:
        slots = [e.add(b, U, 0.25) for b, U in ms]
        e.advance(1)
        sched = autotune.tune(e, steps=1)[0] if tune else e.schedule()
        before = [e.status(q)["steps"] for q in slots]
        st, t_ms = e.advance(steps)
        work = sum(b.X_inner * b.Y_inner * (e.status(q)["steps"] - s0) for (b, _), q, s0 in zip(ms, slots, before))
    finally:
        e.close()
    return {"status": st, "members": len(ms), "steps": steps, "ms": t_ms, "cell_updates_per_s": work / (t_ms * 1e-3),
            "schedule": sched}


def _rel_l1(a, r):
    """L1 of a - r per conserved component, relative to the mean |r| of the density (rho, rho*E
    scaled by their own means; the momenta by the mean momentum magnitude)."""
    d = np.abs(a - r).mean(axis=0)
    scale = np.abs(r).mean(axis=0)
    mom = float(np.sqrt((r[:, 1:4] ** 2).sum(axis=1)).mean())
    scale[1:4] = mom
    return [float(x) for x in d / scale]


COMPONENTS = ["rho", "rho_u", "rho_v", "rho_w", "E"]


def per_component(a, r, names=COMPONENTS):
    """Difference of two inner-cell states per conserved component: L1 (mean |a - r|) and Linf
    (max |a - r|), each also relative to the component's own scale (mean |r| for L1, max |r| for
    Linf); components that are zero in r report their absolute values only. 'worst' names the
    component with the largest relative L1."""
    d = np.abs(np.asarray(a) - np.asarray(r))
    out = {}
    for q, nm in enumerate(names):
        mean, mx = float(np.abs(r[:, q]).mean()), float(np.abs(r[:, q]).max())
        l1, li = float(d[:, q].mean()), float(d[:, q].max())
        out[nm] = {"l1": l1, "linf": li, "l1_rel": l1 / mean if mean > 0 else None,
                   "linf_rel": li / mx if mx > 0 else None}
    rel = {k: v["l1_rel"] for k, v in out.items() if v["l1_rel"] is not None}
    out["worst"] = max(rel, key=rel.get) if rel else None
    return out


def vortex_horizon(n, periods=10, precisions=(0, MIXED), device=0, chunk=4096):
    """The 2D vortex n^2 advanced to t = 10 * periods (whole periods: the exact solution is the
    initial state) in each precision; per precision the steps, the device time, the L1 and Linf
    error of rho against the exact vortex and the drift of the total mass; for the mixed form the
    L1 of each component against the FP64 run (relative as in _rel_l1) and the normwise Linf."""
    from .fluid import Fluid
    t_end = 10.0 * periods
    out = {"workload": f"2D isentropic vortex {n}^2, {periods} periods (t = {t_end:g})"}
    finals = {}
    for prec in precisions:
        b, s, th, U, T = cases.isentropic_vortex(n, precision=prec)
        sl = b.inner_slices()
        inner = lambda a: a.reshape(b.Zmax, b.Ymax, b.Xmax, 5)[sl].reshape(-1, 5)
        f = Fluid(b, s, th, device=device)
        try:
            f.InitialU(U, T)
            f.initialize()
            t, k, ms, st = 0.0, 0, 0.0, 0
            while t < t_end and st == 0:
                st, t, kk, dms = f.advance_timed(chunk, t_end)
                k += kk
                ms += dms
            g = inner(f.get("U"))
        finally:
            f.close()
        u0 = inner(np.asarray(U, dtype=np.float64).reshape(-1))
        rho_ex = cases.isentropic_vortex_exact(b, t_end)[sl].reshape(-1)
        mass0, mass = np.ascontiguousarray(u0[:, 0]).sum(), np.ascontiguousarray(g[:, 0]).sum()
        finals[prec] = g
        out["fp64" if prec == 0 else ("mixed" if prec == MIXED else "strict")] = {
            "status": st, "t": t, "steps": k, "ms": ms,
            "cell_updates_per_s": n * n * k / (ms * 1e-3) if ms > 0 else 0.0,
            "l1_rho_vs_exact": float(np.abs(g[:, 0] - rho_ex).mean()),
            "linf_rho_vs_exact": float(np.abs(g[:, 0] - rho_ex).max()),
            "mass_drift_rel": float((mass - mass0) / mass0)}
    if 0 in finals and MIXED in finals:
        a, r = finals[MIXED], finals[0]
        out["mixed_vs_fp64"] = {
            "l1_rel": _rel_l1(a, r),
            "linf_normwise": float(max(np.abs(a[:, q] - r[:, q]).max() / np.abs(r[:, q]).max()
                                       for q in range(5) if np.abs(r[:, q]).max() > 0)),
            "per_component": per_component(a, r)}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workload", choices=["vortex", "sod", "mixing", "ensemble", "horizon"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--shape", type=int, nargs=3, default=[256, 128, 64])
    ap.add_argument("--members", type=int, default=32)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--precision", choices=["fp64", "mixed", "strict"], default="fp64")
    ap.add_argument("--tables", default=DEFAULT_TABLES)
    ap.add_argument("--viscous", action="store_true", help="mixing: viscous, heat and diffusion fluxes")
    ap.add_argument("--positivity", action="store_true", help="vortex / sod / mixing: positivity-preserving limiter")
    ap.add_argument("--transport-tables", default=DEFAULT_TRANSPORT_TABLES,
                    help="Lennard-Jones rows and collision integrals (transport.dump_transport_tables)")
    ap.add_argument("--tune", action="store_true", help="ensemble: run the schedule autotuner first")
    ap.add_argument("--periods", type=int, default=10, help="horizon: vortex periods (t = 10 per period)")
    ap.add_argument("--only", choices=["fp64", "mixed"], help="horizon: run one precision only")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    prec = {"fp64": 0, "mixed": MIXED, "strict": 2}[a.precision]
    if a.workload == "horizon":
        precs = (0, MIXED) if a.only is None else ((0,) if a.only == "fp64" else (MIXED,))
        print(json.dumps(vortex_horizon(a.size, a.periods, precisions=precs, device=a.device)))
        return 0
    if a.workload == "ensemble":
        out = ensemble(a.members, a.steps, prec, a.device, a.tune)
    else:
        if a.workload == "vortex":
            b, s, th, U, T = cases.isentropic_vortex(a.size, precision=prec)
        elif a.workload == "sod":
            b, s, th, U, T = cases.sod(a.size, precision=prec)
        else:
            th = thermo.load_thermal(cases.MIXING_SPECIES, 0, tables_json=a.tables)
            b, s, th, U, T = cases.mixing_layer(tuple(a.shape), thermal=th, precision=prec)
        s.positivity = int(a.positivity)
        tr = None
        if a.viscous:
            if a.workload != "mixing":
                raise SystemExit("--viscous needs a mixture (the mixing workload)")
            from . import transport
            s.viscous = 7
            tr = transport.fit_transport(cases.MIXING_SPECIES, th, 0, tables_json=a.transport_tables,
                                         inv_spacing=(b._dx, b._dy, b._dz))
        out = single_grid(b, s, th, U, T, a.steps, a.device, tr)
    out.update({"workload": a.workload, "precision": a.precision, "viscous": bool(a.viscous),
                "positivity": bool(a.positivity)})
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
