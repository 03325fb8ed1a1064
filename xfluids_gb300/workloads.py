"""Run one workload of the convective path on the GPU and print its rate (one JSON line).

    python -m xfluids_gb300.workloads vortex   --size 1024 --steps 10 [--precision mixed] [--positivity]
    python -m xfluids_gb300.workloads sod      --size 1024 --steps 100
    python -m xfluids_gb300.workloads mixing   --shape 256 128 64 --steps 2 [--precision mixed] [--viscous]
    python -m xfluids_gb300.workloads ensemble --members 32 --steps 4 [--precision mixed]

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
    finally:
        f.close()
    cells = b.X_inner * b.Y_inner * b.Z_inner
    return {"status": st, "t": t, "steps": k, "ms": ms, "cells": cells, "cell_updates_per_s": cells * k / (ms * 1e-3)}


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


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workload", choices=["vortex", "sod", "mixing", "ensemble"])
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
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    prec = {"fp64": 0, "mixed": MIXED, "strict": 2}[a.precision]
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
