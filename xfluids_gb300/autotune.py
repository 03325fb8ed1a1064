"""Autotuner of the batched ensemble's launch schedule.

The knobs are the options of xfg_ensemble_set_option: the face tile of each size class (how the
128 threads of a face block spread over x and the transverse direction), one fused launch for all
face sweeps of a stage or one per direction, the member order of the launch tables and the
number of fused steps per captured CUDA graph. No knob changes the operations a face, cell or
step computes, so the trials advance the live ensemble and their steps are steps of the solve
itself. FP64 results are bit-identical under every schedule; mixed-precision results agree to FP32
rounding (the compiler may contract an FP32 a*b+c into an FMA differently in each kernel form).

Search: coordinate descent over the knobs in a fixed order; each candidate value is timed over
`steps` fused steps with CUDA events on the ensemble's stream, with the other knobs at their best
so far. Knobs of size classes the ensemble does not contain are skipped. The winner is cached in a
JSON file (XFG_TUNE_CACHE, default ~/.cache/xfluids_gb300/ensemble_schedule.json) under a key made
of the device, precision, scheme order and the ensemble's size-class histogram.
"""
from __future__ import annotations

import json
import math
import os
from collections import Counter

from .ensemble import Ensemble

SPACE = [
    ("tile_2d_large", [5, 6, 7, 4, 3]),
    ("tile_2d_small", [5, 6, 7, 4]),
    ("tile_3d", [5, 6, 4]),
    ("tile_1d", [7, 6, 5]),
    ("fused_faces", [0, 1]),
    ("largest_first", [1, 0]),
    ("graph_steps", [1, 4]),
]


def size_class(block) -> str:
    dims = block.DimX + block.DimY + block.DimZ
    if dims == 1:
        return "tile_1d"
    if dims == 3:
        return "tile_3d"
    return "tile_2d_small" if max(block.X_inner, block.Y_inner, block.Z_inner) < 384 else "tile_2d_large"


def signature(ens: Ensemble, device_name: str = "") -> str:
    """Device, precision, order and a histogram of members by size class and log2 of their cells."""
    h = Counter((size_class(b), int(round(math.log2(max(1, b.X_inner * b.Y_inner * b.Z_inner)))))
                for b in ens.blocks.values())
    hist = ",".join(f"{c}:{k}:{n}" for (c, k), n in sorted(h.items()))
    return f"{device_name}|p{ens.scheme.precision}|o{ens.scheme.scheme_order}|{hist}"


def cache_path() -> str:
    return os.environ.get("XFG_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "xfluids_gb300",
                                                            "ensemble_schedule.json")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, key, value):
    data = _load(path)
    data[key] = value
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(ens: Ensemble, steps: int = 2, space=None, use_cache: bool = True, device_name: str = ""):
    """Pick the fastest schedule for this ensemble and leave it set. Returns (schedule, report):
    report = {"source": "cache" | "search", "trials": [(schedule, ms per step), ...], "key": ...}."""
    space = SPACE if space is None else space
    key = signature(ens, device_name)
    path = cache_path()
    if use_cache:
        hit = _load(path).get(key)
        if hit:
            ens.set_schedule(hit["schedule"])
            return hit["schedule"], {"source": "cache", "key": key, "trials": [], "ms_per_step": hit["ms_per_step"]}
    present = {size_class(b) for b in ens.blocks.values()}
    best = ens.schedule()
    trials = []

    def timed(sched):
        ens.set_schedule(sched)
        _, ms = ens.advance(steps)
        per = ms / steps
        trials.append((dict(sched), per))
        return per

    best_ms = timed(best)
    for knob, values in space:
        if knob.startswith("tile_") and knob not in present:
            continue
        for v in values:
            if v == best[knob]:
                continue
            cand = dict(best, **{knob: v})
            ms = timed(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    ens.set_schedule(best)
    if use_cache:
        _store(path, key, {"schedule": best, "ms_per_step": best_ms})
    return best, {"source": "search", "key": key, "trials": trials, "ms_per_step": best_ms}
