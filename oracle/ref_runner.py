"""Run the reference binaries built by oracle/ref/build_ref.sh (test infrastructure).

run_reference(flavour, block, U, T, steps, t_end) writes the settings JSON the binary reads
(the reference's own JSON keys, src/read_ini/settings/read_json.cpp), the input state, runs the
reference's XFLUIDS/Fluid stage sequence through oracle/ref/ref_driver.cpp and returns the raw
FP64 arrays after every RK stage.
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
PRIMS = ["rho", "p", "u", "v", "w", "c", "H", "T"]

# flavour -> (Emax, NUM_SPECIES)
FLAVOURS = {
    "ncop_w5_llf": (5, 1), "ncop_w7_llf": (5, 1), "ncop_w5_roe": (5, 1), "ncop_w5_glf": (5, 1),
    "cop4g_w5_llf_nasa": (8, 4), "cop5_w7_llf_janaf": (9, 5),
    "ncop_w6_llf": (5, 1), "cop5_w6_roe_janaf": (9, 5),
    "cop5_w5_llf_janaf_visc": (9, 5),
    # built with PositivityPreserving on (-DPOSP=1, and the JSON key below)
    "ncop_w5_llf_pp": (5, 1), "cop5_w5_llf_janaf_pp": (9, 5),
}


def reference_root():
    """Location of the reference sources: $XF_REFERENCE, else the default of the build recipe
    (oracle/ref/build_ref.sh --root). None when no reference checkout is there."""
    root = os.environ.get("XF_REFERENCE")
    if not root:
        r = subprocess.run(["bash", os.path.join(HERE, "ref", "build_ref.sh"), "--root"], capture_output=True,
                           text=True)
        root = r.stdout.strip() if r.returncode == 0 else ""
    return root if root and os.path.isdir(os.path.join(root, "src")) else None


def available(flavour: str) -> bool:
    return os.access(os.path.join(REF_DIR, flavour, "xfluids_ref"), os.X_OK)


def _case_json(block, cfl, domain, positivity=False):
    res = [block.X_inner if block.DimX else 0, block.Y_inner if block.DimY else 0,
           block.Z_inner if block.DimZ else 0]
    return {
        "run": {"blockSize_x": 2, "blockSize_y": 2, "blockSize_z": 2, "DtBlockSize": 4, "nStepMax": 1000000,
                "nOutMax": 0, "OutInterval": 100000000, "OutBoundary": 0, "CFLnumber": cfl, "OutDAT": 0,
                "OutVTI": 0, "UseAdvRange": False, "OutTimeStamps": ["1000.0: {-C=X,0.0,0.0;-V=rho,P,T}"]},
        "mpi": {"mx": 1, "my": 1, "mz": 1, "DeviceSelect": [1, 0, 0]},
        "equations": {"Sources_React": False, "PositivityPreserving": bool(positivity)},
        "sources": {},
        "mesh": {"DOMAIN_Size": list(domain), "Resolution": res, "Boundarys": [int(b) for b in block.Boundarys],
                 "Ghost_width": [block.Bwidth_X or 4, block.Bwidth_Y or 4, block.Bwidth_Z or 4]},
        "init": {},
    }


def read_transport(path):
    """The fitted transport coefficients dumped by a viscous reference build (XFREF_TRANSPORT)."""
    raw = open(path, "rb").read()
    ns, order = struct.unpack_from("<ii", raw, 0)
    a = np.frombuffer(raw, dtype=np.float64, offset=8)
    o = 0
    out = {}
    for name, n in (("visc", ns * order), ("therm", ns * order), ("dkj", ns * ns * order), ("chara", ns * 9),
                    ("limits", 2)):
        out[name] = a[o:o + n].copy()
        o += n
    out["ns"], out["order"] = ns, order
    return out


def time_reference(flavour, block, U, T=None, steps=1, domain=None):
    """Seconds the reference build spends in `steps` time steps (its own clock around the step
    loop, no per-stage records) and its final U (AoS)."""
    E, NS = FLAVOURS[flavour]
    if not available(flavour):
        raise FileNotFoundError(f"reference flavour {flavour} is not built (oracle/ref/build_ref.sh)")
    if domain is None:
        domain = (block.dx * block.X_inner, block.dy * block.Y_inner, block.dz * block.Z_inner)
    N = block.ncell
    U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
    with open(os.path.join(REF_DIR, flavour, "case.json"), "w") as f:
        json.dump(_case_json(block, block.CFLnumber, domain), f)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<iqi", E, N, 1 if T is not None else 0))
            f.write(U.tobytes())
            if T is not None:
                f.write(np.ascontiguousarray(T, dtype=np.float64).tobytes())
        env = dict(os.environ, XFREF_IN=fin, XFREF_OUT=fout, XFREF_STEPS=str(steps), XFREF_TIMING="1")
        r = subprocess.run([os.path.join(".", flavour, "xfluids_ref")], cwd=REF_DIR, env=env, capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")
        line = [x for x in r.stdout.splitlines() if x.startswith("xfref_time")][-1].split()
        Uf = np.fromfile(fout, dtype=np.float64)
    return float(line[1]), int(line[2]), Uf


def run_reference(flavour, block, U, T=None, steps=1, t_end=1e300, domain=None, transport_out=None):
    """Returns a list of stage records {step, flag, dt, t, U, U1, LU, rho, ..., y}."""
    E, NS = FLAVOURS[flavour]
    exe_rel = os.path.join(".", flavour, "xfluids_ref")
    if not available(flavour):
        raise FileNotFoundError(f"reference flavour {flavour} is not built (oracle/ref/build_ref.sh)")
    if domain is None:
        domain = (block.dx * block.X_inner, block.dy * block.Y_inner, block.dz * block.Z_inner)
    N = block.ncell
    U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
    assert U.size == E * N
    with open(os.path.join(REF_DIR, flavour, "case.json"), "w") as f:
        json.dump(_case_json(block, block.CFLnumber, domain, positivity=flavour.endswith("_pp")), f)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<iqi", E, N, 1 if T is not None else 0))
            f.write(U.tobytes())
            if T is not None:
                f.write(np.ascontiguousarray(T, dtype=np.float64).tobytes())
        env = dict(os.environ, XFREF_IN=fin, XFREF_OUT=fout, XFREF_STEPS=str(steps), XFREF_TEND=repr(float(t_end)))
        if transport_out:
            env["XFREF_TRANSPORT"] = os.path.abspath(transport_out)
        r = subprocess.run([exe_rel], cwd=REF_DIR, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]} {r.stdout[-2000:]}")
        raw = open(fout, "rb").read()
    out, off = [], 0
    rec_doubles = 3 * E * N + len(PRIMS) * N + NS * N
    while off < len(raw):
        step, flag, dt, t = struct.unpack_from("<iidd", raw, off)
        off += 24
        a = np.frombuffer(raw, dtype=np.float64, count=rec_doubles, offset=off)
        off += 8 * rec_doubles
        rec = {"step": step, "flag": flag, "dt": dt, "t": t}
        p = 0
        for nm in ("U", "U1", "LU"):
            rec[nm] = a[p:p + E * N].copy()
            p += E * N
        for nm in PRIMS:
            rec[nm] = a[p:p + N].copy()
            p += N
        rec["y"] = a[p:p + NS * N].copy()
        out.append(rec)
    return out
