"""Generate the golden fixtures tests/golden/*.npz from the reference's own build.

Each case is run stage by stage through the reference's class XFLUIDS / Fluid, compiled from the
unmodified reference sources by oracle/ref/build_ref.sh and driven by oracle/ref/ref_driver.cpp.
The fixture holds the inputs (U, T, block, scheme) and, after every RK stage of 2 steps, dt and the
inner-cell U and LU; the primitives after the last stage. Needs the reference sources ($XF_REFERENCE, else the default of oracle/ref/build_ref.sh).

usage: python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import helpers as H  # noqa: E402
from oracle.ref_runner import read_transport, run_reference  # noqa: E402
from xfluids_gb300 import cases  # noqa: E402
from xfluids_gb300.abi import ROE, GLF, SYMMETRY  # noqa: E402

CASES = {
    # name: (flavour, builder, domain)
    "vortex24_w5_llf": ("ncop_w5_llf", lambda: cases.isentropic_vortex(24), None),
    "sod64_w5_llf": ("ncop_w5_llf", lambda: cases.sod(64), None),
    "blast3d_w5_llf": ("ncop_w5_llf", lambda: H.blast3d((16, 8, 6)), (1.0, 0.6, 0.5)),
    "sod64_w7_llf": ("ncop_w7_llf", lambda: H.sod_like(64, order=7), None),
    "riemann20_w7_sym": ("ncop_w7_llf", lambda: H.riemann_small(20, order=7, bc=SYMMETRY), None),
    "riemann20_w5_roe": ("ncop_w5_roe", lambda: H.riemann_small(20, artificial=ROE), None),
    "blast3d_w5_glf": ("ncop_w5_glf", lambda: H.blast3d((16, 8, 6), artificial=GLF), (1.0, 0.6, 0.5)),
    "insert64_cop4_ghost_nasa_w5": ("cop4g_w5_llf_nasa", lambda: H.insert_st(64), (0.1, 1.0, 1.0)),
    "mixing5_12x8x6_janaf_w7": ("cop5_w7_llf_janaf", lambda: H.mixing_small((12, 8, 6)),
                                (0.01, 0.01 * 8 / 12, 0.01 * 6 / 12)),
    # WENO-CU6 (scheme order 6)
    "riemann20_cu6_llf": ("ncop_w6_llf", H.with_order(lambda: H.riemann_small(20), 6), None),
    "mixing5_12x8x6_janaf_cu6_roe": ("cop5_w6_roe_janaf",
                                     H.with_order(lambda: H.mixing_small((12, 8, 6), order=5, artificial=ROE), 6),
                                     (0.01, 0.01 * 8 / 12, 0.01 * 6 / 12)),
    # viscous + heat conduction + diffusion (fourth order), fitted transport data of the reference
    "visc_mixing5_12x8x6_janaf_w5": ("cop5_w5_llf_janaf_visc",
                                     H.with_viscous(lambda: H.mixing_small((12, 8, 6), order=5)),
                                     (0.01, 0.01 * 8 / 12, 0.01 * 6 / 12)),
    "visc_mixing5_16x12_janaf_w5": ("cop5_w5_llf_janaf_visc",
                                    H.with_viscous(lambda: H.mixing_small((16, 12, 0), order=5)),
                                    (0.01, 0.01 * 12 / 16, 1.0)),
    # PositivityPreserving on: cases where the limiter acts (without it the first two go negative)
    "pp_riemann88_32_w5_llf": ("ncop_w5_llf_pp", H.with_positivity(lambda: H.riemann_member(88, 32)), None),
    "pp_riemann1d108_w5_llf": ("ncop_w5_llf_pp", H.with_positivity(H.riemann1d_strong), None),
    "pp_mixing5_12x8x6_janaf_w5": ("cop5_w5_llf_janaf_pp",
                                   H.with_positivity(lambda: H.mixing_small((12, 8, 6), order=5)),
                                   (0.01, 0.01 * 8 / 12, 0.01 * 6 / 12)),
}


def block_fields(b):
    return {k: getattr(b, k) for k, _ in b._fields_ if k != "Boundarys"} | {"Boundarys": list(b.Boundarys)}


def main(only=None):
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    for name, (flav, mk, domain) in CASES.items():
        if only and name not in only:
            continue
        b, s, th, U, T = mk()
        tpath = os.path.join(HERE, ".transport.bin")
        recs = run_reference(flav, b, U, T, steps=2, domain=domain, transport_out=tpath if s.viscous else None)
        E = s.Emax
        out = {
            "flavour": flav, "U0": U, "T0": T if T is not None else np.zeros(0),
            "block": np.array(repr(block_fields(b))), "scheme": np.array(repr({k: getattr(s, k) for k, _ in s._fields_})),
            "dt": np.array([r["dt"] for r in recs]), "step": np.array([r["step"] for r in recs]),
            "flag": np.array([r["flag"] for r in recs]),
            "U": np.stack([H.inner_aos(b, r["U"], E) for r in recs]),
            "LU": np.stack([H.inner_aos(b, r["LU"], E) for r in recs]),
        }
        last = recs[-1]
        for nm in ("rho", "p", "u", "v", "w", "c", "H", "T", "y"):
            out["last_" + nm] = last[nm]
        if s.cop:
            out["species"] = np.array(cases.MIXING_SPECIES if s.num_species == 5 else ["H2", "O2", "AR", "N2"])
        if s.viscous:  # the reference's fitted transport data, the input of the viscous fluxes
            t = read_transport(tpath)
            os.remove(tpath)
            for k in ("visc", "therm", "dkj", "chara", "limits"):
                out["tr_" + k] = t[k]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(recs)} stages, {os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    main(sys.argv[1:])
