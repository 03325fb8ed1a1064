"""The C++ replacement of the reference's src/Fluids.cpp (xfluids_gb300/host/Fluids_gb300.cpp)
compiles against the reference's unmodified headers and links with its main.cpp, XFLUIDS.cpp and
read_ini objects and libxfluids_gb300.so: for the single gas and for the viscous 5-species mixture
(the #if Visc branch that passes Setup's fitted transport data). Runs where the reference sources
and its objects (oracle/ref/build_ref.sh) are present."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.ref_runner import reference_root

REF = reference_root() or ""
OUT = os.path.join(ROOT, "oracle", "_ref")
LIB = os.path.join(ROOT, "xfluids_gb300", "_build", "libxfluids_gb300.so")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")
def test_dropin_builds_and_links_against_the_reference():
    for flav in ("ncop_w5_llf", "cop5_w5_llf_janaf_visc"):
        if not os.path.isdir(os.path.join(OUT, flav, "obj")):
            pytest.skip(f"reference objects of {flav} not built (oracle/ref/build_ref.sh)")
    if not os.path.exists(LIB):
        pytest.skip("libxfluids_gb300.so not built")
    for flav in ("ncop_w5_llf", "cop5_w5_llf_janaf_visc"):
        exe = os.path.join(OUT, "dropin_" + flav, "xfluids_gb300_dropin")
        if os.path.exists(exe):
            os.remove(exe)
    r = subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref", "build_ref.sh"), "dropin"],
                       capture_output=True, text=True, env={**os.environ, "XF_REFERENCE": REF})
    assert r.returncode == 0, r.stderr[-3000:]
    for flav in ("ncop_w5_llf", "cop5_w5_llf_janaf_visc"):
        assert os.path.exists(os.path.join(OUT, "dropin_" + flav, "xfluids_gb300_dropin")), r.stdout
