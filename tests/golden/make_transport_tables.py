"""Write tests/golden/transport_tables.json: the Lennard-Jones rows of the mixtures used by the
tests and the bench, and the collision-integral tables, read from the reference's runtime.dat
(this container). The fitted transport data of the viscous fixtures are checked against
xfluids_gb300.transport.fit_transport on these inputs (tests/test_transport_fit_cpu.py).

    python tests/golden/make_transport_tables.py [runtime.dat directory]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from xfluids_gb300 import transport  # noqa: E402

SPECIES = ["H2", "O2", "N2", "H2O", "AR"]


def main(runtime_dir=None):
    if not runtime_dir:
        from oracle.ref_runner import reference_root
        runtime_dir = os.path.join(reference_root() or "", "runtime.dat")
    out = os.path.join(HERE, "transport_tables.json")
    transport.dump_transport_tables(runtime_dir, SPECIES, out)
    print("wrote", out)


if __name__ == "__main__":
    main(*sys.argv[1:])
