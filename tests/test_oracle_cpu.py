"""CPU checks of the oracle: conservation, free-stream preservation, analytic solutions, flop count."""
import math

import numpy as np
import pytest

import helpers as H
from oracle import xfo
from oracle.xfo import Oracle
from xfluids_gb300 import cases
from xfluids_gb300.abi import PERIODIC, LLF, ROE, GLF
from xfluids_gb300.mesh import make_block, make_scheme, empty_thermal


def _sums(b, o, E):
    return H.inner_aos(b, o.get("U"), E).sum(axis=0)


@pytest.mark.parametrize("order", [5, 7])
def test_periodic_conservation(order):
    b, s, th, U, T = cases.isentropic_vortex(48)
    s.scheme_order = order
    o = Oracle(b, s, th, U, T)
    o.initialize()
    m0 = _sums(b, o, 5)
    for _ in range(4):
        o.step()
    m1 = _sums(b, o, 5)
    scale = np.abs(H.inner_aos(b, o.get("U"), 5)).sum(axis=0)
    assert np.all(np.abs(m1 - m0) <= 1e-13 * scale)


@pytest.mark.parametrize("artificial", [LLF, ROE, GLF])
@pytest.mark.parametrize("order", [5, 7])
def test_free_stream_preserved(order, artificial):
    b = make_block((16, 12, 0), (1.0, 1.0, 1.0), [PERIODIC] * 6)
    s = make_scheme(scheme_order=order, artificial_type=artificial)
    n = b.ncell
    U = cases.conserved_ideal(np.full(n, 1.3), np.full(n, 0.7), np.full(n, -0.4), np.zeros(n), np.full(n, 2.1))
    o = Oracle(b, s, empty_thermal(), U)
    o.initialize()
    for _ in range(2):
        o.step()
    Ui = H.inner_aos(b, o.get("U"), 5)
    assert np.abs(Ui - U[: len(Ui)]).max() < 1e-13


def test_free_stream_mixture():
    b, s, th, U, T = H.mixing_small((12, 8, 6))
    n = b.ncell
    U = np.tile(U[len(U) // 2], (n, 1))  # one cell's state everywhere
    T = np.full(n, T[len(T) // 2])
    o = Oracle(b, s, th, U, T)
    o.initialize()
    o.step()
    Ui = H.inner_aos(b, o.get("U"), 9)
    assert np.abs(Ui - U[0]).max() / np.abs(U[0]).max() < 1e-12


def test_vortex_translates():
    """After t the exact solution is the initial vortex moved by (t, t) (periodic)."""
    n = 64
    b, s, th, U, T = cases.isentropic_vortex(n)
    o = Oracle(b, s, th, U, T)
    o.initialize()
    t_end = 0.5
    t = 0.0
    while t < t_end:
        t, _ = o.step(t_end)
    X, Y, _ = cases.cell_centres(b)
    xv = np.mod(X - t - 5.0 + 5.0, 10.0) - 5.0
    yv = np.mod(Y - t - 5.0 + 5.0, 10.0) - 5.0
    r2 = xv * xv + yv * yv
    rho_ex = (1.0 - 25.0 * np.exp(1.0 - r2) / 28.0 / math.pi ** 2) ** 2.5
    rho = o.get("U").reshape(b.Zmax, b.Ymax, b.Xmax, 5)[..., 0]
    sl = b.inner_slices()
    err = np.abs(rho[sl] - rho_ex[sl]).mean()
    assert err < 2e-3, err


@pytest.mark.parametrize("order", [5, 7])
def test_sod_against_exact(order):
    b, s, th, U, T = cases.sod(256, order=order)
    o = Oracle(b, s, th, U, T)
    o.initialize()
    t = 0.0
    while t < 0.2:
        t, _ = o.step(0.2)
    assert t == 0.2
    X, _, _ = cases.cell_centres(b)
    sl = b.inner_slices()
    rho = o.get("U").reshape(b.Zmax, b.Ymax, b.Xmax, 5)[..., 0][sl].ravel()
    ex = cases.sod_exact_density(X[sl].ravel(), 0.2)
    assert np.abs(rho - ex).mean() < 6e-3


def test_flop_count_per_face():
    b, s, th, U, T = cases.isentropic_vortex(32)
    c = xfo.count_flops(b, s, th, U, T, 1)
    per_face = c["faces_x"] / 3 / (33 * 32)
    assert 1000 < per_face < 2000
    assert c["faces_x"] == c["faces_y"]
    assert c["boundary"] == 0


def test_thermo_reader_matches_fixture():
    import os
    from xfluids_gb300 import thermo
    from oracle.ref_runner import reference_root
    root = reference_root()
    rt = os.path.join(root, "runtime.dat") if root else ""
    if not os.path.isdir(rt):
        pytest.skip("reference runtime.dat not present")
    for sp, k in [(cases.MIXING_SPECIES, 0), (["H2", "O2", "AR", "N2"], 1)]:
        a = thermo.load_thermal(sp, k, runtime_dir=rt)
        b = thermo.load_thermal(sp, k, tables_json=H.THERMO_JSON)
        assert bytes(a) == bytes(b)
