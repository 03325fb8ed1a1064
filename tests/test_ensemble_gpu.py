"""Batched ensemble engine (xfg_ensemble_*, xfluids_gb300/ensemble.py).

Every member advanced inside the ensemble must equal the same grid advanced alone through the
single-grid path (Fluid.advance, itself parity-checked against the oracle): same number of steps,
same time, same state within the FP64 parity bound. Also: graph replay equals direct launches
bit for bit, members stop at their own target time, admission by slot and pool budget, slot reuse.
"""
import numpy as np
import pytest

from helpers import PARITY_TOL, blast3d, normwise, riemann_small, sod_like
from xfluids_gb300 import cases
from xfluids_gb300.abi import GLF, LLF, PERIODIC, ROE
from xfluids_gb300.ensemble import Ensemble
from xfluids_gb300.fluid import Fluid
from xfluids_gb300.mesh import empty_thermal, make_scheme

pytestmark = pytest.mark.gpu

FP64, MIXED = 0, 1
# mixed-precision members against the mixed single-grid path: the same FP32 expressions compiled
# into other kernels may contract differently into FMAs, so the two agree to FP32 rounding only
# (dt, and hence t, to about 1e-7 relative); bounds for state (normwise) and time:
MIXED_TOL = 1e-5
MIXED_T_TOL = 1e-6


def members():
    out = []
    for mk in (lambda: sod_like(96), lambda: cases.isentropic_vortex(32), lambda: riemann_small(40),
               lambda: blast3d(), lambda: riemann_small(24, seed=5, bc=PERIODIC)):
        b, _, _, U, _ = mk()
        out.append((b, np.ascontiguousarray(U, dtype=np.float64).reshape(-1)))
    return out


def alone(b, U, scheme, nsteps, target=1e300):
    f = Fluid(b, scheme, empty_thermal())
    try:
        f.InitialU(U)
        f.initialize()
        st, t, n = f.advance(nsteps, target)
        assert st == 0
        return f.get("U").reshape(-1), t, n
    finally:
        f.close()


def pool_for(blocks, precision, extra=0):
    return sum(Ensemble.member_bytes(b, precision) for b in blocks) + 4096 * len(blocks) + extra


@pytest.mark.parametrize("order,art,prec", [(5, LLF, FP64), (7, ROE, FP64), (5, ROE, FP64), (5, LLF, MIXED),
                                            (7, LLF, MIXED), (6, LLF, FP64), (6, ROE, MIXED), (5, GLF, FP64),
                                            (7, GLF, FP64), (5, GLF, MIXED)])
def test_members_equal_single_grid_runs(cuda_lib, order, art, prec):
    scheme = make_scheme(cop=False, scheme_order=order, artificial_type=art, precision=prec)
    ms = members()
    nsteps = 6
    # member 1 stops half way through: its target is half the time the free run reaches
    _, t_free, _ = alone(ms[1][0], ms[1][1], scheme, nsteps)
    targets = [1e300] * len(ms)
    targets[1] = 0.5 * t_free
    e = Ensemble(scheme, capacity=8, pool_bytes=pool_for([b for b, _ in ms], prec))
    try:
        slots = [e.add(b, U, tg) for (b, U), tg in zip(ms, targets)]
        assert None not in slots and e.active == len(ms)
        st, dev_ms = e.advance(nsteps)
        assert st == 0 and dev_ms > 0
        for (b, U), tg, s in zip(ms, targets, slots):
            ref, t_ref, n_ref = alone(b, U, scheme, nsteps, tg)
            info = e.status(s)
            got = e.get_state(s)
            assert info["error"] == 0
            assert info["steps"] == n_ref
            assert info["t"] == pytest.approx(t_ref, rel=1e-13 if prec == FP64 else MIXED_T_TOL, abs=0)
            err = normwise(got, ref, 5).max()
            assert err <= (PARITY_TOL if prec == FP64 else MIXED_TOL), (s, err)
        assert e.status(slots[1])["done"] and e.status(slots[1])["t"] == pytest.approx(targets[1], rel=1e-15)
        assert not e.status(slots[0])["done"]
    finally:
        e.close()


@pytest.mark.parametrize("prec", [FP64, MIXED], ids=["fp64", "mixed"])
def test_members_with_positivity_limiter_equal_single_grid_runs(cuda_lib, prec):
    """With the positivity limiter on, every member (among them member 88 of the seeded ensemble,
    whose first stage turns the density negative without the limiter) equals its single-grid run."""
    from helpers import riemann_member
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=prec, positivity=True)
    b88, _, _, U88, _ = riemann_member(88, 32)
    ms = [(b88, U88)] + members()[:3]
    nsteps = 6
    e = Ensemble(scheme, capacity=len(ms), pool_bytes=pool_for([b for b, _ in ms], prec))
    try:
        slots = [e.add(b, U, 1e300) for b, U in ms]
        st, _ = e.advance(nsteps)
        assert st == 0
        for (b, U), s in zip(ms, slots):
            ref, t_ref, n_ref = alone(b, U, scheme, nsteps)
            info = e.status(s)
            assert info["error"] == 0 and info["steps"] == n_ref == nsteps
            assert info["t"] == pytest.approx(t_ref, rel=1e-13 if prec == FP64 else MIXED_T_TOL, abs=0)
            err = normwise(e.get_state(s), ref, 5).max()
            assert err <= (PARITY_TOL if prec == FP64 else MIXED_TOL), (s, err)
    finally:
        e.close()


def run_ensemble(scheme, ms, nsteps, use_graph, largest_first=1, chunks=1, **sched):
    e = Ensemble(scheme, capacity=len(ms), pool_bytes=pool_for([b for b, _ in ms], scheme.precision))
    try:
        e.set_option("largest_first", largest_first)
        e.set_schedule(sched)
        slots = [e.add(b, U, 1e300) for b, U in ms]
        for _ in range(chunks):
            assert e.advance(nsteps // chunks, use_graph=use_graph)[0] == 0
        return [e.get_state(s) for s in slots], [e.status(s)["t"] for s in slots]
    finally:
        e.close()


def test_graph_replay_and_launch_order_are_bitwise_neutral(cuda_lib):
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=FP64)
    ms = members()
    direct, t_direct = run_ensemble(scheme, ms, 4, use_graph=False)
    graph, t_graph = run_ensemble(scheme, ms, 4, use_graph=True, chunks=2)
    slot_order, t_slot = run_ensemble(scheme, ms, 4, use_graph=True, largest_first=0)
    for a, b, c in zip(direct, graph, slot_order):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    assert t_direct == t_graph == t_slot
    # face tiles, the fused face launch and multi-step graphs (4 steps = one 3-step graph + 1)
    for sched in (dict(fused_faces=1), dict(tile_1d=5, tile_2d_small=7, tile_3d=6), dict(tile_2d_small=3, tile_3d=4),
                  dict(graph_steps=3, fused_faces=1, tile_1d=6, tile_2d_small=4)):
        other, t_other = run_ensemble(scheme, ms, 4, use_graph=True, **sched)
        for a, b in zip(direct, other):
            assert np.array_equal(a, b), sched
        assert t_other == t_direct


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_autotuner_picks_and_caches_a_schedule(cuda_lib, tmp_path, monkeypatch, prec):
    from xfluids_gb300 import autotune
    monkeypatch.setenv("XFG_TUNE_CACHE", str(tmp_path / "sched.json"))
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=prec)
    ms = members()
    e = Ensemble(scheme, capacity=len(ms), pool_bytes=pool_for([b for b, _ in ms], prec))
    try:
        slots = [e.add(b, U, 1e300) for b, U in ms]
        best, rep = autotune.tune(e, steps=1)
        assert rep["source"] == "search" and len(rep["trials"]) >= 8
        assert e.schedule() == best
        steps_tuning = e.status(slots[0])["steps"]
        assert steps_tuning == len(rep["trials"])      # trials advanced the live ensemble
        best2, rep2 = autotune.tune(e, steps=1)
        assert rep2["source"] == "cache" and best2 == best
        # the tuned run equals the single-grid runs over the same number of steps
        e.advance(2)
        for (b, U), s in zip(ms, slots):
            ref, _, _ = alone(b, U, scheme, steps_tuning + 2)
            assert normwise(e.get_state(s), ref, 5).max() <= (PARITY_TOL if prec == FP64 else MIXED_TOL)
    finally:
        e.close()


def test_admission_by_slot_and_pool_budget(cuda_lib):
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=FP64)
    ms = members()
    b0, U0 = ms[2]
    need = Ensemble.member_bytes(b0, FP64)
    # pool for one member only
    e = Ensemble(scheme, capacity=4, pool_bytes=need + 1024)
    try:
        s0 = e.add(b0, U0, 1e300)
        assert s0 is not None
        assert e.add(b0, U0, 1e300) is None          # no pool memory: admission waits
        e.remove(s0)
        assert e.free_bytes == need + 1024
        s1 = e.add(b0, U0, 1e300)                     # the slot and the memory are reused
        assert s1 is not None
        assert e.advance(2)[0] == 0
        ref, t_ref, _ = alone(b0, U0, scheme, 2)
        assert normwise(e.get_state(s1), ref, 5).max() <= PARITY_TOL
    finally:
        e.close()
    # capacity: two slots
    e = Ensemble(scheme, capacity=2, pool_bytes=pool_for([b0] * 3, FP64))
    try:
        assert e.add(b0, U0, 1e300) is not None and e.add(b0, U0, 1e300) is not None
        assert e.add(b0, U0, 1e300) is None           # no free slot
    finally:
        e.close()


def test_members_join_and_leave_between_advances(cuda_lib):
    """A member added after others have run equals its own run alone; removing a member does not
    disturb the others."""
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=FP64)
    ms = members()
    e = Ensemble(scheme, capacity=8, pool_bytes=pool_for([b for b, _ in ms], FP64))
    try:
        s = [e.add(*ms[q], 1e300) for q in range(3)]
        assert e.advance(3)[0] == 0
        e.remove(s[1])
        s3 = e.add(*ms[3], 1e300)
        assert e.advance(2)[0] == 0
        for slot, q, n in ((s[0], 0, 5), (s[2], 2, 5), (s3, 3, 2)):
            ref, t_ref, _ = alone(*ms[q], scheme, n)
            assert e.status(slot)["steps"] == n
            assert normwise(e.get_state(slot), ref, 5).max() <= PARITY_TOL
    finally:
        e.close()



def failing_member(n=32):
    """Member 88 of the seeded 256-member Riemann ensemble: the first RK stage of the unlimited
    characteristic WENO5 drives the density negative (the oracle shows the same at step 0)."""
    _, rng = cases.ensemble_sizes(256, 0)
    for _ in range(88):
        cases.riemann_states(rng)
    b, _, _, U, _ = cases.riemann2d(n, cases.riemann_states(rng))
    return b, np.ascontiguousarray(U).reshape(-1)


def test_member_with_numerical_error_stops_and_others_go_on(cuda_lib):
    scheme = make_scheme(cop=False, scheme_order=5, artificial_type=LLF, precision=FP64)
    ms = members()[:3]
    bad = failing_member()
    e = Ensemble(scheme, capacity=4, pool_bytes=pool_for([b for b, _ in ms] + [bad[0]], FP64))
    try:
        slots = [e.add(b, U, 1e300) for b, U in ms]
        sb = e.add(*bad, 1e300)
        st, _ = e.advance(4)
        assert st != 0                                   # worst member code is reported
        info = e.status(sb)
        assert info["error"] != 0 and info["done"] and info["steps"] == 1
        for (b, U), s in zip(ms, slots):
            ref, _, n_ref = alone(b, U, scheme, 4)
            assert e.status(s)["error"] == 0 and e.status(s)["steps"] == n_ref == 4
            assert normwise(e.get_state(s), ref, 5).max() <= PARITY_TOL
    finally:
        e.close()
    # the same grid alone reports the error too
    f = Fluid(bad[0], scheme, empty_thermal())
    try:
        f.InitialU(bad[1])
        f.initialize()
        st, _, _ = f.advance(1)
        assert st != 0
    finally:
        f.close()


def _mixture_members(order):
    """5-species JANAF mixtures of uneven sizes: three temporal mixing layers (3D) and a 2D block
    with walls and a periodic pair (the ragged mixture case of the random tests)."""
    from helpers import mixing_small
    from test_fuzz_gpu import _tiny_case
    out = []
    for shape in ((16, 12, 8), (24, 16, 8), (12, 20, 6)):
        b, s, th, U, T = mixing_small(shape, order=order)
        out.append((b, U, T))
    b, s, th, U, T = _tiny_case((5, 9, 0), (0.01, 0.013, 1.0), [4, 1, 3, 3, 0, 0], order, cop=True)
    out.append((b, U, T))
    return s, th, out


def _l1_rel(a, r, E):
    """Per component mean |a - r| over the mean |r| (absolute where r is identically zero)."""
    a, r = np.asarray(a).reshape(-1, E), np.asarray(r).reshape(-1, E)
    num, den = np.abs(a - r).mean(axis=0), np.abs(r).mean(axis=0)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)


@pytest.mark.parametrize("order,prec", [(7, FP64), (7, MIXED), (5, FP64), (5, MIXED)],
                         ids=["w7-fp64", "w7-mixed", "w5-fp64", "w5-mixed"])
def test_mixture_members_equal_single_grid_runs(cuda_lib, order, prec):
    """Mixture members (the temperature Newton iteration, the per-cell sound-speed terms, the
    mixture Roe state) advanced in one ensemble equal the same blocks advanced alone: FP64 to
    1e-12. The mixed members run the same device code as the single-grid mixed kernels but in
    other kernels, whose FP32 contraction may differ; on these small noisy mixing layers (1 %
    velocity noise on 8 to 24 cells) a rounding difference of the FP32 reconstruction grows over
    the steps like the mixed form's own difference from FP64. So a mixed member is checked against
    the FP64 single-grid run: per component its L1 difference stays within 3x the single-grid mixed
    run's own difference (the kernels of this build give bitwise-equal members)."""
    s, th, ms = _mixture_members(order)
    s.precision = prec
    E = s.Emax
    nsteps = 4
    pool = sum(Ensemble.member_bytes(b, prec, scheme=s) for b, _, _ in ms) + 4096 * len(ms)
    e = Ensemble(s, capacity=len(ms), pool_bytes=pool, thermal=th)

    def alone_run(precision):
        s.precision = precision
        f = Fluid(b, s, th)
        f.InitialU(U, T)
        f.initialize()
        out = f.advance(nsteps), f.get("U").reshape(-1).copy()
        f.close()
        s.precision = prec
        return out

    try:
        slots = [e.add(b, U, 1e300, T=T) for b, U, T in ms]
        assert None not in slots
        st, _ = e.advance(nsteps)
        assert st == 0
        for (b, U, T), slot in zip(ms, slots):
            (st1, t_ref, n_ref), ref = alone_run(prec)
            info = e.status(slot)
            assert st1 == 0 and info["error"] == 0 and info["steps"] == n_ref
            assert info["t"] == pytest.approx(t_ref, rel=1e-13 if prec == FP64 else MIXED_T_TOL, abs=0)
            got = e.get_state(slot)
            err = normwise(got, ref, E).max()
            print(f"member {slot} {b.X_inner}x{b.Y_inner}x{b.Z_inner}: normwise vs alone {err:.3e}")
            if prec == FP64:
                assert err <= PARITY_TOL, (slot, err)
                continue
            (_, t64, _), r64 = alone_run(FP64)
            own, ens = _l1_rel(ref, r64, E), _l1_rel(got, r64, E)
            print(f"   L1 vs FP64 per component: alone {np.array2string(own, precision=2)}, "
                  f"member {np.array2string(ens, precision=2)}")
            assert np.all(ens <= 3.0 * own + 1e-9), (slot, own, ens)
    finally:
        e.close()


@pytest.mark.parametrize("prec", [FP64, MIXED], ids=["fp64", "mixed"])
def test_viscous_mixture_members_equal_single_grid_runs(cuda_lib, prec):
    """Viscous stress and heat conduction in the ensemble (Visc | Visc_Heat | Visc_Diffu, the
    reference's fitted transport data): 3D mixing layers and a 2D walled block advanced together
    equal the same blocks advanced alone with xfg_set_transport (FP64 to 1e-12; mixed members are
    checked against the FP64 single-grid runs as in the inviscid mixture test)."""
    import os
    import helpers as H
    z = np.load(os.path.join(H.GOLDEN, "visc_mixing5_12x8x6_janaf_w5.npz"))
    tr = H.transport_of(z)
    s, th, ms = _mixture_members(5)
    s.viscous = 7
    s.precision = prec
    E = s.Emax
    nsteps = 3
    pool = sum(Ensemble.member_bytes(b, prec, scheme=s) for b, _, _ in ms) + 4096 * len(ms)
    e = Ensemble(s, capacity=len(ms), pool_bytes=pool, thermal=th)

    def alone_run(precision):
        s.precision = precision
        f = Fluid(b, s, th)
        f.set_transport(tr)
        f.InitialU(U, T)
        f.initialize()
        out = f.advance(nsteps), f.get("U").reshape(-1).copy()
        f.close()
        s.precision = prec
        return out

    try:
        slots = [e.add(b, U, 1e300, T=T) for b, U, T in ms]
        assert None not in slots
        from xfluids_gb300.abi import XfgError
        with pytest.raises(XfgError):
            e.advance(1)                  # no transport data yet
        e.set_transport(tr)
        st, _ = e.advance(nsteps)
        assert st == 0
        for (b, U, T), slot in zip(ms, slots):
            (st1, t_ref, n_ref), ref = alone_run(prec)
            info = e.status(slot)
            assert st1 == 0 and info["error"] == 0 and info["steps"] == n_ref
            assert info["t"] == pytest.approx(t_ref, rel=1e-13 if prec == FP64 else MIXED_T_TOL, abs=0)
            got = e.get_state(slot)
            err = normwise(got, ref, E).max()
            print(f"viscous member {slot} {b.X_inner}x{b.Y_inner}x{b.Z_inner}: normwise vs alone {err:.3e}")
            if prec == FP64:
                assert err <= PARITY_TOL, (slot, err)
                continue
            (_, t64, _), r64 = alone_run(FP64)
            own, ens = _l1_rel(ref, r64, E), _l1_rel(got, r64, E)
            assert np.all(ens <= 3.0 * own + 1e-9), (slot, own, ens)
    finally:
        e.close()
