"""Adaptive merging on the device path vs the oracle, bit for bit.

With merging on, every step also runs the single sweep inside collections,
the motion-metric histories, and the merge / unmerge bookkeeping.  In
reference order all of it is deterministic (insertion-ordered pair sets), so
after every step the device path must reproduce the oracle exactly: the
top-level body list with each collection's members in order, the full-solve
contact list with its multipliers, every body's state, and the merge and
unmerge event counts.
"""
import numpy as np
import pytest

from adaptivemerging_gb300 import scenes
from helpers import compare_bodies, compare_contacts, params
from oracle_binding import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "tower12": (lambda: scenes.tower(12, seed=4, density=1.0), 0.01, 160, dict(friction=0.6, iterations=60)),
    "pile": (lambda: scenes.random_pile(20, seed=9, kinds=("box", "sphere")), 0.01, 220,
             dict(friction=0.7, iterations=60)),
    "wall_small": (lambda: scenes.wall(cols=8, rows=6, seed=13), 0.005, 160, dict(friction=0.5, iterations=80)),
}


def test_merging_bit_exact_clumps_in_funnel(gpu_lib):
    """Sphere-tree clumps poured through a funnel of pinned panels onto a
    platform (the large-scene workload's geometry, 120 clumps): tree-tree and
    tree-box collisions with merging on stay bit-exact through the first
    merges and unmerges (checked every 5 steps over 1400 steps)."""
    from adaptivemerging_gb300 import native
    sc = scenes.funnel_clumps(120, seed=5)
    P = params(enable_merging=1, friction=0.7, iterations=60)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    for s in range(1400):
        g.step(0.002)
        o.step(0.002)
        if s % 5 == 4 or s == 1399:
            tg, to = g.topology(), o.topology()
            assert tg == to, f"step {s}: topology differs"
            msg = compare_contacts(g.contacts(), o.contacts())
            assert msg is None, f"step {s}: {msg}"
            msg = compare_bodies(g.bodies(), o.bodies())
            assert msg is None, f"step {s}: {msg}"
    c = o.counters()
    pg = g.perf()
    assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"])
    assert c["merges"] > 0 and c["unmerges"] > 0, c


def test_kinematic_platform_bit_exact(gpu_lib):
    """The large-scene workload's shaking platform (am_set_kinematic: the
    pinned platform oscillates vertically, 2 Hz, 0.05 m; sleeping off so no
    clump rests asleep on it): 120 clumps poured onto it, merging on, stay
    bit-exact with the oracle's restatement (checked every 10 steps over 1400
    steps), and the platform's contacts carry its prescribed velocity into the
    solve."""
    from adaptivemerging_gb300 import native
    sc = scenes.funnel_clumps(120, seed=5)
    P = params(enable_merging=1, enable_sleeping=0, friction=0.7, iterations=60)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    pb = scenes.FUNNEL_PLATFORM
    dt = 0.002
    g.set_kinematic(pb, (0, 1, 0), 0.05, 2.0, dt)
    o.set_kinematic(pb, (0, 1, 0), 0.05, 2.0, dt)
    on_platform = 0
    for s in range(1400):
        g.step(dt)
        o.step(dt)
        if s % 10 == 9 or s == 1399:
            tg, to = g.topology(), o.topology()
            assert tg == to, f"step {s}: topology differs"
            cg = g.contacts()
            msg = compare_contacts(cg, o.contacts())
            assert msg is None, f"step {s}: {msg}"
            msg = compare_bodies(g.bodies(), o.bodies())
            assert msg is None, f"step {s}: {msg}"
            on_platform = max(on_platform, int(np.sum((cg["body1"] == pb) | (cg["body2"] == pb))))
    c = o.counters()
    pg = g.perf()
    assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"])
    assert on_platform > 0, "no clump reached the platform"
    vy = g.bodies()["v"][pb][1]
    assert vy != 0.0


def test_kinematic_body_rules(gpu_lib):
    """am_set_kinematic refuses a moving support while sleeping is on (and
    am_set_params refuses turning sleeping on under one): the reference's
    sleeping treats pinned bodies as static.  A new scene loaded into the
    context clears every kinematic body, so it steps as a fresh context."""
    import ctypes as C
    from adaptivemerging_gb300 import native
    pb = scenes.FUNNEL_PLATFORM
    sc = scenes.funnel_clumps(6, seed=5)
    P_sleep = params(enable_merging=1, enable_sleeping=1, friction=0.7, iterations=40)
    P = params(enable_merging=1, enable_sleeping=0, friction=0.7, iterations=40)
    g = native.System(sc, P_sleep)
    with pytest.raises(native.AmError) as e:
        g.set_kinematic(pb, (0, 1, 0), 0.05, 0.5, 0.002)
    assert e.value.code == -6
    g.close()
    g = native.System(sc, P)
    g.set_kinematic(pb, (0, 1, 0), 0.05, 0.5, 0.002)
    with pytest.raises(native.AmError) as e:
        g.set_params(P_sleep)
    assert e.value.code == -6
    g.set_params(P)
    g.step(0.002, 5)
    second = scenes.tower(6, seed=1)
    s2 = second.struct()
    g._check(native.lib().am_set_scene(g.h, C.byref(s2)))
    g._s, g.n, g.scene = s2, second.n, second
    g.set_params(P_sleep)   # no kinematic body is left
    fresh = native.System(second, P_sleep)
    for _ in range(20):
        g.step(0.01)
        fresh.step(0.01)
    assert np.array_equal(g.bodies()["x"], fresh.bodies()["x"])
    g.close()
    fresh.close()


@pytest.mark.parametrize("name", list(CASES))
def test_merging_bit_exact(gpu_lib, name):
    from adaptivemerging_gb300 import native
    make, dt, steps, over = CASES[name]
    sc = make()
    P = params(enable_merging=1, **over)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    merged = 0
    for s in range(steps):
        g.step(dt)
        o.step(dt)
        tg, to = g.topology(), o.topology()
        assert tg == to, f"step {s}: topology differs\n{tg}\n{to}"
        cg, co = g.contacts(), o.contacts()
        assert len(cg["body1"]) == len(co["body1"]), f"step {s}: contacts {len(cg['body1'])} vs {len(co['body1'])}"
        msg = compare_contacts(cg, co)
        assert msg is None, f"step {s}: {msg}"
        msg = compare_bodies(g.bodies(), o.bodies())
        assert msg is None, f"step {s}: {msg}"
        c = o.counters()
        pg = g.perf()
        assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"]), f"step {s}"
        merged = max(merged, sum(1 for t in to if isinstance(t, tuple)))
    assert merged > 0, "scenario never formed a collection"


def test_device_matches_committed_golden(gpu_lib):
    """The device path reproduces the committed oracle fixture of the tower
    workload (merging on) step for step."""
    import json
    import os
    from adaptivemerging_gb300 import abi, native
    from test_oracle_cpu import _digest
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tower_c1.json")) as f:
        gold = json.load(f)
    g = native.System(scenes.tower(**gold["scene"]), abi.default_params(**gold["params"]))
    for s, want in enumerate(gold["steps"]):
        g.step(gold["dt"])
        assert _digest(g) == want, f"step {s}"


# AM_ORDER_COLOURED; AM_ORDER_MIXED with its kernel form chosen per step, and on a grid
@pytest.mark.parametrize("order,form", [(1, -1), (2, -1), (2, 0)], ids=["fp64", "mixed", "mixed-grid"])
@pytest.mark.parametrize("name,warm,cap", [("wall_small", 94, 60000), ("tower12", 54, 500000)])
def test_coloured_converged_with_collections(gpu_lib, name, warm, cap, order, form):
    """The coloured FP64 full solve (AM_ORDER_COLOURED) with merged
    collections as solve bodies: from an identical merged state (reference
    order first, bit-exact), one step solved to a fixed point on both sides
    gives the oracle's multipliers within 1e-6 relative.  The step is not a
    merge step (merge events every 10 steps), so both sides keep the same
    topology through it; its full-solve contacts include contacts of
    collections with other bodies.  The light tower converges slowly: the
    oracle needs about 244 000 sweeps to a change below 1e-13 at this step."""
    from adaptivemerging_gb300 import abi, native
    make, dt, _, over = CASES[name]
    sc = make()
    g = native.System(sc, params(enable_merging=1, **over))
    o = Oracle(sc, params(enable_merging=1, **over))
    g.step(dt, warm)
    o.step(dt, warm)
    assert g.topology() == o.topology()
    conv = dict(over, iterations=cap, tolerance=1e-13)
    g.set_params(params(enable_merging=1, solver_order=order, **conv))
    g.set_mixed_form(form)
    o.set_params(params(enable_merging=1, **conv))
    g.step(dt)
    o.step(dt)
    to = o.topology()
    assert g.topology() == to
    parent = o.bodies()["parent"]
    co = o.contacts()
    lg, lo = g.contacts()["lambda"], co["lambda"]
    assert lg.shape == lo.shape and lo.size > 0
    touching = int(np.sum((parent[co["body1"]] >= 0) | (parent[co["body2"]] >= 0)))
    assert touching > 0 and any(isinstance(t, tuple) for t in to), "no collection in the solve"
    err = float(np.abs(lg - lo).max()) / max(1.0, float(np.abs(lo).max()))
    st = g.stats()
    print(f"{name}: contacts {lo.shape[0]} ({touching} on collections) rel err {err:.2e} sweeps {st.sweeps} "
          f"residual_rel {st.residual_rel:.2e}")
    assert o.counters()["sweeps"] < cap and st.sweeps < cap, "not converged"
    assert err <= 1e-6, err
    assert st.residual_rel <= 1e-6


@pytest.mark.parametrize("name", ["tower12", "wall_small"])
def test_merge_tests_match_oracle(gpu_lib, name):
    """am_merge_tests, the read-only merge / unmerge predicates a host that
    keeps its own merging logic reads, equal the oracle's after every step:
    the same pairs in the reference's iteration order, the same outcomes and
    bit-identical motion metrics; merge tests turn positive in both scenes,
    unmerge tests in the wall."""
    from adaptivemerging_gb300 import native
    make, dt, steps, over = CASES[name]
    sc = make()
    P = params(enable_merging=1, **over)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    seen = {0: 0, 1: 0}
    for s in range(steps):
        g.step(dt)
        o.step(dt)
        tg, to = g.merge_tests(), o.merge_tests()
        for k in ("body1", "body2", "kind", "result", "metric"):
            assert np.array_equal(tg[k], to[k]), f"step {s}: {k}"
        for kind in (0, 1):
            seen[kind] += int(((tg["kind"] == kind) & (tg["result"] == 1)).sum())
    print(f"{name}: positive merge tests {seen[0]}, unmerge tests {seen[1]}")
    assert seen[0] > 0 and (seen[1] > 0 or name != "wall_small")


@pytest.mark.parametrize("name", ["tower12", "wall_small"])
def test_phase_driven_merging_step_matches_oracle(gpu_lib, name):
    """A host loop drives the merging step phase by phase through the C ABI
    (am_step_phase), reads the merge / unmerge predicates (am_merge_tests)
    and the single sweep's contact order (am_single_sweep_order) and runs the
    single sweep itself with that order (am_single_sweep): topology, contacts,
    bodies and event counts stay bit-exact to the oracle every step.  The
    order is honoured: the same step with the order reversed leaves other
    multipliers on the contacts inside collections."""
    from adaptivemerging_gb300 import abi, native
    make, dt, steps, over = CASES[name]
    sc = make()
    P = params(enable_merging=1, **over)
    g = native.System(sc, P)
    h = native.System(sc, P)            # the same steps, until it takes one reversed order
    o = Oracle(sc, P)
    swept = 0
    reversed_checked = False
    for s in range(steps):
        for q in ((g, h) if h is not None else (g,)):
            q.step_phase(abi.MPHASES.index("collide"), dt)
            q.step_phase(abi.MPHASES.index("warm_start"), dt)
        refs = g.single_sweep_order()
        swept += len(refs)
        g.single_sweep(refs, dt)
        if h is not None:
            rev = len(refs) > 4 and not reversed_checked
            h.single_sweep(refs[::-1] if rev else h.single_sweep_order(), dt)
        for q in ((g, h) if h is not None else (g,)):
            for ph in ("unmerge", "solve", "advance", "merge", "finish"):
                q.step_phase(abi.MPHASES.index(ph), dt)
        o.step(dt)
        if h is not None and rev:
            # the single sweep's multipliers (on contacts inside collections) differ
            assert h.get_state() != g.get_state(), "reversed order gave the same state"
            reversed_checked = True
            h = None
        assert g.topology() == o.topology(), f"step {s}: topology"
        cg, co = g.contacts(), o.contacts()
        assert len(cg["body1"]) == len(co["body1"]), f"step {s}"
        msg = compare_contacts(cg, co)
        assert msg is None, f"step {s}: {msg}"
        msg = compare_bodies(g.bodies(), o.bodies())
        assert msg is None, f"step {s}: {msg}"
        c, pg = o.counters(), g.perf()
        assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"]), f"step {s}"
        tg, to = g.merge_tests(), o.merge_tests()
        assert all(np.array_equal(tg[k], to[k]) for k in tg), f"step {s}: merge tests"
    assert swept > 0 and reversed_checked and o.counters()["merges"] > 0


def test_large_pour_with_merging_is_deterministic(gpu_lib):
    """3000 clumps poured through the funnel with merging on (list order, as
    the drop-in runs it): two runs from the same scene hold the same state,
    byte for byte, after 620 steps.  By then collections of hundreds of clumps
    meet every body in their reach, the case where the member pairs of a
    collection's candidates once exceeded the pair scan's 2^20 entries."""
    from adaptivemerging_gb300 import native
    sc = scenes.funnel_clumps(3000, seed=5)
    P = params(enable_merging=1, enable_sleeping=0, friction=0.7, iterations=100)

    def run():
        g = native.System(sc, P)
        g.set_kinematic(scenes.FUNNEL_PLATFORM, (0, 1, 0), 0.05, 0.5, 0.002)
        g.step(0.002, 620)
        blob = g.get_state()
        merges = g.perf().merge_events
        g.close()
        return blob, merges

    a, ma = run()
    b, mb = run()
    assert ma > 0
    assert a == b
