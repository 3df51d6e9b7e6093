"""The oracle's prescribed oscillation of a pinned body (the restatement of
am_set_kinematic that the device is checked against): the platform of the
funnel scene follows x0 + axis * a * sin(w n dt), v = axis * a * w * cos(w n dt)
at the start of step n, clumps that rest on it are carried along, and a body
that is not pinned is refused."""
import math

import numpy as np
import pytest

from adaptivemerging_gb300 import scenes
from helpers import params
from oracle_binding import Oracle


def test_platform_follows_the_prescribed_oscillation():
    sc = scenes.funnel_clumps(6, seed=5)
    o = Oracle(sc, params(enable_merging=1, enable_sleeping=0, friction=0.7, iterations=40))
    pb = scenes.FUNNEL_PLATFORM
    x0 = o.bodies()["x"][pb].copy()
    dt, a, f = 0.002, 0.05, 2.0
    w = 2 * math.pi * f
    o.set_kinematic(pb, (0, 1, 0), a, f, dt)
    for n in range(120):
        o.step(dt)
        b = o.bodies()
        assert abs(b["x"][pb][1] - (x0[1] + a * math.sin(w * n * dt))) <= 1e-12
        assert abs(b["v"][pb][1] - a * w * math.cos(w * n * dt)) <= 1e-12
        assert b["x"][pb][0] == x0[0] and b["x"][pb][2] == x0[2]


def test_non_pinned_body_refused():
    sc = scenes.funnel_clumps(6, seed=5)
    o = Oracle(sc, params())
    with pytest.raises(AssertionError):
        o.set_kinematic(sc.n - 1, (0, 1, 0), 0.05, 0.5, 0.002)


def _in_collection(o, body):
    return any(isinstance(i, tuple) and body in i for i in o.topology())


def test_kinematic_body_never_merges():
    """A collection that holds a pinned body stays put, so a platform merged
    with the clumps on it would stop carrying them while it moved through
    them.  Without the rule this pour merges the platform at step 760, at the
    bottom of its stroke; with it the platform stays out of every collection
    and keeps its prescribed motion while the clumps merge among themselves."""
    sc = scenes.funnel_clumps(120, seed=5)
    o = Oracle(sc, params(friction=0.7, enable_merging=1, enable_sleeping=0))
    pb = scenes.FUNNEL_PLATFORM
    x0 = o.bodies()["x"][pb].copy()
    dt, a, f = 0.002, 0.05, 0.5
    w = 2 * math.pi * f
    o.set_kinematic(pb, (0, 1, 0), a, f, dt)
    for n in range(900):
        o.step(dt)
        assert not _in_collection(o, pb), n + 1
        b = o.bodies()
        assert abs(b["v"][pb][1] - a * w * math.cos(w * n * dt)) <= 1e-12
        assert abs(b["x"][pb][1] - (x0[1] + a * math.sin(w * n * dt))) <= 1e-12
    assert o.counters()["merges"] > 0
    tests = o.merge_tests()
    kin_pairs = (tests["body1"] == pb) | (tests["body2"] == pb)
    assert kin_pairs.any() and not tests["result"][kin_pairs & (tests["kind"] == 0)].any()


def test_body_inside_a_collection_cannot_become_kinematic():
    sc = scenes.funnel_clumps(120, seed=5)
    o = Oracle(sc, params(friction=0.7, enable_merging=1, enable_sleeping=0))
    pb = scenes.FUNNEL_PLATFORM
    for _ in range(3000):
        o.step(0.002)
        if _in_collection(o, pb):
            break
    assert _in_collection(o, pb)
    with pytest.raises(AssertionError):
        o.set_kinematic(pb, (0, 1, 0), 0.05, 0.5, 0.002)


def test_kinematic_body_refused_while_sleeping():
    """The reference's sleeping treats pinned bodies as static (pinned-asleep
    pairs are skipped, and contacts with pinned bodies neither keep a body
    awake nor wake it), so a moving support needs sleeping off."""
    sc = scenes.funnel_clumps(6, seed=5)
    o = Oracle(sc, params(enable_sleeping=1))
    with pytest.raises(AssertionError):
        o.set_kinematic(scenes.FUNNEL_PLATFORM, (0, 1, 0), 0.05, 0.5, 0.002)
    o.set_kinematic(scenes.FUNNEL_PLATFORM, (0, 1, 0), 0.0, 0.5, 0.002)   # removing is always allowed
