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
