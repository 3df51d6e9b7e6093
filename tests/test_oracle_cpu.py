"""CPU checks of the oracle (the restatement of the reference path).

The reference ships no tests for its 3D engine, so the oracle is pinned by
(1) analytic known answers for each collider, (2) invariants (rigid-motion
invariance, body-order symmetry, free flight, determinism, PGS fixed point),
and (3) committed golden fixtures of the tower workload that guard the oracle
itself against regressions (tests/golden/make_golden.py regenerates them).
"""
import json
import math
import os

import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scenes
from adaptivemerging_gb300.scenes import Builder, axis_angle
from helpers import params
from oracle_binding import Oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def collide(sc, **over):
    o = Oracle(sc, params(**over))
    o.begin_step()
    o.collide()
    return o.contacts()


def world_points(sc, c, k):
    """contact point k in world coordinates from body-1 frame storage"""
    b = c["body1"][k]
    R = sc["R"][9 * b:9 * b + 9].reshape(3, 3) if sc["type"][b] != abi.AM_PLANE else np.eye(3)
    x = sc["x"][3 * b:3 * b + 3] if sc["type"][b] != abi.AM_PLANE else np.zeros(3)
    return R @ c["frame"][k, 0:3] + x, R @ c["frame"][k, 3:6]


def test_box_on_plane_known_answer():
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0))
    B.box((1, 1, 1), (0, 0.45, 0))
    sc = B.build()
    c = collide(sc)
    assert list(c["info"]) == [2, 3, 6, 7]          # corners with -y, BoxPlane.java:37-44 order
    assert list(c["body1"]) == [0] * 4 and list(c["body2"]) == [1] * 4   # plane is body 1
    assert np.allclose(c["violation"][:, 0], -0.05, atol=1e-15)
    for k in range(4):
        p, n = world_points(sc, c, k)
        assert np.allclose(n, [0, 1, 0]) and abs(p[1] + 0.05) < 1e-15


def test_box_box_face_known_answer():
    B = Builder()
    B.plane((0, -10, 0), (0, 1, 0))
    B.box((1, 1, 1), (0, 0, 0))
    B.box((1, 1, 1), (0.2, 0.95, 0.1))
    c = collide(scenes_only := B.build())
    sel = (c["body1"] == 1) & (c["body2"] == 2)
    assert sel.sum() == 4
    assert np.allclose(c["violation"][sel, 0], -0.05, atol=1e-12)
    ks = np.nonzero(sel)[0]
    assert list(c["info"][ks]) == [0, 1, 2, 3]
    for k in ks:
        p, n = world_points(scenes_only, c, k)
        assert np.allclose(np.abs(n), [0, 1, 0])


def test_sphere_sphere_and_plane_known_answer():
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0))
    B.sphere(0.5, (0, 0.4, 0))
    B.sphere(0.5, (0.9, 0.6, 0))
    sc = B.build()
    c = collide(sc)
    # plane-sphere pairs come first (row 0 of the pair loop), then sphere-sphere
    ps = [k for k in range(len(c["body1"])) if c["body2"][k] == 0]
    assert len(ps) == 1
    k = ps[0]
    assert c["body1"][k] == 1 and abs(c["violation"][k, 0] + 0.1) < 1e-12
    p, n = world_points(sc, c, k)
    assert np.allclose(n, [0, -1, 0]) and np.allclose(p, [0, 0, 0], atol=1e-15)
    ss = [k for k in range(len(c["body1"])) if c["body1"][k] == 1 and c["body2"][k] == 2]
    d = math.hypot(0.9, 0.2)
    assert len(ss) == 1 and abs(c["violation"][ss[0], 0] - (d - 1.0)) < 1e-12


def test_box_sphere_known_answer():
    B = Builder()
    B.plane((0, -10, 0), (0, 1, 0))
    B.box((1, 1, 1), (0, 0, 0))
    B.sphere(0.3, (0.1, 0.7, -0.05))
    sc = B.build()
    c = collide(sc)
    k = [i for i in range(len(c["body1"])) if c["body1"][i] == 1 and c["body2"][i] == 2]
    assert len(k) == 1
    k = k[0]
    assert abs(c["violation"][k, 0] + 0.1) < 1e-12
    p, n = world_points(sc, c, k)
    assert np.allclose(n, [0, 1, 0]) and np.allclose(p, [0.1, 0.5, -0.05])


def _two_boxes(R, t):
    B = Builder()
    B.plane((0, -50, 0), (0, 1, 0))
    R = np.asarray(R).reshape(3, 3)
    q1 = R @ np.array([0, 0, 0.0]) + t
    q2 = R @ np.array([0.3, 0.9, -0.2]) + t
    r2 = R @ np.asarray(axis_angle((0.2, 1, 0.3), 0.4)).reshape(3, 3)
    B.box((1, 1, 1), tuple(q1), R=list(R.reshape(-1)))
    B.box((1.2, 0.8, 1.0), tuple(q2), R=list(r2.reshape(-1)))
    return B.build()


def test_box_box_rigid_motion_invariance():
    base = collide(_two_boxes(np.eye(3), np.zeros(3)))
    R = np.asarray(axis_angle((1, 2, 3), 0.77)).reshape(3, 3)
    moved = collide(_two_boxes(R, np.array([3.0, -2.0, 5.0])))
    sel_b = (base["body1"] == 1) & (base["body2"] == 2)
    sel_m = (moved["body1"] == 1) & (moved["body2"] == 2)
    assert sel_b.sum() == sel_m.sum() > 0
    assert np.allclose(np.sort(base["violation"][sel_b, 0]), np.sort(moved["violation"][sel_m, 0]), atol=1e-12)


def test_box_box_order_symmetry():
    sc = _two_boxes(np.eye(3), np.zeros(3))
    B = Builder()
    B.plane((0, -50, 0), (0, 1, 0))
    for i in (2, 1):   # swapped body order
        s = np.asarray(sc["shape"][4 * i:4 * i + 3])
        B.box(tuple(s), tuple(sc["x"][3 * i:3 * i + 3]), R=list(sc["R"][9 * i:9 * i + 9]))
    a, b = collide(sc), collide(B.build())
    da = np.sort(a["violation"][(a["body1"] == 1), 0])
    db = np.sort(b["violation"][(b["body1"] == 1), 0])
    assert len(da) == len(db) > 0 and np.allclose(da, db, atol=1e-9)


def test_free_flight():
    B = Builder()
    B.box((1, 1, 1), (0, 10, 0), v=(1.0, 2.0, 0.5), omega=(0, 0, 0))
    o = Oracle(B.build(), params())
    o.step(0.01)
    b = o.bodies()
    assert np.allclose(b["v"][0], [1.0, 2.0 - 9.81 * 0.01, 0.5], atol=1e-15)
    assert np.allclose(b["x"][0], [0.01, 10 + 0.01 * (2.0 - 0.0981), 0.005], atol=1e-15)


def test_determinism_and_pgs_fixed_point():
    sc = scenes.tower(6, seed=1)
    P = params(iterations=5000, tolerance=1e-14)
    a, b = Oracle(sc, P), Oracle(sc, P)
    a.step(0.01, 8)
    b.step(0.01, 8)
    ca, cb = a.contacts(), b.contacts()
    assert np.array_equal(ca["lambda"], cb["lambda"])
    assert a.counters()["last_change"] < 1e-12
    assert (ca["lambda"][:, 0] >= 0).all()
    mu = 0.6
    assert (np.abs(ca["lambda"][:, 1]) <= mu * ca["lambda"][:, 0] + 1e-12).all()


def test_residual_target_stop():
    """The oracle's residual-target stop (used for the equal-residual CPU
    baseline) ends the solve on a check sweep once the relative natural-map
    residual is below the target, at the same fixed point as a long solve."""
    sc = scenes.random_pile(24, seed=5, kinds=("box", "sphere"))
    base = params(iterations=100)
    a, b = Oracle(sc, base), Oracle(sc, base)
    a.step(0.005, 60)
    b.step(0.005, 60)
    a.set_params(params(iterations=20000, tolerance=0.0))
    a.set_residual_target(1e-9, 10)
    b.set_params(params(iterations=20000, tolerance=1e-15))
    a.step(0.005)
    b.step(0.005)
    sw = a.counters()["sweeps"]
    assert 0 < sw < 20000 and sw % 10 == 0
    la, lb = a.contacts()["lambda"], b.contacts()["lambda"]
    assert la.shape == lb.shape and la.size
    assert np.abs(la - lb).max() <= 1e-6 * max(1.0, np.abs(lb).max())


def _digest(o):
    c = o.contacts()
    b = o.bodies()
    keys = np.stack([c["body1"], c["body2"], c["bv1"], c["bv2"], c["info"]], 1) if len(c["body1"]) else np.zeros((0, 5))
    return {"n": int(len(c["body1"])), "keys": int(np.int64(np.sum(keys * np.arange(1, 6)))) if len(keys) else 0,
            "lam": float(np.sum(c["lambda"])).hex(), "x": float(np.sum(b["x"])).hex(),
            "top": o.topology().__repr__()}


def test_golden_tower():
    with open(os.path.join(GOLD, "tower_c1.json")) as f:
        gold = json.load(f)
    sc = scenes.tower(**gold["scene"])
    o = Oracle(sc, abi.default_params(**gold["params"]))
    for s, want in enumerate(gold["steps"]):
        o.step(gold["dt"])
        assert _digest(o) == want, f"step {s}"
