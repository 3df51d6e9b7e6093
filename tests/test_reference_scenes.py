"""The reference's own scene files (scenes3D/tower30.xml, denseTower25.xml),
as parsed by this repository's loader and stored in
tests/golden/reference_scenes.json by make_reference_scenes.py.

- CPU: the oracle runs both scenes; its top-level body count matches the
  reference's recorded metrics for tower30 (136 in the rows of steps 2-9).
  The recorded contact counts are not reproduced: the metrics file holds
  about 534 contacts at the second step where the oracle (and the
  reference's BoxBox.java in this tree, which keeps every clipped point)
  gives 1548, six per box-box pair.  An earlier recorded run
  (scenes3D/csv/old) starts at 1543, within 1 % of the oracle.  The runs
  used scene or code states that are not in the tree (their merging differs
  from the tree's and from each other's), so the counts pin little and are
  reported beside the oracle's.
- GPU: the device path in reference order reproduces the oracle bit for bit
  on both scenes with the scenes' own parameters and merging on (every 10
  steps for 400 steps: topology, contacts, bodies, merge / unmerge counts).
- "meshes": scenes3D/allBodyTypes.xml without its spring-hung platform, four
  mesh bodies (sphere trees of 210 to 920 spheres, three levels, up to 30
  children a node) with two boxes and a sphere, falling 30 m onto a plane
  under the reference's default gravity (1 m/s^2): the oracle lands them, and
  the device matches it bit for bit through the landing (steps 700-1000).
- seesaw.xml and chariot.xml, composite bodies without springs: on the
  oracle only (CPU), deterministic, at rest, contacts naming composites.
"""
import json
import os

import numpy as np
import pytest

from adaptivemerging_gb300 import abi
from helpers import compare_bodies, compare_contacts
from oracle_binding import Oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name):
    with open(os.path.join(HERE, "golden", "reference_scenes.json")) as f:
        d = json.load(f)
    s = d["scenes"][name]
    sc = abi.SceneArrays(**s["arrays"])
    P = abi.am_params()
    for k, v in s["params"].items():
        setattr(P, k, v)
    return sc, P, d


def test_tower30_oracle_against_recorded_metrics():
    sc, P, d = _load("tower30")
    rows = d["tower30_csv_bodies_contacts"]
    assert sc.n == 136 and len(rows) >= 20
    o = Oracle(sc, P)
    ours = []
    for k in range(12):
        o.step(0.01)
        ours.append((o.counters()["top"], o.num_contacts()))
    # row r of the metrics file is written by step r + 2 (the first call writes the header)
    for r in range(8):
        assert ours[r + 1][0] == rows[r][0] == 136
    print("step, recorded contacts, oracle contacts:",
          [(r + 2, rows[r][1], ours[r + 1][1]) for r in range(8)])
    # The earlier run (scenes3D/csv/old) starts from the same 136 bodies with
    # 1543 contacts, the count of six clipped points per box-box pair that the
    # colliders in the tree produce (the oracle: 1548 at its first steps).
    old = d["tower30_old_csv_bodies_contacts"]
    assert old[0][0] == 136 and abs(old[0][1] - ours[0][1]) <= 0.01 * old[0][1]
    # From step 10, the first merge step (stepsBetweenMergeEvents = 10), the
    # oracle holds every box in one collection with the plane; neither
    # recorded run does (the later one keeps 136 bodies for 269 rows, the
    # earlier one merges from its second row), so merging pins nothing here.
    assert ours[9][0] == 1


@pytest.mark.parametrize("name", ["tower30", "denseTower25"])
def test_reference_scene_runs_on_oracle(name):
    sc, P, _ = _load(name)
    o = Oracle(sc, P)
    o.step(0.01, 150)
    c = o.counters()
    assert o.num_contacts() >= 0 and np.isfinite(o.bodies()["x"]).all()
    assert c["merges"] > 0, c


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tower30", "denseTower25"])
def test_reference_scene_device_bit_exact(gpu_lib, name):
    from adaptivemerging_gb300 import native
    sc, P, _ = _load(name)
    assert P.enable_merging == 1 and P.solver_order == abi.AM_ORDER_REFERENCE
    g = native.System(sc, P)
    o = Oracle(sc, P)
    seen = 0
    for s in range(400):
        g.step(0.01)
        o.step(0.01)
        if s % 10 == 9:
            assert g.topology() == o.topology(), f"step {s}: topology"
            cg, co = g.contacts(), o.contacts()
            seen += len(co["body1"])
            assert len(cg["body1"]) == len(co["body1"]), f"step {s}"
            msg = compare_contacts(cg, co)
            assert msg is None, f"step {s}: {msg}"
            msg = compare_bodies(g.bodies(), o.bodies())
            assert msg is None, f"step {s}: {msg}"
            c, pg = o.counters(), g.perf()
            assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"]), f"step {s}"
    c = o.counters()
    print(f"{name}: {c['merges']} merges, {c['unmerges']} unmerges, {seen} contacts checked")
    assert seen > 0 and c["merges"] > 0


def test_mesh_scene_lands_on_oracle():
    sc, P, _ = _load("meshes")
    assert sc.n == 8 and len(sc.a["node_r"]) == 2288
    o = Oracle(sc, P)
    most = 0
    for _ in range(100):
        o.step(0.01, 10)
        most = max(most, o.num_contacts())
    assert most > 0 and np.isfinite(o.bodies()["x"]).all()


@pytest.mark.gpu
def test_mesh_scene_device_bit_exact(gpu_lib):
    from adaptivemerging_gb300 import native
    sc, P, _ = _load("meshes")
    g = native.System(sc, P)
    o = Oracle(sc, P)
    seen = 0
    for s in range(1000):
        g.step(0.01)
        o.step(0.01)
        if s >= 699 and s % 10 == 9:
            assert g.topology() == o.topology(), f"step {s}: topology"
            cg, co = g.contacts(), o.contacts()
            seen += len(co["body1"])
            assert len(cg["body1"]) == len(co["body1"]), f"step {s}"
            msg = compare_contacts(cg, co)
            assert msg is None, f"step {s}: {msg}"
            msg = compare_bodies(g.bodies(), o.bodies())
            assert msg is None, f"step {s}: {msg}"
    print(f"meshes: {seen} contacts checked")
    assert seen > 0


@pytest.mark.parametrize("name,steps", [("seesaw", 1500), ("chariot", 1100)])
def test_composite_scene_on_oracle(name, steps):
    """The reference's composite scenes (seesaw.xml: a plank composite on a
    two-box pivot composite; chariot.xml: six composites among 115 boxes and
    spheres) with their own parameters: two oracle runs agree bit for bit, the
    state stays finite, every contact names a scene body (a composite, never
    a sub-body), and the composites come to rest.  The library refuses the
    composite body type, so these are oracle-only until a device path
    exists."""
    from adaptivemerging_gb300 import scenes
    sc, P, _ = _load(name)
    runs = []
    for _ in range(2):
        o = Oracle(sc, P)
        for s in range(steps):
            o.step(0.01)
            if s % 100 == 99:
                c = o.contacts()
                ids = np.concatenate([c["body1"], c["body2"]])
                assert ((ids >= 0) & (ids < sc.n)).all()
        runs.append((o.bodies(), o.counters()))
    (b1, c1), (b2, c2) = runs
    for k in ("x", "R", "v", "omega"):
        assert np.array_equal(b1[k], b2[k])
    assert c1 == c2 and np.isfinite(b1["x"]).all()
    comp = np.asarray(sc.a["type"]) == scenes.COMPOSITE
    assert comp.sum() >= 2 and float(np.abs(b1["v"][comp]).max()) < 1e-3
