"""Composite bodies in the oracle (the reference's RigidBodyGeomComposite:
XMLParser.createComposite, CollisionProcessor.narrowPhase :711-722,
Contact.set :167-181, the composite branch of warmStart :488-503).  The
library does not step composites yet and refuses their body type
(AM_COMPOSITE); these CPU tests hold the oracle's restatement that a device
path will be checked against.

- createComposite's mass properties on a known answer (two boxes: mass,
  centre, parallel-axis inertia, box, sub-body poses).
- A composite of one box at its own origin places that box exactly at the
  composite's pose, so a scene with it steps bit-for-bit like the same scene
  with a plain box, merging on: contacts (bodies, info, multipliers), bodies
  and merge events.
- A two-part composite dropped on a plane comes to rest on both parts, and
  every contact names the composite, never a sub-body."""
import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scene_xml, scenes
from helpers import params
from oracle_binding import Oracle

TWO_BOXES = """<root>
  <body type="composite" name="pair">
    <x>0 3 0</x>
    <body type="box" name="a" dim="1 1 1" density="2"><x>-1 0 0</x></body>
    <body type="box" name="b" dim="1 1 1" density="2"><x>1 0 0</x></body>
  </body>
  <body type="plane" name="floor" p="0 0 0" n="0 1 0"/>
</root>"""


def test_composite_mass_properties():
    sc, _, names = scene_xml.load(TWO_BOXES, composites=True)
    a = sc.a
    assert names == ["pair", "floor"] and a["type"][0] == scenes.COMPOSITE
    # two boxes of 2 kg at x = -1 and 1: mass 4, centre at the element's x
    assert a["mass"][0] == 4.0 and list(a["x"][:3]) == [0.0, 3.0, 0.0]
    # each box I = 2/12 (1 + 1) = 1/3 about every axis, plus m d^2 = 2 about y and z
    I = np.asarray(a["inertia"][:9]).reshape(3, 3)
    assert np.allclose(I, np.diag([2 / 3, 2 / 3 + 4, 2 / 3 + 4]), rtol=0, atol=1e-15)
    assert list(a["bbox"][:6]) == [-1.5, -0.5, -0.5, 1.5, 0.5, 0.5]
    assert list(a["sub_parent"]) == [0, 0] and list(a["sub_type"]) == [abi.AM_BOX, abi.AM_BOX]
    assert list(a["sub_t"]) == [-1.0, 0.0, 0.0, 1.0, 0.0, 0.0] and sc.struct().n_subs == 2


def test_composites_need_the_option():
    with pytest.raises(scene_xml.NotSupported):
        scene_xml.load(TWO_BOXES)


def _stack(one_box_composite):
    b = scenes.Builder()
    if one_box_composite:
        m = 1.0 * 1.0 * 1.0 * 500.0
        i = 1.0 / 12 * m * (1.0 + 1.0)
        b.composite((0.0, 0.5, 0.0), m, np.diag([i, i, i]), [-0.5, -0.5, -0.5, 0.5, 0.5, 0.5],
                    [(abi.AM_BOX, [1.0, 1.0, 1.0, 0.0], scenes.IDENT, [0.0, 0.0, 0.0])])
    else:
        b.box((1.0, 1.0, 1.0), (0.0, 0.5, 0.0), density=500.0)
    b.box((0.8, 0.4, 0.8), (0.05, 1.2, 0.0), R=scenes.yaw(0.3), density=500.0)
    b.sphere(0.2, (-0.1, 1.8, 0.1), density=500.0)
    b.plane((0, 0, 0), (0, 1, 0))
    return b.build()


def test_one_box_composite_steps_as_the_box():
    P = params(enable_merging=1, gravity_amount=9.81)
    oc, ob = Oracle(_stack(True), P), Oracle(_stack(False), P)
    for s in range(300):
        oc.step(0.01)
        ob.step(0.01)
        cc, cb = oc.contacts(), ob.contacts()
        for k in ("body1", "body2", "info", "lambda"):
            assert np.array_equal(cc[k], cb[k]), (s, k)
        bc, bb = oc.bodies(), ob.bodies()
        for k in ("x", "R", "v", "omega"):
            assert np.array_equal(bc[k], bb[k]), (s, k)
    assert oc.counters()["merges"] == ob.counters()["merges"] > 0
    assert oc.topology() == ob.topology()


def test_two_part_composite_rests_on_both_parts():
    sc, P, _ = scene_xml.load(TWO_BOXES, params=params(gravity_amount=9.81, enable_merging=0), composites=True)
    o = Oracle(sc, P)
    for _ in range(400):
        o.step(0.01)
        c = o.contacts()
        assert set(np.concatenate([c["body1"], c["body2"]]).tolist()) <= {0, 1}
    b = o.bodies()
    assert abs(b["x"][0][1] - 0.5) < 1e-2 and abs(b["v"][0]).max() < 1e-3
    c = o.contacts()
    xs = [float(p) for p in c["frame"].reshape(-1, 12)[:, 0]] if len(c["body1"]) else []
    assert len(c["body1"]) == 8 and min(xs) < -1.0 and max(xs) > 1.0   # four corners under each box


def test_sphere_sub_body_against_a_box():
    """A box resting on a composite's sphere sub-body: the contact's
    composite side is a non-box sub-body, the warm-start branch where the
    reference takes the plain warm start and then also runs the box-box
    search (CollisionProcessor.java:494-503).  The pile comes to rest,
    persisting contacts are warm started (not fresh), and two runs agree bit
    for bit."""
    def scene():
        b = scenes.Builder()
        m_box, m_sph = 8.0 * 100.0, 4.0 / 3 * np.pi * 0.5 ** 3 * 100.0
        # composite: a 2 x 0.5 x 2 slab with a sphere of radius 0.5 on top of it
        com_y = (m_box * 0.0 + m_sph * 0.75) / (m_box + m_sph)
        I_box = np.diag([m_box / 12 * (0.25 + 4), m_box / 12 * 8, m_box / 12 * (4 + 0.25)])
        I_sph = np.eye(3) * 0.4 * m_sph * 0.25
        d = np.array([0.0, com_y, 0.0])
        par = lambda m, r: m * (np.dot(r, r) * np.eye(3) - np.outer(r, r))
        I = I_box + par(m_box, d) + I_sph + par(m_sph, np.array([0.0, 0.75, 0.0]) - d)
        b.composite((0.0, 0.25 + com_y, 0.0), m_box + m_sph, I, [-1.0, -0.25 - com_y, -1.0, 1.0, 1.25 - com_y, 1.0],
                    [(abi.AM_BOX, [2.0, 0.5, 2.0, 0.0], scenes.IDENT, [0.0, -com_y, 0.0]),
                     (abi.AM_SPHERE, [0.5, 0.0, 0.0, 0.0], scenes.IDENT, [0.0, 0.75 - com_y, 0.0])])
        b.box((0.6, 0.3, 0.6), (0.0, 1.5 + 0.15 + 0.005, 0.0), density=100.0)
        b.plane((0, 0, 0), (0, 1, 0))
        return b.build()
    P = params(gravity_amount=9.81, enable_merging=0, iterations=60)
    runs = []
    for _ in range(2):
        o = Oracle(scene(), P)
        warm = 0
        for s in range(200):
            o.step(0.01)
            c = o.contacts()
            on_sphere = (c["body1"] == 1) & (c["body2"] == 0) | (c["body1"] == 0) & (c["body2"] == 1)
            warm += int(np.sum(on_sphere & (c["fresh"] == 0)))
        runs.append((o.bodies(), warm))
    (b1, w1), (b2, w2) = runs
    assert w1 == w2 and w1 > 0
    for k in ("x", "v"):
        assert np.array_equal(b1[k], b2[k])
    # the box rests on the sphere (sunk a little under the default contact compliance)
    assert abs(b1["v"][1]).max() < 1e-2 and abs(b1["x"][1][1] - 1.65) < 0.05
