"""The XML scene loader (the reference's scene format, XMLParser.java):
mass properties, axis-angle orientation, collision overrides, the refusal of
unsupported elements, and the loaded scene on the oracle (CPU) and, marked
gpu, bit-exact on the device path."""
import math

import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scene_xml
from helpers import params

DOC = """<?xml version="1.0" ?>
<root>
  <collision iterations="40" feedbackStiffness="0.3" friction="0.6" enableCompliance="true"/>
  <body type="plane" name="ground" p="0 0 0" n="0 2 0"/>
  <body type="box" name="base" dim="2 1 2" density="500" scale="1">
    <x>0 0.5 0</x>
    <R>0 1 0 0.3</R>
    <pinned>false</pinned>
  </body>
  <body type="box" name="top" dim="1 1 1" density="1000">
    <x>0.1 1.49 0</x>
    <R>0 0 1 0</R>
    <v>0 -0.1 0</v>
    <friction>0.5</friction>
  </body>
  <body type="sphere" name="ball" r="0.25" density="2000">
    <x>0.2 2.24 0.1</x>
    <omega>0 0 1</omega>
    <restitution>0.2</restitution>
    <magnetic>false</magnetic>
  </body>
  <body type="box" name="wall" dim="1 3 1">
    <x>3 1.5 0</x>
    <pinned>true</pinned>
  </body>
</root>
"""


def test_loader_mass_orientation_and_parameters():
    sc, P, names = scene_xml.load(DOC)
    assert names == ["ground", "base", "top", "ball", "wall"]
    assert list(sc["type"]) == [abi.AM_PLANE, abi.AM_BOX, abi.AM_BOX, abi.AM_SPHERE, abi.AM_BOX]
    # box: m = sx sy sz density, I = m/12 (..); sphere: 4/3 pi r^3 density, 2/5 m r^2
    assert sc["mass"][1] == 2 * 1 * 2 * 500
    assert np.allclose(sc["inertia"][9:18].reshape(3, 3), np.diag([2000 / 12 * 5, 2000 / 12 * 8, 2000 / 12 * 5]))
    m = 4.0 / 3 * math.pi * 0.25 ** 3 * 2000
    assert abs(sc["mass"][3] - m) < 1e-9 and abs(sc["inertia"][27] - 0.4 * m * 0.0625) < 1e-9
    R = sc["R"][9:18].reshape(3, 3)
    c, s = math.cos(0.3), math.sin(0.3)
    assert np.allclose(R, [[c, 0, s], [0, 1, 0], [-s, 0, c]])
    assert np.array_equal(sc["R"][18:27], np.eye(3).reshape(-1))          # zero angle
    assert list(sc["pinned"]) == [1, 0, 0, 0, 1]
    assert sc["friction"][2] == 0.5 and sc["restitution"][3] == 0.2 and sc["friction"][1] == 0.8
    assert P.iterations == 40 and P.feedback_stiffness == 0.3 and P.friction_override == 1
    assert P.friction == 0.6 and P.enable_compliance == 1 and P.restitution_override == 0


def test_loader_refuses_unsupported_elements():
    with pytest.raises(scene_xml.NotSupported):
        scene_xml.load('<root><body type="composite" name="c"/></root>')
    with pytest.raises(scene_xml.NotSupported):
        scene_xml.load('<root><body type="box" dim="1 1 1"><spring pB="0 0 0" pW="0 1 0"/></body></root>')
    with pytest.raises(scene_xml.NotSupported):
        scene_xml.load('<root><collision enablePostStabilization="true" iterations="10"/>'
                       '<body type="box" dim="1 1 1"/></root>')
    sc, P, _ = scene_xml.load('<root><collision enablePostStabilization="false" iterations="10"/>'
                              '<system mouseSpringStiffness="3"/><body type="box" dim="1 1 1"/></root>')
    assert sc.n == 1 and P.iterations == 10


def test_loaded_scene_runs_on_the_oracle():
    from oracle_binding import Oracle
    sc, P, _ = scene_xml.load(DOC)
    P.gravity_amount = 9.81
    o = Oracle(sc, P)
    o.step(0.01, 30)
    x = o.bodies()["x"]
    assert np.isfinite(x).all() and o.num_contacts() > 0
    assert x[4][1] == 1.5                                             # the pinned wall stays


@pytest.mark.gpu
def test_loaded_scene_bit_exact_on_device(gpu_lib):
    from adaptivemerging_gb300 import native
    from helpers import compare_bodies, compare_contacts
    from oracle_binding import Oracle
    sc, P, _ = scene_xml.load(DOC)
    P.gravity_amount = 9.81
    g = native.System(sc, P)
    o = Oracle(sc, P)
    for _ in range(30):
        g.step(0.01)
        o.step(0.01)
        assert compare_contacts(g.contacts(), o.contacts()) is None
        assert compare_bodies(g.bodies(), o.bodies()) is None


def _cube_files(tmp_path):
    """A 1 m cube (vertices 0..1, 12 outward triangles) and a 3-sphere tree."""
    obj = tmp_path / "cube.obj"
    v = [(x, y, z) for x in (0, 1) for y in (0, 1) for z in (0, 1)]
    idx = {p: i + 1 for i, p in enumerate(v)}
    quads = [((0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)), ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)),
             ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)), ((0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)),
             ((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)), ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1))]
    lines = [f"v {x} {y} {z}" for x, y, z in v]
    for q in quads:
        a, b, c, d = (idx[p] for p in q)
        lines += [f"f {a}/1/1 {b}/1/1 {c}/1/1", f"f {a} {c} {d}"]
    obj.write_text("\n".join(lines) + "\n")
    sph = tmp_path / "cube.sph"
    sph.write_text("3\n0.5 0.5 0.5 0.9\n0.5 0.5 0.25 0.45\n0.5 0.5 0.75 0.45\n1 2 2 3\n")
    return obj, sph


def test_mesh_body_mass_properties_and_tree(tmp_path):
    """createMesh (XMLParser.java:449-539): a cube soup scaled by 2 at
    density 3 has mass 24, its centre of mass at (1, 1, 1) and inertia
    m (2^2 + 2^2) / 12 = 16 about each axis; the sphere tree is scaled and
    moved to the centre of mass, the root first and its two children after
    it in file order."""
    obj, sph = _cube_files(tmp_path)
    doc = (f'<root><body type="mesh" name="cube" scale="2" density="3" obj="{obj.name}" st="{sph.name}">'
           f'<x>0 5 0</x></body></root>')
    sc, _, names = scene_xml.load(doc, data_root=str(tmp_path))
    a = sc.a
    assert names == ["cube"] and a["type"][0] == abi.AM_TREE
    assert abs(a["mass"][0] - 24.0) < 1e-12
    I = np.asarray(a["inertia"][:9]).reshape(3, 3)
    assert np.allclose(I, 16.0 * np.eye(3), atol=1e-12)
    r0 = a["body_root"][0]
    assert a["node_child0"][r0] == r0 + 1 and a["node_nchild"][r0] == 2
    c = np.asarray(a["node_c"]).reshape(-1, 3)
    assert np.allclose(c[r0], 0.0) and np.allclose(c[r0 + 1], (0, 0, -0.5)) and np.allclose(c[r0 + 2], (0, 0, 0.5))
    assert np.allclose(np.asarray(a["node_r"])[r0:r0 + 3], (1.8, 0.9, 0.9))
    # boundingBoxB is the box of the scaled vertices about the centre of mass,
    # not the box of the leaf spheres (which reach 0.45 + 0.9 = 1.35 above it)
    assert list(a["bbox"][:6]) == [-1.0, -1.0, -1.0, 1.0, 1.0, 1.0]


def test_mesh_box_follows_the_reference_arithmetic():
    """XMLParser.java:474-493: Math.min / Math.max from MAX_VALUE and
    Double.MIN_VALUE.  An axis on which no vertex is positive keeps
    MIN_VALUE (the smallest positive double) as its upper bound, and the
    sign of a zero follows Java's min (-0.0 below +0.0)."""
    box = scene_xml.mesh_box([(-1.0, 0.0, -2.0), (-0.5, -0.0, 3.0)])
    assert box[:3] == [-1.0, -0.0, -2.0] and math.copysign(1, box[1]) < 0
    assert box[3:] == [5e-324, 5e-324, 3.0]


def test_mesh_box_moves_the_motion_metric():
    """The merge test's relative-velocity metric samples the corners of the
    body's boundingBoxB (MotionMetricProcessor.java:39-73), so a mesh body's
    box must be its mesh's.  Two identical tumbling mesh bodies, one given
    the mesh box and one the leaf-sphere box, resting on a plane: the
    metric of each body's pair with the plane differs."""
    from oracle_binding import Oracle
    from adaptivemerging_gb300.scenes import Builder
    out = []
    for box in ([-0.5, -0.5, -0.5, 0.5, 0.5, 0.5], None):
        b = Builder()
        b.tree([(0, 0, 0), (0, 0, -0.25), (0, 0, 0.25)], [0.9, 0.45, 0.45], [[1, 2], [], []], (0, 0.45, 0),
               1000.0, 1000.0 / 6 * np.eye(3), omega=(0.0, 0.3, 0.0), bbox=box)
        b.plane((0, 0, 0), (0, 1, 0))
        o = Oracle(b.build(), params(enable_merging=1, enable_sleeping=0, gravity_amount=9.81))
        o.step(0.01, 5)
        out.append(o.merge_tests()["metric"])
    assert len(out[0]) == 1 and len(out[1]) == 1 and out[0][0] != out[1][0]


def test_mesh_body_settles_on_oracle(tmp_path):
    """The cube mesh body dropped on a plane lands on its sphere tree's leaves
    in the oracle and comes to rest on them."""
    from oracle_binding import Oracle
    obj, sph = _cube_files(tmp_path)
    doc = (f'<root><body type="mesh" name="cube" scale="1" density="1000" obj="{obj.name}" st="{sph.name}">'
           f'<x>0 1 0</x></body><body type="plane" name="floor" p="0 0 0" n="0 1 0"/></root>')
    sc, P, _ = scene_xml.load(doc, data_root=str(tmp_path))
    o = Oracle(sc, P)
    most = 0
    for _ in range(300):
        o.step(0.01)
        most = max(most, o.num_contacts())
    b = o.bodies()
    assert most > 0
    assert abs(b["v"][0]).max() < 1e-2
    assert 0.4 < b["x"][0][1] < 0.46         # resting on the leaves (r 0.45, at the centre's height)
