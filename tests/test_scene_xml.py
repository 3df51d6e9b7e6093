"""The XML scene loader (the reference's scene format, XMLParser.java):
mass properties, axis-angle orientation, collision overrides, the refusal of
unsupported elements, and the loaded scene on the oracle (CPU) and, marked
gpu, bit-exact on the device path."""
import math

import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scene_xml

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
