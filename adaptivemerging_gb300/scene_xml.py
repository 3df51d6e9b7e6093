"""Loader for the reference's XML scene files (XMLParser.java:40-661).

The supported subset is what the contact path simulates:
- ``<body type="box">`` with ``dim``, optional ``density`` (1) and ``scale``
  (XMLParser.java:360-397);
- ``<body type="sphere">`` with ``r`` and optional ``density`` (:420-447);
- ``<body type="plane">`` with ``p`` and ``n``, always pinned (:405-416).

Each body may carry the child elements ``x``, ``R`` (axis x y z and angle),
``v``, ``omega``, ``friction``, ``restitution`` and ``pinned``
(setCommonAttributes, :545-590). ``magnetic``, ``factorypart`` and
``temporarilyPinned`` do not affect the contact path and are ignored.

The ``<collision>`` element sets ``iterations``, ``feedbackStiffness``,
``enableCompliance``, and ``restitution`` / ``friction``. The last two also
switch the corresponding override on, as the reference does (:100-137).

Composite and mesh bodies, springs and spinners are not part of this
implementation. They raise ``NotSupported`` instead of being skipped, so a
scene never loads silently different from the reference.
"""
import xml.etree.ElementTree as ET

from . import abi
from .scenes import IDENT, Builder, axis_angle


class NotSupported(ValueError):
    pass


def _vec(text, n=3):
    v = [float(t) for t in text.split()]
    if len(v) != n:
        raise ValueError(f"expected {n} numbers, got {text!r}")
    return v


def _common(el):
    """x, R, v, omega, friction, restitution, pinned of one body element."""
    out = {"x": (0.0, 0.0, 0.0), "R": IDENT, "v": (0.0, 0.0, 0.0), "omega": (0.0, 0.0, 0.0),
           "friction": 0.8, "restitution": 0.0, "pinned": False}
    for ch in el:
        tag = ch.tag.lower()
        text = (ch.text or "").strip()
        if tag == "x":
            out["x"] = tuple(_vec(text))
        elif tag == "r":
            ax = _vec(text, 4)
            norm = (ax[0] ** 2 + ax[1] ** 2 + ax[2] ** 2) ** 0.5
            out["R"] = IDENT if norm == 0.0 else axis_angle(ax[:3], ax[3])
        elif tag == "v":
            out["v"] = tuple(_vec(text))
        elif tag == "omega":
            out["omega"] = tuple(_vec(text))
        elif tag == "friction":
            out["friction"] = float(text.split()[0])
        elif tag == "restitution":
            out["restitution"] = float(text.split()[0])
        elif tag == "pinned":
            out["pinned"] = text.split()[0].lower() == "true"
        elif tag in ("magnetic", "factorypart", "temporarilypinned", "col"):
            pass
        elif tag in ("spring", "spinner", "body"):
            raise NotSupported(f"<{ch.tag}> in body {el.get('name')!r}")
    return out


def load(source, params=None):
    """Parse an XML scene (a path, or the document text when it starts with
    '<').  Returns (SceneArrays, am_params, body names in list order)."""
    root = ET.fromstring(source) if source.lstrip().startswith("<") else ET.parse(source).getroot()
    P = params if params is not None else abi.default_params()
    for el in root:
        if el.tag.lower() != "collision":
            continue
        a = el.attrib
        if "iterations" in a:
            P.iterations = int(a["iterations"])
        if "feedbackStiffness" in a:
            P.feedback_stiffness = float(a["feedbackStiffness"])
        if "restitution" in a:
            P.restitution = float(a["restitution"])
            P.restitution_override = 1
        if "friction" in a:
            P.friction = float(a["friction"])
            P.friction_override = 1
        if "enableCompliance" in a:
            P.enable_compliance = int(a["enableCompliance"].lower() == "true")
    b = Builder()
    names = []
    for el in root:
        if el.tag.lower() != "body":
            continue
        kind = el.get("type", "").lower()
        name = el.get("name", "")
        c = _common(el)
        density = float(el.get("density", "1"))
        if kind == "box":
            s = _vec(el.get("dim"))
            if "scale" in el.attrib:
                k = float(el.get("scale"))
                s = [k * q for q in s]
            b.box(s, c["x"], R=c["R"], density=density, pinned=c["pinned"], v=c["v"], omega=c["omega"],
                  friction=c["friction"], restitution=c["restitution"])
        elif kind == "sphere":
            b.sphere(float(el.get("r")), c["x"], density=density, pinned=c["pinned"], v=c["v"],
                     omega=c["omega"], friction=c["friction"], restitution=c["restitution"], R=c["R"])
        elif kind == "plane":
            b.plane(tuple(_vec(el.get("p"))), tuple(_vec(el.get("n"))), friction=c["friction"],
                    restitution=c["restitution"])
        else:
            raise NotSupported(f"body type {kind!r} ({name!r})")
        names.append(name)
    return b.build(), P, names
