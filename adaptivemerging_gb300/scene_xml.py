"""Loader for the reference's XML scene files (XMLParser.java:40-661).

The supported subset is what the contact path simulates:
- ``<body type="box">`` with ``dim``, optional ``density`` (1) and ``scale``
  (XMLParser.java:360-397);
- ``<body type="sphere">`` with ``r`` and optional ``density`` (:420-447);
- ``<body type="plane">`` with ``p`` and ``n``, always pinned (:405-416);
- ``<body type="mesh">`` with ``obj``, ``st``, ``scale`` and optional
  ``density`` (createMesh, :449-539): mass, centre of mass and inertia of the
  scaled triangle soup, the box of its vertices about the centre of mass
  (the body's boundingBoxB, where the motion metric samples velocities), and
  the sphere tree of the ``.sph`` file, scaled and moved to the centre of
  mass.  Otherwise the mesh only draws; the sphere tree is what collides.

Each body may carry the child elements ``x``, ``R`` (axis x y z and angle),
``v``, ``omega``, ``friction``, ``restitution`` and ``pinned``
(setCommonAttributes, :545-590). ``magnetic``, ``factorypart`` and
``temporarilyPinned`` do not affect the contact path and are ignored.

The ``<collision>`` element sets ``iterations``, ``feedbackStiffness``,
``enableCompliance``, and ``restitution`` / ``friction``. The last two also
switch the corresponding override on, as the reference does (:100-137).
The ``<system>`` element only sets the mouse spring (:69-89) and is ignored.

Composite bodies, springs, spinners and ``enablePostStabilization="true"``
are not part of this implementation. They raise ``NotSupported`` instead of
being skipped, so a scene never loads silently different from the reference.
"""
import math
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import abi
from .scenes import IDENT, Builder, axis_angle


class NotSupported(ValueError):
    pass


def _vec(text, n=3):
    v = [float(t) for t in text.split()]
    if len(v) != n:
        raise ValueError(f"expected {n} numbers, got {text!r}")
    return v


def _common(el, composite=False):
    """x, R, v, omega, friction, restitution, pinned of one body element.
    ``events`` records the order of x, R and pinned, which decides when the
    reference refreshes the rotational inertia (setCommonAttributes)."""
    out = {"x": (0.0, 0.0, 0.0), "R": IDENT, "v": (0.0, 0.0, 0.0), "omega": (0.0, 0.0, 0.0),
           "friction": 0.8, "restitution": 0.0, "pinned": False, "events": []}
    for ch in el:
        tag = ch.tag.lower()
        text = (ch.text or "").strip()
        if tag == "x":
            out["x"] = tuple(_vec(text))
            out["events"].append(("x", out["R"], out["pinned"]))
        elif tag == "r":
            ax = _vec(text, 4)
            norm = (ax[0] ** 2 + ax[1] ** 2 + ax[2] ** 2) ** 0.5
            out["R"] = IDENT if norm == 0.0 else axis_angle(ax[:3], ax[3])
            out["events"].append(("R", out["R"], out["pinned"]))
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
        elif tag == "body" and composite:
            pass   # a composite's sub-body, read by _composite
        elif tag in ("spring", "spinner", "body"):
            raise NotSupported(f"<{ch.tag}> in body {el.get('name')!r}")
    return out


def _mul(A, B):
    """javax.vecmath Matrix3d.mul(A, B), row-major lists of 9."""
    return [A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c] for r in range(3) for c in range(3)]


def _mul_tr(A, B):
    """Matrix3d.mulTransposeRight(A, B) = A B^T."""
    return [A[3 * r] * B[3 * c] + A[3 * r + 1] * B[3 * c + 1] + A[3 * r + 2] * B[3 * c + 2]
            for r in range(3) for c in range(3)]


def _rm0rt(R, M0):
    """RigidTransform3D.computeRM0RT: R M0 R^T."""
    return _mul_tr(_mul(R, M0), R)


def _transform(R, t, p):
    """RigidTransform3D.transform(Point3d): R p + t, Matrix3d.transform order."""
    return [R[3 * r] * p[0] + R[3 * r + 1] * p[1] + R[3 * r + 2] * p[2] + t[r] for r in range(3)]


def _sub_body(el):
    """One box or sphere inside a composite, as createBox / createSphere and
    setCommonAttributes leave it (XMLParser.java:360-447, 545-590): mass,
    massAngular (refreshed to R M0 R^T at each x and R element while not
    pinned, and once more at the end for a box), pose and boundingBoxB.
    Other types give no sub-body, as in the reference (:216-231)."""
    kind = el.get("type", "").lower()
    c = _common(el)
    density = float(el.get("density", "1"))
    if kind == "box":
        s = _vec(el.get("dim"))
        if "scale" in el.attrib:
            k = float(el.get("scale"))
            s = [q * k for q in s]
        m = s[0] * s[1] * s[2] * density
        M0 = [1.0 / 12 * m * (s[1] * s[1] + s[2] * s[2]), 0.0, 0.0,
              0.0, 1.0 / 12 * m * (s[0] * s[0] + s[2] * s[2]), 0.0,
              0.0, 0.0, 1.0 / 12 * m * (s[0] * s[0] + s[1] * s[1])]
        h = [q * 0.5 for q in s]
        shape = [s[0], s[1], s[2], 0.0]
        typ = abi.AM_BOX
    elif kind == "sphere":
        r = float(el.get("r"))
        m = 4.0 / 3 * math.pi * r * r * r * density
        i = 2.0 / 5 * m * r * r
        M0 = [i, 0.0, 0.0, 0.0, i, 0.0, 0.0, 0.0, i]
        h = [r, r, r]
        shape = [r, 0.0, 0.0, 0.0]
        typ = abi.AM_SPHERE
    else:
        return None
    Ma = list(M0)
    for _, R, pinned in c["events"]:
        if not pinned:
            Ma = _rm0rt(R, M0)
    if kind == "box" and not c["pinned"]:
        Ma = _rm0rt(c["R"], M0)
    bb = [(-h[0], -h[1], -h[2]), (-h[0], -h[1], h[2]), (-h[0], h[1], -h[2]), (-h[0], h[1], h[2]),
          (h[0], -h[1], -h[2]), (h[0], -h[1], h[2]), (h[0], h[1], -h[2]), (h[0], h[1], h[2])]
    return {"type": typ, "shape": shape, "m": m, "M": Ma, "R": list(c["R"]), "x": list(c["x"]), "bbB": bb}


def _composite(el):
    """createComposite (XMLParser.java:180-352): the sub-bodies' total mass,
    centre of mass, inertia (their massAngular plus the parallel-axis term,
    summed in list order) and box (corners placed by each sub-body's pose,
    Math.min / Math.max from MAX_VALUE and Double.MIN_VALUE, then moved to the
    centre of mass); the composite's x is its element's x plus that centre,
    unrotated, as the reference adds it (:311-312); each sub-body's pose in
    the composite is its own rotation and its position less the centre."""
    subs = [q for q in (_sub_body(ch) for ch in el if ch.tag.lower() == "body") if q is not None]
    if not subs:
        raise NotSupported(f"composite {el.get('name')!r} without box or sphere bodies")
    mass = 0.0
    com = [0.0, 0.0, 0.0]
    for q in subs:
        mass += q["m"]
        com = [q["m"] * q["x"][k] + com[k] for k in range(3)]
    com = [v * (1.0 / mass) for v in com]
    M = [0.0] * 9
    for q in subs:
        M = [M[k] + q["M"][k] for k in range(9)]
        x, y, z = (q["x"][0] - com[0], q["x"][1] - com[1], q["x"][2] - com[2])
        x2, y2, z2 = x * x, y * y, z * z
        op = [y2 + z2, -x * y, -x * z, -y * x, x2 + z2, -y * z, -z * x, -z * y, x2 + y2]
        M = [M[k] + op[k] * q["m"] for k in range(9)]
    ll = [1.7976931348623157e308] * 3
    ur = [_DOUBLE_MIN_VALUE] * 3
    for q in subs:
        for p in q["bbB"]:
            w = _transform(q["R"], q["x"], p)
            for k in range(3):
                ll[k] = _jmin(w[k], ll[k])
                ur[k] = _jmax(w[k], ur[k])
    ll = [ll[k] - com[k] for k in range(3)]
    ur = [ur[k] - com[k] for k in range(3)]
    c = _common(el, composite=True)
    x = [c["x"][k] + com[k] for k in range(3)]
    parts = [(q["type"], q["shape"], q["R"], [q["x"][k] - com[k] for k in range(3)]) for q in subs]
    return c, x, mass, M, ll + ur, parts


def read_obj(path):
    """Vertices and faces of a Wavefront OBJ file as PolygonSoup reads it
    (tools/moments/PolygonSoup.java:40-115): ``v x y z`` lines, and ``f``
    lines whose tokens start with a 1-based vertex index (texture and normal
    indices after a slash are ignored)."""
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                t = line.split()
                verts.append((float(t[1]), float(t[2]), float(t[3])))
            elif line.startswith("f "):
                faces.append([int(tok.split("/")[0]) - 1 for tok in line[2:].split()])
    return np.array(verts, float).reshape(-1, 3), faces


def mesh_mass_properties(verts, faces, density):
    """Mass, centre of mass and inertia about it (VolInt.computeMassProperties,
    tools/moments/VolInt.java:316-380), from the volume integrals of the
    closed triangle soup that getPolyhedron builds from the first three
    vertices of every face (PolygonSoup.java:157-166).  The integrals T0, T1,
    T2 and TP are Mirtich's (1996); here they are summed over the signed
    tetrahedra spanned by the origin and each triangle, which gives the same
    values up to rounding.  As the reference does, an inside-out soup (negative
    mass) gets its mass negated and nothing else."""
    tri = np.array([f[:3] for f in faces], int)
    a, b, c = verts[tri[:, 0]], verts[tri[:, 1]], verts[tri[:, 2]]
    d = np.einsum("ij,ij->i", a, np.cross(b, c))          # 6 x signed volume
    S = a + b + c
    T0 = d.sum() / 6.0
    T1 = (d[:, None] * S).sum(0) / 24.0
    # integral of x_i x_j over the tetrahedron (0, a, b, c): d/120 (sum of v_i v_j over a, b, c + S_i S_j)
    Q = (np.einsum("k,ki,kj->ij", d, a, a) + np.einsum("k,ki,kj->ij", d, b, b) + np.einsum("k,ki,kj->ij", d, c, c)
         + np.einsum("k,ki,kj->ij", d, S, S)) / 120.0
    T2 = np.diag(Q)
    TP = np.array([Q[0, 1], Q[1, 2], Q[2, 0]])
    mass = density * T0
    r = T1 / T0
    J = np.zeros((3, 3))
    J[0, 0] = density * (T2[1] + T2[2])
    J[1, 1] = density * (T2[2] + T2[0])
    J[2, 2] = density * (T2[0] + T2[1])
    J[0, 1] = J[1, 0] = -density * TP[0]
    J[1, 2] = J[2, 1] = -density * TP[1]
    J[2, 0] = J[0, 2] = -density * TP[2]
    J[0, 0] -= mass * (r[1] * r[1] + r[2] * r[2])
    J[1, 1] -= mass * (r[2] * r[2] + r[0] * r[0])
    J[2, 2] -= mass * (r[0] * r[0] + r[1] * r[1])
    J[0, 1] = J[1, 0] = J[0, 1] + mass * r[0] * r[1]
    J[1, 2] = J[2, 1] = J[1, 2] + mass * r[1] * r[2]
    J[2, 0] = J[0, 2] = J[2, 0] + mass * r[2] * r[0]
    if mass < 0:
        mass = -mass
    return float(mass), r, J


_DOUBLE_MIN_VALUE = float.fromhex("0x0.0000000000001p-1022")   # java.lang.Double.MIN_VALUE


def _jmin(a, b):
    """java.lang.Math.min for doubles: NaN first, -0.0 below +0.0."""
    if a != a:
        return a
    if a == 0.0 and b == 0.0 and math.copysign(1.0, b) < 0:
        return b
    return a if a <= b else b


def _jmax(a, b):
    """java.lang.Math.max for doubles: NaN first, +0.0 above -0.0."""
    if a != a:
        return a
    if a == 0.0 and b == 0.0 and math.copysign(1.0, a) < 0:
        return b
    return a if a >= b else b


def mesh_box(points):
    """The mesh body's boundingBoxB corners as (ll, ur) (XMLParser.java:
    474-493): over the scaled vertices moved to the centre of mass, in the
    file's order.  As in the reference, the upper corner starts at
    Double.MIN_VALUE (the smallest positive double), so an axis on which
    every vertex is negative keeps that value."""
    ll = [1.7976931348623157e308] * 3
    ur = [_DOUBLE_MIN_VALUE] * 3
    for p in points:
        for k in range(3):
            q = float(p[k])
            ll[k] = _jmin(q, ll[k])
            ur[k] = _jmax(q, ur[k])
    return ll + ur


def read_sphere_tree(path):
    """A ``.sph`` sphere tree as createMesh reads it (XMLParser.java:499-534):
    the number of spheres, one ``x y z r`` line per sphere, then lines
    ``parent count child ...`` with 1-based indices.  Sphere 1 is the root.
    Returns (centres, radii, children as lists of 0-based indices)."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    cr = np.array([[float(t) for t in lines[1 + k].split()[:4]] for k in range(n)], float).reshape(-1, 4)
    children = {k: [] for k in range(n)}
    for line in lines[1 + n:]:
        t = line.split()
        if len(t) < 2:
            break          # the reference's scanner stops at the first line without a parent and a count
        p, cnt = int(t[0]) - 1, int(t[1])
        children[p] = [int(q) - 1 for q in t[2:2 + cnt]]
    return cr[:, :3], cr[:, 3], children


def load(source, params=None, data_root=None, composites=False):
    """Parse an XML scene (a path, or the document text when it starts with
    '<').  Mesh bodies name their ``obj`` and ``st`` files relative to the
    reference project's root, which `data_root` gives (default: the parent of
    the XML file's directory, as for ``scenes3D/*.xml``).  Returns
    (SceneArrays, am_params, body names in list order)."""
    text = source.lstrip().startswith("<")
    root = ET.fromstring(source) if text else ET.parse(source).getroot()
    if data_root is None and not text:
        data_root = os.path.dirname(os.path.dirname(os.path.abspath(source)))
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
        if a.get("enablePostStabilization", "").lower() == "true":
            raise NotSupported("enablePostStabilization (the post-stabilization solve, "
                               "RigidBodySystem.java:354-376)")
    b = Builder()
    names = []
    for el in root:
        if el.tag.lower() != "body":
            continue
        kind = el.get("type", "").lower()
        name = el.get("name", "")
        c = _common(el, composite=(kind == "composite" and composites))
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
        elif kind == "mesh":
            if data_root is None:
                raise NotSupported(f"mesh body {name!r}: no data root for its files")
            scale = float(el.get("scale"))
            verts, faces = read_obj(os.path.join(data_root, el.get("obj")))
            mass, com, J = mesh_mass_properties(verts * scale, faces, density)
            cs, rs, children = read_sphere_tree(os.path.join(data_root, el.get("st")))
            b.tree(cs * scale - com, rs * scale, children, c["x"], mass, J, R=c["R"], v=c["v"], omega=c["omega"],
                   friction=c["friction"], restitution=c["restitution"], pinned=c["pinned"],
                   bbox=mesh_box(verts * scale - com))
        elif kind == "composite" and composites:
            cc, x, mass, M, box, parts = _composite(el)
            b.composite(x, mass, M, box, parts, R=cc["R"], v=cc["v"], omega=cc["omega"], friction=cc["friction"],
                        restitution=cc["restitution"], pinned=cc["pinned"])
        else:
            raise NotSupported(f"body type {kind!r} ({name!r})")
        names.append(name)
    return b.build(), P, names
