"""Seeded synthetic scenes (structure-of-arrays am_scene inputs).

Mass properties follow the reference scene loader (XMLParser.java:360-447):
box mass = sx*sy*sz*density, inertia = m/12 diag(sy^2+sz^2, sx^2+sz^2,
sx^2+sy^2); sphere mass = 4/3 pi r^3 density, inertia = 2/5 m r^2 I.  The
reference's benchmark scenes are not public datasets; these generators build
the benchmark workloads (tower, brick wall + projectile, batched bins, clumps)
from a seed with the sizes and distributions the benchmark names.
"""
import math

import numpy as np

from .abi import AM_BOX, AM_COMPOSITE, AM_PLANE, AM_SPHERE, AM_TREE, SceneArrays


def yaw(theta):
    """Rotation about +y (row-major)."""
    c, s = math.cos(theta), math.sin(theta)
    return [c, 0.0, s, 0.0, 1.0, 0.0, -s, 0.0, c]


def axis_angle(ax, theta):
    ax = np.asarray(ax, float)
    ax = ax / np.linalg.norm(ax)
    x, y, z = ax
    c, s = math.cos(theta), math.sin(theta)
    t = 1 - c
    return [t * x * x + c, t * x * y - s * z, t * x * z + s * y,
            t * x * y + s * z, t * y * y + c, t * y * z - s * x,
            t * x * z - s * y, t * y * z + s * x, t * z * z + c]


IDENT = [1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0]

# Composite bodies (AM_COMPOSITE): the oracle steps them; the library has no
# device path for them yet and refuses the type.
COMPOSITE = AM_COMPOSITE


class Builder:
    def __init__(self):
        self.b = []          # per-body dicts
        self.nodes = []      # (c, r, child0, nchild)
        self.subs = []       # composite sub-bodies: (parent, type, shape[4], R[9], t[3])

    def _add(self, **kw):
        d = dict(type=AM_BOX, pinned=0, x=(0, 0, 0), R=IDENT, v=(0, 0, 0), omega=(0, 0, 0),
                 mass=0.0, inertia=[0.0] * 9, friction=0.8, restitution=0.0,
                 shape=(0, 0, 0, 0), root=-1, bbox=None)
        d.update(kw)
        self.b.append(d)
        return len(self.b) - 1

    def box(self, size, x, R=IDENT, density=1.0, pinned=False, v=(0, 0, 0), omega=(0, 0, 0),
            friction=0.8, restitution=0.0):
        sx, sy, sz = size
        m = sx * sy * sz * density
        I = [1.0 / 12 * m * (sy * sy + sz * sz), 0, 0, 0, 1.0 / 12 * m * (sx * sx + sz * sz), 0,
             0, 0, 1.0 / 12 * m * (sx * sx + sy * sy)]
        return self._add(type=AM_BOX, pinned=int(pinned), x=x, R=R, v=v, omega=omega, mass=m,
                         inertia=I, friction=friction, restitution=restitution,
                         shape=(sx, sy, sz, 0.0))

    def sphere(self, r, x, density=1.0, mass=None, pinned=False, v=(0, 0, 0), omega=(0, 0, 0),
               friction=0.8, restitution=0.0, R=IDENT):
        m = 4.0 / 3 * math.pi * r * r * r * density if mass is None else float(mass)
        i = 2.0 / 5 * m * r * r
        root = len(self.nodes)
        self.nodes.append(((0.0, 0.0, 0.0), r, -1, 0))
        return self._add(type=AM_SPHERE, pinned=int(pinned), x=x, R=R, v=v, omega=omega, mass=m,
                         inertia=[i, 0, 0, 0, i, 0, 0, 0, i], friction=friction,
                         restitution=restitution, shape=(r, 0, 0, 0), root=root)

    def plane(self, p, n, friction=0.8, restitution=0.0):
        return self._add(type=AM_PLANE, pinned=1, x=p, shape=(n[0], n[1], n[2], 0.0),
                         friction=friction, restitution=restitution)

    def clump(self, centres, radii, x, density=1.0, R=IDENT, v=(0, 0, 0), friction=0.8,
              restitution=0.0):
        """Sphere-tree body: a root sphere enclosing leaf spheres (2-level
        BVNode tree).  Mass and inertia sum the leaf spheres with the
        parallel-axis theorem about their mass-weighted centre, and the leaf
        centres are re-expressed about that centre."""
        centres = np.asarray(centres, float)
        radii = np.asarray(radii, float)
        ms = 4.0 / 3 * math.pi * radii ** 3 * density
        m = float(ms.sum())
        com = (ms[:, None] * centres).sum(0) / m
        c = centres - com
        I = np.zeros((3, 3))
        for k in range(len(radii)):
            I += 2.0 / 5 * ms[k] * radii[k] ** 2 * np.eye(3)
            d = c[k]
            I += ms[k] * (np.dot(d, d) * np.eye(3) - np.outer(d, d))
        rr = float(max(np.linalg.norm(c[k]) + radii[k] for k in range(len(radii))))
        root = len(self.nodes)
        self.nodes.append(((0.0, 0.0, 0.0), rr, root + 1, len(radii)))
        for k in range(len(radii)):
            self.nodes.append((tuple(c[k]), float(radii[k]), -1, 0))
        return self._add(type=AM_TREE, x=tuple(np.asarray(x, float) + 0.0), R=R, v=v, mass=m,
                         inertia=list(I.reshape(-1)), friction=friction,
                         restitution=restitution, root=root)

    def tree(self, centres, radii, children, x, mass, inertia, R=IDENT, v=(0, 0, 0), omega=(0, 0, 0),
             friction=0.8, restitution=0.0, pinned=False, bbox=None):
        """Sphere-tree body of any depth: node k has centre centres[k] and
        radius radii[k] in body coordinates and the child nodes children[k]
        (in their order); node 0 is the root.  The nodes are stored breadth
        first, so every node's children sit together in that order.  `bbox`
        (ll, ur: six numbers in body coordinates) is the body's bounding box
        for the motion metric, a mesh body's mesh box; without it the box of
        the leaf spheres is used."""
        order, pos = [0], {0: 0}
        for k in order:
            for q in children[k]:
                if q not in pos:
                    pos[q] = len(order)
                    order.append(q)
        base = len(self.nodes)
        for k in order:
            ch = list(children[k])
            if [pos[q] for q in ch] != list(range(pos[ch[0]], pos[ch[0]] + len(ch))) if ch else False:
                raise ValueError("sphere tree: a node is the child of more than one node")
            c0 = base + pos[ch[0]] if ch else -1
            self.nodes.append((tuple(float(t) for t in centres[k]), float(radii[k]), c0, len(ch)))
        return self._add(type=AM_TREE, x=tuple(float(t) for t in x), R=R, v=v, omega=omega, mass=float(mass),
                         inertia=[float(t) for t in np.asarray(inertia, float).reshape(-1)], friction=friction,
                         restitution=restitution, root=base, pinned=int(bool(pinned)),
                         bbox=None if bbox is None else [float(t) for t in bbox])

    def composite(self, x, mass, inertia, bbox, subs, R=IDENT, v=(0, 0, 0), omega=(0, 0, 0), friction=0.8,
                  restitution=0.0, pinned=False):
        """A composite body (the reference's RigidBodyGeomComposite): rigid
        body data as given, and its box and sphere sub-bodies as (type,
        shape[4], R[9], t[3]) with their pose in the composite's frame (the
        am_scene sub-body arrays).  Only the oracle steps composites; the
        library refuses their body type."""
        i = self._add(type=COMPOSITE, pinned=int(bool(pinned)), x=tuple(float(t) for t in x), R=R, v=v,
                      omega=omega, mass=float(mass), inertia=[float(t) for t in np.asarray(inertia).reshape(-1)],
                      friction=friction, restitution=restitution, bbox=[float(t) for t in bbox])
        for typ, shape, Rs, ts in subs:
            self.subs.append((i, typ, list(shape), list(Rs), list(ts)))
        return i

    def build(self):
        n = len(self.b)
        f = lambda k, w: np.array([d[k] for d in self.b], float).reshape(n * w)
        nodes = self.nodes if self.nodes else []
        extra = {}
        if self.subs:
            extra.update(sub_parent=[q[0] for q in self.subs], sub_type=[q[1] for q in self.subs],
                         sub_shape=np.array([q[2] for q in self.subs], float).reshape(-1),
                         sub_R=np.array([q[3] for q in self.subs], float).reshape(-1),
                         sub_t=np.array([q[4] for q in self.subs], float).reshape(-1))
        if any(d["bbox"] is not None for d in self.b):
            extra["bbox"] = np.array([d["bbox"] if d["bbox"] is not None else [np.nan] * 6 for d in self.b],
                                     float).reshape(-1)
        sc = SceneArrays(
            type=[d["type"] for d in self.b], pinned=[d["pinned"] for d in self.b],
            x=f("x", 3), R=f("R", 9), v=f("v", 3), omega=f("omega", 3),
            mass=[d["mass"] for d in self.b], inertia=f("inertia", 9),
            friction=[d["friction"] for d in self.b], restitution=[d["restitution"] for d in self.b],
            shape=f("shape", 4), body_root=[d["root"] for d in self.b],
            node_c=np.array([c for c, _, _, _ in nodes], float).reshape(-1),
            node_r=np.array([r for _, r, _, _ in nodes], float),
            node_child0=[c0 for _, _, c0, _ in nodes], node_nchild=[nc for _, _, _, nc in nodes],
            **extra,
        )
        return sc


# --------------------------------------------------------------------------
# Benchmark workloads
def tower(n_boxes=25, seed=1, size=(1.0, 0.5, 1.0), density=1000.0):
    """Tower of `n_boxes` boxes (1.0 x 0.5 x 1.0 m, density 1000) stacked on a
    static ground plane; each box offset by U(+-0.01) m in x/z and U(+-0.5)
    degrees of yaw."""
    rng = np.random.default_rng(seed)
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0))
    h = size[1]
    for i in range(n_boxes):
        dx, dz = rng.uniform(-0.01, 0.01, 2)
        th = math.radians(rng.uniform(-0.5, 0.5))
        B.box(size, (dx, h / 2 + h * i, dz), R=yaw(th), density=density)
    return B.build()


def wall(cols=40, rows=25, seed=2, brick=(0.4, 0.2, 0.2), density=1000.0, gap=0.01,
         projectile=True):
    """Running-bond wall of cols x rows bricks (0.4 x 0.2 x 0.2 m, density
    1000, positions jittered U(+-2 mm) in x/z) on a ground plane, and a sphere
    projectile (r = 0.3 m, 50 kg) fired at 15 m/s at a seeded height."""
    rng = np.random.default_rng(seed)
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0))
    bx, by, bz = brick
    pitch = bx + gap
    for j in range(rows):
        off = 0.5 * pitch * (j % 2)
        for i in range(cols):
            dx, dz = rng.uniform(-0.002, 0.002, 2)
            x = -0.5 * cols * pitch + (i + 0.5) * pitch + off + dx
            B.box(brick, (x, by / 2 + by * j, dz), density=density)
    if projectile:
        hgt = float(rng.uniform(0.5, rows * by * 0.8))
        B.sphere(0.3, (0.0, hgt, -3.0), mass=50.0, v=(0.0, 0.0, 15.0))
    return B.build()


def random_pile(n=30, seed=0, kinds=("box", "sphere"), extent=3.0, height=4.0):
    """Small random scene for parity tests: boxes and spheres over a plane,
    dropped from a jittered grid (no initial overlaps)."""
    rng = np.random.default_rng(seed)
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0))
    side = int(math.ceil(n ** (1 / 3)))
    k = 0
    for iy in range(side * 4):
        for ix in range(side):
            for iz in range(side):
                if k >= n:
                    break
                p = (-extent / 2 + (ix + 0.5) * extent / side + rng.uniform(-0.05, 0.05),
                     0.6 + iy * 0.9 + rng.uniform(0, 0.05),
                     -extent / 2 + (iz + 0.5) * extent / side + rng.uniform(-0.05, 0.05))
                kind = kinds[int(rng.integers(len(kinds)))]
                if kind == "box":
                    s = tuple(rng.uniform(0.2, 0.6, 3))
                    B.box(s, p, R=axis_angle(rng.normal(size=3), rng.uniform(0, math.pi)),
                          density=rng.uniform(500, 2000), friction=float(rng.uniform(0.3, 0.9)))
                elif kind == "sphere":
                    B.sphere(float(rng.uniform(0.1, 0.3)), p, density=rng.uniform(500, 2000),
                             friction=float(rng.uniform(0.3, 0.9)))
                else:
                    m = int(rng.integers(4, 9))
                    cs = rng.uniform(-0.12, 0.12, (m, 3))
                    rs = rng.uniform(0.06, 0.12, m)
                    B.clump(cs, rs, p, density=rng.uniform(500, 2000))
                k += 1
    return B.build()


FUNNEL_PLATFORM = 1   # body index of funnel_clumps' platform


def funnel_clumps(n_clumps=200, seed=5, top=3.0, bottom=0.5, height=3.0, base=1.0):
    """Clumps poured into a funnel over a platform (the large-scene workload's
    geometry, scaled by `n_clumps`).  Each clump is a sphere tree of 4-16
    spheres, r U(0.02, 0.08) m, in a compact random cluster, density
    U(500, 2000).  The funnel is four pinned box panels forming a truncated
    pyramid (half-widths `top` to `bottom`) whose lower rim sits `base` m
    above a pinned platform box (body FUNNEL_PLATFORM) on the ground plane.
    The clumps start in a jittered grid inside the funnel, so they meet the
    panels at once.  The platform is pinned; the large-scene workload makes
    it oscillate with am_set_kinematic (0.5 Hz, 0.05 m, vertical)."""
    rng = np.random.default_rng(seed)
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0), friction=0.7)
    B.box((2.0 * (bottom + 1.0), 0.2, 2.0 * (bottom + 1.0)), (0.0, 0.1, 0.0), pinned=True, friction=0.7)
    y0 = 0.2 + base
    slope = math.atan2(top - bottom, height)          # panel tilt from vertical
    length = math.hypot(top - bottom, height)
    cy = y0 + height / 2
    ch = (top + bottom) / 2
    t = 0.05
    for (ax, sx, sz, px, pz, sign) in ((2, 2 * top, t, 0.0, ch, 1.0), (2, 2 * top, t, 0.0, -ch, -1.0),
                                      (0, t, 2 * top, ch, 0.0, -1.0), (0, t, 2 * top, -ch, 0.0, 1.0)):
        # the panel's long side runs along the slope: tilt about the horizontal axis parallel to it
        # (about +x, +angle tips the top towards +z; about +z, +angle tips it towards -x)
        axis = (1.0, 0.0, 0.0) if ax == 2 else (0.0, 0.0, 1.0)
        R = axis_angle(axis, sign * slope)
        size = (sx, length, sz)
        B.box(size, (px, cy, pz), R=R, pinned=True, friction=0.7)
    pitch = 0.3
    k = 0
    layer = 0
    while k < n_clumps:
        y = y0 + height * 0.35 + layer * pitch
        half = bottom + (top - bottom) * min(1.0, (y - y0) / height) - 0.25
        m = max(1, int(2 * half / pitch))
        for i in range(m):
            for j in range(m):
                if k >= n_clumps:
                    break
                x = -half + (i + 0.5) * (2 * half / m) + rng.uniform(-0.02, 0.02)
                z = -half + (j + 0.5) * (2 * half / m) + rng.uniform(-0.02, 0.02)
                nsph = int(rng.integers(4, 17))
                rs = rng.uniform(0.02, 0.08, nsph)
                cs = rng.normal(size=(nsph, 3)) * 0.04
                B.clump(cs, rs, (x, y, z), density=float(rng.uniform(500, 2000)), friction=0.7,
                        R=axis_angle(rng.normal(size=3), rng.uniform(0, math.pi)))
                k += 1
        layer += 1
    return B.build()


def bin_scene(n_bodies, seed, extent=10.0, wall_height=12.0, box_frac=0.5, gap=0.01):
    """One scene of the batched workload: `n_bodies` boxes (sides U(0.1, 1.0)
    m) and spheres (r U(0.05, 0.5) m), density U(500, 2000) kg/m3, in a 10 x
    10 m bin (four pinned box walls on a ground plane).  Bodies are dropped
    from a jittered grid of columns: each body starts `gap` (1 cm) above the
    one below it, axis aligned, so no two bodies overlap initially (a negative
    gap starts them in slight contact).  All bodies of the
    scene share a friction coefficient mu ~ U(0.3, 0.8) (the reference's
    friction mixing rule then gives mu for every contact)."""
    rng = np.random.default_rng(seed)
    mu = float(rng.uniform(0.3, 0.8))
    B = Builder()
    B.plane((0, 0, 0), (0, 1, 0), friction=mu)
    t = 0.5
    h = extent / 2 + t / 2
    for (x, z, sx, sz) in ((h, 0, t, extent + 2 * t), (-h, 0, t, extent + 2 * t),
                           (0, h, extent, t), (0, -h, extent, t)):
        B.box((sx, wall_height, sz), (x, wall_height / 2, z), pinned=True, density=1000.0, friction=mu)
    pitch = 1.05
    ncol = int(extent / pitch)
    tops = np.zeros((ncol, ncol))
    for k in range(n_bodies):
        c = int(rng.integers(ncol * ncol))
        i, j = divmod(c, ncol)
        x = -extent / 2 + (i + 0.5) * pitch + rng.uniform(-0.02, 0.02)
        z = -extent / 2 + (j + 0.5) * pitch + rng.uniform(-0.02, 0.02)
        dens = float(rng.uniform(500, 2000))
        if rng.uniform() < box_frac:
            s = tuple(float(v) for v in rng.uniform(0.1, 1.0, 3))
            y = tops[i, j] + gap + s[1] / 2
            B.box(s, (x, y, z), density=dens, friction=mu)
            tops[i, j] = y + s[1] / 2
        else:
            r = float(rng.uniform(0.05, 0.5))
            y = tops[i, j] + gap + r
            B.sphere(r, (x, y, z), density=dens, friction=mu)
            tops[i, j] = y + r
    return B.build()


def batch_scenes(n_scenes=512, seed=3, n_min=20, n_max=2000):
    """The batched workload: `n_scenes` independent bins whose body counts are
    log-uniform in [n_min, n_max] (seeded)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_scenes)).astype(int)
    return [bin_scene(int(n), seed * 100003 + k) for k, n in enumerate(counts)]
