"""The broad phase's FP32 tests may only decide pairs the exact FP64 quick exit
(BoxBox.java:466, BoxSphere.java:157, BVSphere.java:184-186) decides the same
way: far_apart32 only pairs it rejects, near32 only pairs it accepts.
Restated here in float32 with numpy and driven at the boundary: centres at
distance (ra + rb)(1 +- tiny), at coordinates up to 1e4 m."""
import numpy as np


def far_apart32(ca, cb):
    f = np.float32
    a = ca.astype(f)
    b = cb.astype(f)
    d = a[:, :3] - b[:, :3]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    size = f(1) + np.abs(a[:, 0]) + np.abs(a[:, 1]) + np.abs(a[:, 2]) + np.abs(b[:, 0]) + np.abs(b[:, 1]) + np.abs(b[:, 2])
    T = (a[:, 3] + b[:, 3]) * f(1.00001) + f(1e-6) * size
    return d2 > T * T


def near32(ca, cb):
    f = np.float32
    a = ca.astype(f)
    b = cb.astype(f)
    d = a[:, :3] - b[:, :3]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    size = f(1) + np.abs(a[:, 0]) + np.abs(a[:, 1]) + np.abs(a[:, 2]) + np.abs(b[:, 0]) + np.abs(b[:, 1]) + np.abs(b[:, 2])
    T = (a[:, 3] + b[:, 3]) * f(0.99999) - f(1e-6) * size
    return (T > 0) & (d2 < T * T)


def test_prefilter_is_conservative():
    rng = np.random.default_rng(0)
    for scale in (1.0, 10.0, 100.0, 1e4):
        n = 200_000
        ca = np.zeros((n, 4))
        cb = np.zeros((n, 4))
        ca[:, :3] = rng.uniform(-scale, scale, (n, 3))
        ca[:, 3] = rng.uniform(0.01, 1.0, n)
        cb[:, 3] = rng.uniform(0.01, 1.0, n)
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1)[:, None]
        rr = ca[:, 3] + cb[:, 3]
        dist = rr * (1 + rng.uniform(-1e-5, 1e-5, n) * rng.choice([1e-3, 1.0, 10.0], n))
        cb[:, :3] = ca[:, :3] + u * dist[:, None]
        exact_reject = np.linalg.norm(cb[:, :3] - ca[:, :3], axis=1) > rr
        far = far_apart32(ca, cb)
        assert not np.any(far & ~exact_reject), scale
        near = near32(ca, cb)
        assert not np.any(near & exact_reject), scale
        # and it does reject clearly separated pairs
        cb2 = cb.copy()
        cb2[:, :3] = ca[:, :3] + u * (2.0 * rr)[:, None]
        assert far_apart32(ca, cb2).mean() > 0.99
        # and accepts clearly overlapping ones
        cb3 = cb.copy()
        cb3[:, :3] = ca[:, :3] + u * (0.5 * rr)[:, None]
        if scale <= 100.0:
            assert near32(ca, cb3).mean() > 0.99
