"""Scene generators: mass properties follow the reference loader
(XMLParser.java:360-447) and the benchmark workloads have their stated sizes."""
import math

import numpy as np

from adaptivemerging_gb300 import abi, scenes


def test_box_and_sphere_mass_properties():
    B = scenes.Builder()
    B.box((1.0, 0.5, 2.0), (0, 0, 0), density=1000.0)
    B.sphere(0.3, (0, 2, 0), density=2.0)
    s = B.build()
    m = 1.0 * 0.5 * 2.0 * 1000.0
    assert s["mass"][0] == m
    I = s["inertia"][0:9].reshape(3, 3)
    assert I[0, 0] == 1.0 / 12 * m * (0.25 + 4.0) and I[1, 1] == 1.0 / 12 * m * (1.0 + 4.0)
    ms = 4.0 / 3 * math.pi * 0.3 ** 3 * 2.0
    assert s["mass"][1] == ms and s["inertia"][9] == 2.0 / 5 * ms * 0.3 * 0.3


def test_workload_sizes():
    w = scenes.wall()
    assert w.n == 1 + 40 * 25 + 1
    assert (w["type"] == abi.AM_BOX).sum() == 1000 and (w["type"] == abi.AM_SPHERE).sum() == 1
    proj = np.nonzero(w["type"] == abi.AM_SPHERE)[0][0]
    assert w["mass"][proj] == 50.0 and w["v"][3 * proj + 2] == 15.0
    t = scenes.tower(25, seed=1)
    assert t.n == 26 and np.allclose(t["mass"][1:], 500.0)


def test_clump_tree_is_consistent():
    B = scenes.Builder()
    B.clump([(0, 0, 0), (0.1, 0, 0), (0, 0.1, 0.05)], [0.05, 0.06, 0.04], (0, 1, 0), density=1000.0)
    s = B.build()
    root = s["body_root"][0]
    c0, n = s["node_child0"][root], s["node_nchild"][root]
    assert n == 3 and c0 == root + 1
    cs = s["node_c"].reshape(-1, 3)[c0:c0 + n]
    rs = s["node_r"][c0:c0 + n]
    ms = rs ** 3
    assert np.allclose((ms[:, None] * cs).sum(0), 0, atol=1e-15)      # leaves re-centred on the COM
    assert all(np.linalg.norm(cs[k]) + rs[k] <= s["node_r"][root] + 1e-15 for k in range(n))
