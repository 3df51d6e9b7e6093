"""Batched scenes: collision and contact setup stay bit-exact per scene (the
FP64 pipeline is shared), and the FP32 one-CTA-per-scene solve converges to
the oracle's FP64 fixed point within FP32 tolerance."""
import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scenes
from helpers import compare_contacts, params
from oracle_binding import Oracle

pytestmark = pytest.mark.gpu

DT = 0.005


def _scenes():
    # bodies start 1 mm into each other, so the first step already has contacts
    return [scenes.bin_scene(n, 1000 + n, gap=-0.001) for n in (25, 40, 60, 33, 80)]


def _local(c, off, node_off, plane_ids):
    """map global body / bv ids of one scene's contacts back to scene-local ids"""
    out = dict(c)
    out["body1"] = c["body1"] - off
    out["body2"] = c["body2"] - off
    for k in ("bv1", "bv2"):
        v = c[k].copy()
        real = v >= 0
        v[real] -= node_off
        pl = v <= -2
        v[pl] = -2 - ((-2 - v[pl]) - off)
        out[k] = v
    return out


def _split(cg, sc_list):
    offs = np.cumsum([0] + [s.n for s in sc_list])
    node_offs = np.cumsum([0] + [s.n_nodes for s in sc_list])
    parts = []
    for k in range(len(sc_list)):
        sel = (cg["body1"] >= offs[k]) & (cg["body1"] < offs[k + 1])
        part = {f: v[sel] for f, v in cg.items()}
        parts.append(_local(part, offs[k], node_offs[k], None))
    return parts


def test_batch_contacts_match_per_scene_oracle(gpu_lib):
    from adaptivemerging_gb300 import native
    sc = _scenes()
    P = params(friction_override=0, iterations=100)
    # the FP32 solve makes states diverge after a step, so the contacts of the
    # first step (identical states) are compared
    g2 = native.BatchSystem(sc, P, threads=128, residual_target=0.0, check_every=0)
    g2.collision_detection(DT)
    parts = _split(g2.contacts(), sc)
    assert sum(len(p["body1"]) for p in parts) > 100
    for k, s in enumerate(sc):
        o = Oracle(s, P)
        o.begin_step()
        o.collide()
        co = o.contacts()
        msg = compare_contacts(parts[k], co, fields=("body1", "body2", "bv1", "bv2", "info", "frame", "jac", "violation"))
        assert msg is None, f"scene {k}: {msg}"


def test_batch_fp32_solve_converges_to_oracle(gpu_lib):
    from adaptivemerging_gb300 import native
    sc = _scenes()
    P = params(friction_override=0, iterations=4000, tolerance=0.0)
    g = native.BatchSystem(sc, P, threads=128, residual_target=0.0, check_every=0)
    ors = [Oracle(s, P) for s in sc]
    g.step(DT)
    for o in ors:
        o.step(DT)
    parts = _split(g.contacts(), sc)
    worst = 0.0
    n = 0
    for k, o in enumerate(ors):
        co = o.contacts()
        if len(co["body1"]) == 0:
            continue
        assert np.array_equal(parts[k]["body1"], co["body1"]) and np.array_equal(parts[k]["info"], co["info"])
        lo, lg = co["lambda"], parts[k]["lambda"]
        scale = max(1.0, float(np.abs(lo).max()))
        worst = max(worst, float(np.abs(lg - lo).max()) / scale)
        n += len(lo)
    assert n > 0
    print(f"batched FP32 vs oracle FP64 converged: {n} contacts, rel err {worst:.2e}")
    assert worst <= 2e-4


def test_batch_residual_target_stops_early(gpu_lib):
    from adaptivemerging_gb300 import native
    sc = _scenes()
    P = params(friction_override=0, iterations=2000)
    g = native.BatchSystem(sc, P, threads=0, residual_target=1e-5, check_every=10)
    for _ in range(20):
        g.step(DT)
    st = g.batch_stats()
    assert st.n_scenes == len(sc) and st.threads in (64, 128, 256, 512)
    assert st.converged == len(sc) and st.sweeps_max < 2000 and st.residual_max <= 1e-5


@pytest.mark.parametrize("accel", [0, 1])
def test_cluster_path_converges_to_oracle(gpu_lib, accel):
    """A bin too large for one CTA's shared memory is solved by a thread-block
    cluster; its converged multipliers match the FP64 oracle like the one-CTA
    path's, and the streaming one-CTA path (clusters off) agrees, with and
    without the conjugate-gradient acceleration."""
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(1400, 77, gap=-0.001), scenes.bin_scene(40, 78, gap=-0.001)]
    P = params(friction_override=0, iterations=20000 if not accel else 6000, tolerance=0.0)
    g = native.BatchSystem(sc, P, threads=256, residual_target=0.0, check_every=0)
    h = native.BatchSystem(sc, P, threads=256, residual_target=0.0, check_every=0)
    g.set_accel(accel)
    h.set_accel(accel)
    h.set_clusters(False)
    g.step(DT)
    h.step(DT)
    st = g.batch_stats()
    assert st.cluster_scenes == 1 and st.cluster_size in (2, 4, 8), (st.cluster_scenes, st.cluster_size)
    assert h.batch_stats().cluster_scenes == 0
    o = Oracle(sc[0], P)
    o.step(DT)
    co = o.contacts()
    part = _split(g.contacts(), sc)[0]
    parth = _split(h.contacts(), sc)[0]
    assert len(co["body1"]) > 1000
    assert np.array_equal(part["body1"], co["body1"]) and np.array_equal(part["info"], co["info"])
    scale = max(1.0, float(np.abs(co["lambda"]).max()))
    err = float(np.abs(part["lambda"] - co["lambda"]).max()) / scale
    errh = float(np.abs(parth["lambda"] - co["lambda"]).max()) / scale
    print(f"cluster of {st.cluster_size}: {len(co['body1'])} contacts, rel err {err:.2e} (one CTA streaming {errh:.2e})")
    assert err <= 2e-4 and errh <= 2e-4
    # same sweeps, same per-group arithmetic: the two kernels agree bit for bit
    assert np.array_equal(part["lambda"], parth["lambda"])


@pytest.mark.parametrize("accel", [0, 1])
def test_results_do_not_depend_on_kernel_shape(gpu_lib, accel):
    """A batch stepped with the residual target gives bit-identical states
    whatever CTA size, staging capacity, size classes and cluster use it runs
    with (the scenes stop at the same check and the per-group arithmetic is
    shared).  With the conjugate-gradient acceleration on, its |g|^2 sum runs
    in one fixed order in every kernel, so the same holds; the last
    configuration repeats the first, so two runs of one shape agree too."""
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(n, 500 + n, gap=0.01) for n in (25, 40, 120, 300, 900, 1500)]
    P = params(friction_override=0, iterations=3000)
    runs = []
    for threads, stage, clusters, classes in ((128, 64, True, True), (256, 256, True, False),
                                              (512, 128, False, True), (256, 256, True, True),
                                              (128, 64, True, True)):
        g = native.BatchSystem(sc, P, threads=threads, residual_target=1e-6, check_every=10)
        g.set_accel(accel)
        g.set_stage(stage)
        g.set_clusters(clusters)
        g.set_size_classes(classes)
        for _ in range(25):
            g.step(DT)
        runs.append((g.bodies()["x"], g.contacts()["lambda"], g.batch_stats().cluster_scenes))
        g.close()
    assert runs[1][2] > 0 and runs[2][2] == 0
    for x, lam, _ in runs[1:]:
        assert np.array_equal(x, runs[0][0]) and np.array_equal(lam, runs[0][1])


def test_batch_edge_cases(gpu_lib):
    """Ragged batches: a scene without contacts (bodies far apart), a scene
    with only pinned bodies and a plane, one-body scenes and ordinary bins
    step together; every scene's stats are sane and the contact-free scenes
    report no sweeps."""
    from adaptivemerging_gb300 import native
    b = scenes.Builder()
    b.plane((0, 0, 0), (0, 1, 0))
    for k in range(5):
        b.sphere(0.2, (10.0 * k, 5.0, 0.0))          # far apart, falling: no contacts yet
    apart = b.build()
    b = scenes.Builder()
    b.plane((0, 0, 0), (0, 1, 0))
    b.box((1, 1, 1), (0, 0.5, 0), pinned=True)
    pinned = b.build()
    b = scenes.Builder()
    b.plane((0, 0, 0), (0, 1, 0))
    b.sphere(0.3, (0, 0.29, 0))                      # resting on the plane
    single = b.build()
    sc = [apart, scenes.bin_scene(50, 5, gap=-0.001), pinned, single, scenes.bin_scene(300, 6, gap=-0.001)]
    g = native.BatchSystem(sc, params(friction_override=0, iterations=2000), threads=0, residual_target=1e-6,
                           check_every=10)
    for _ in range(3):
        g.step(DT)
    ss = g.scene_stats()
    st = g.batch_stats()
    assert st.n_scenes == len(sc)
    assert ss["sweeps"][0] == 0 and ss["sweeps"][2] == 0
    assert ss["sweeps"][3] > 0 and ss["sweeps"][1] > 0 and ss["sweeps"][4] > 0
    assert (ss["residual"] <= 1e-6).all(), ss["residual"]
    x = g.bodies()["x"]
    assert np.isfinite(x).all()
    # per-scene solve times of the last step: every scene ran on a real SM,
    # inside the step, longer solves for the scenes that swept
    tm = g.scene_times()
    assert (tm["start_ns"] >= 0).all() and (tm["end_ns"] >= tm["start_ns"]).all()
    assert tm["start_ns"].min() == 0 and tm["end_ns"].max() < 10**9
    assert ((tm["sm"] >= 0) & (tm["sm"] < 1024)).all()
    assert tm["end_ns"][4] > tm["start_ns"][4]


def test_batch_rejects_oversized_scene(gpu_lib):
    """A scene whose body count exceeds the sweep's shared memory is refused
    with AM_E_CAPACITY on the first step, not run."""
    from adaptivemerging_gb300 import native
    b = scenes.Builder()
    b.plane((0, 0, 0), (0, 1, 0))
    for k in range(9000):
        b.sphere(0.05, ((k % 100) * 0.5, 0.049 + (k // 100) * 0.5, 0.0))
    g = native.BatchSystem([b.build()], params(friction_override=0, iterations=100), threads=0,
                           residual_target=1e-6, check_every=10)
    with pytest.raises(native.AmError) as e:
        g.step(DT)
    assert e.value.code == -2


def _mixed_scenes():
    """Scenes of every body kind the batch takes: sphere-tree clumps resting
    1 mm into a plane, boxes and spheres in a bin, a short tower."""
    b = scenes.Builder()
    b.plane((0, 0, 0), (0, 1, 0))
    rng = np.random.default_rng(11)
    for k in range(6):
        cen = rng.uniform(-0.08, 0.08, (5, 3))
        rad = rng.uniform(0.03, 0.06, 5)
        low = float((cen[:, 1] - rad).min())
        b.clump(cen, rad, (0.5 * k, -low - 0.001, 0.0), density=800.0)
    b.box((0.3, 0.3, 0.3), (0.25, 0.149, 0.5), density=500.0)
    clumps = b.build()
    return [clumps, scenes.bin_scene(45, 77, gap=-0.001), scenes.tower(5, seed=3)]


def test_batch_mixed_bodies_compliance_restitution(gpu_lib):
    """Clumps, boxes and spheres with compliance and restitution on: the first
    step's contacts (two-pass narrow phase, trees present) equal each scene's
    oracle bit for bit, and the FP32 solve converges to the oracle's FP64
    multipliers."""
    from adaptivemerging_gb300 import native
    sc = _mixed_scenes()
    P = params(friction_override=0, iterations=4000, tolerance=0.0, enable_compliance=1, compliance=1e-3,
               restitution=0.3)
    g = native.BatchSystem(sc, P, threads=0, residual_target=0.0, check_every=0)
    g.collision_detection(DT)
    parts = _split(g.contacts(), sc)
    for k, s in enumerate(sc):
        o = Oracle(s, P)
        o.begin_step()
        o.collide()
        msg = compare_contacts(parts[k], o.contacts(),
                               fields=("body1", "body2", "bv1", "bv2", "info", "frame", "jac", "violation"))
        assert msg is None, f"scene {k}: {msg}"
    g2 = native.BatchSystem(sc, P, threads=0, residual_target=0.0, check_every=0)
    g2.step(DT)
    parts = _split(g2.contacts(), sc)
    worst, n = 0.0, 0
    for k, s in enumerate(sc):
        o = Oracle(s, P)
        o.step(DT)
        co = o.contacts()
        assert np.array_equal(parts[k]["body1"], co["body1"]) and np.array_equal(parts[k]["info"], co["info"])
        if len(co["lambda"]):
            scale = max(1.0, float(np.abs(co["lambda"]).max()))
            worst = max(worst, float(np.abs(parts[k]["lambda"] - co["lambda"]).max()) / scale)
            n += len(co["lambda"])
    assert n > 50
    print(f"mixed batch: {n} contacts, rel err {worst:.2e}")
    assert worst <= 2e-4


def test_nncg_fewer_sweeps_same_fixed_point(gpu_lib):
    """The conjugate-gradient acceleration keeps the PGS fixed point: after the
    same plain steps, one step solved to the residual target with and without
    it takes at least 1.5 times fewer sweeps summed over the bins, with
    multipliers within FP32 tolerance of each other; run to its fixed point
    (a fixed 20000 sweeps) it gives the FP64 oracle's multipliers from the
    same state within 2e-4."""
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(n, 600 + n, gap=0.01) for n in (60, 150, 300, 700, 1200)]
    P = params(friction_override=0, iterations=30000)
    a = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    b = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    for _ in range(30):
        a.step(DT)
        b.step(DT)
    assert np.array_equal(a.bodies()["x"], b.bodies()["x"])
    bod = a.bodies()
    b.set_accel(1)
    a.step(DT)
    b.step(DT)
    sa, sb = a.scene_stats(), b.scene_stats()
    assert (sa["residual"] <= 1e-6).all() and (sb["residual"] <= 1e-6).all(), (sa["residual"], sb["residual"])
    ratio = sa["sweeps"].sum() / max(1, sb["sweeps"].sum())
    print("sweeps plain", sa["sweeps"], "nncg", sb["sweeps"], f"ratio {ratio:.2f}")
    assert ratio >= 1.5
    la, lb = a.contacts()["lambda"], b.contacts()["lambda"]
    scale = max(1.0, float(np.abs(la).max()))
    assert float(np.abs(la - lb).max()) / scale <= 2e-4
    # the largest bin against the oracle from the same state (no warm start there)
    k = len(sc) - 1
    lo, hi = a.offsets[k], a.offsets[k + 1]
    arr = {q: np.array(v, copy=True) for q, v in sc[k].a.items()}
    body = arr["type"] != abi.AM_PLANE
    for key, m in (("x", 3), ("R", 9), ("v", 3), ("omega", 3)):
        t = arr[key].reshape(-1, m)
        t[body] = bod[key][lo:hi][body]
        arr[key] = t.reshape(-1)
    o = Oracle(abi.SceneArrays(**arr), params(friction_override=0, iterations=400000, tolerance=0.0))
    o.set_residual_target(1e-10, 10)
    o.step(DT)
    co = o.contacts()
    c = native.BatchSystem([abi.SceneArrays(**arr)], params(friction_override=0, iterations=20000), threads=0,
                           residual_target=0.0, check_every=0)
    c.set_accel(1)
    c.step(DT)
    part = _split(c.contacts(), [sc[k]])[0]
    assert np.array_equal(part["body1"], co["body1"]) and np.array_equal(part["info"], co["info"])
    err = float(np.abs(part["lambda"] - co["lambda"]).max()) / max(1.0, float(np.abs(co["lambda"]).max()))
    print(f"nncg vs oracle: {len(co['body1'])} contacts, rel err {err:.2e}")
    assert err <= 2e-4
