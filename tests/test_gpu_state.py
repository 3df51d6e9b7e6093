"""am_get_state / am_put_state: a snapshot taken between steps and restored
into a fresh context loaded with the same scene resumes bit-identically (the
stand-in for RigidBodySystem.reset's rebuild of the reference's Java
objects), with merging on (collections, body-pair histories, contacts inside
collections) and for a batch.  Refusals: a blob of another scene, a cut
blob, a buffer too small."""
import numpy as np
import pytest

from adaptivemerging_gb300 import scenes
from helpers import compare_bodies, compare_contacts, params

pytestmark = pytest.mark.gpu


def _trace(g, steps, dt):
    out = []
    for _ in range(steps):
        g.step(dt)
        p = g.perf()
        out.append((g.topology(), g.contacts(), g.bodies(), (p.merge_events, p.unmerge_events)))
    return out


def _same(a, b):
    for s, (x, y) in enumerate(zip(a, b)):
        assert x[0] == y[0], f"step {s}: topology"
        assert len(x[1]["body1"]) == len(y[1]["body1"]), f"step {s}: contacts"
        msg = compare_contacts(x[1], y[1], fields=("body1", "body2", "bv1", "bv2", "info", "frame", "jac",
                                                   "violation", "lambda", "bD", "state", "fresh"))
        assert msg is None, f"step {s}: {msg}"
        msg = compare_bodies(x[2], y[2], fields=("x", "R", "v", "omega", "sleeping", "parent"))
        assert msg is None, f"step {s}: {msg}"
        assert x[3] == y[3], f"step {s}: merge / unmerge events"


@pytest.mark.parametrize("name,make,dt,warm,over", [
    ("wall_small", lambda: scenes.wall(cols=8, rows=6, seed=13), 0.005, 97, dict(friction=0.5, iterations=80)),
    ("tower12", lambda: scenes.tower(12, seed=4, density=1.0), 0.01, 54, dict(friction=0.6, iterations=60)),
])
def test_snapshot_resumes_bit_identically_with_merging(gpu_lib, name, make, dt, warm, over):
    from adaptivemerging_gb300 import native
    sc = make()
    P = params(enable_merging=1, **over)
    g = native.System(sc, P)
    g.step(dt, warm)
    blob = g.get_state()
    assert any(isinstance(t, tuple) for t in g.topology()), "no collection at the snapshot"
    after = _trace(g, 40, dt)
    h = native.System(sc, P)
    h.step(dt, 3)                                  # a different state, overwritten by the snapshot
    h.put_state(blob)
    _same(after, _trace(h, 40, dt))
    assert after[-1][3][0] > 0


def test_snapshot_resumes_batch(gpu_lib):
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(n, 40 + n, gap=-0.001) for n in (30, 90, 250)]
    P = params(friction_override=0, iterations=3000)
    g = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    for _ in range(12):
        g.step(0.005)
    blob = g.get_state()
    a = [(g.step(0.005), g.bodies()["x"].copy(), g.contacts()["lambda"].copy())[1:] for _ in range(8)]
    h = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    h.put_state(blob)
    b = [(h.step(0.005), h.bodies()["x"].copy(), h.contacts()["lambda"].copy())[1:] for _ in range(8)]
    for s, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1]), f"step {s}"


def test_snapshot_refusals(gpu_lib):
    import ctypes as C
    from adaptivemerging_gb300 import native
    P = params(enable_merging=1, friction=0.6, iterations=40)
    g = native.System(scenes.tower(6, seed=1), P)
    g.step(0.01, 5)
    blob = g.get_state()
    n = C.c_int64(0)
    buf = C.create_string_buffer(16)
    assert native.lib().am_get_state(g.h, buf, 16, C.byref(n)) == -2 and n.value == len(blob)
    other = native.System(scenes.tower(7, seed=1), P)
    with pytest.raises(native.AmError) as e:
        other.put_state(blob)
    assert e.value.code == -6                      # AM_E_STATE: another scene
    same = native.System(scenes.tower(6, seed=1), P)
    with pytest.raises(native.AmError) as e:
        same.put_state(blob[:len(blob) // 2])
    assert e.value.code == -1                      # AM_E_ARG: cut blob
    with pytest.raises(native.AmError) as e:
        same.put_state(b"XXXX" + blob[4:])
    assert e.value.code == -1                      # AM_E_ARG: not a snapshot
    same.put_state(blob)                           # the whole blob still restores
    g.step(0.01)
    same.step(0.01)
    assert np.array_equal(g.bodies()["x"], same.bodies()["x"])


def test_put_bodies_with_collections_round_trip(gpu_lib):
    """am_put_bodies while collections exist: writing back the state just read
    changes nothing (the members keep the state their collection gives them),
    and a changed free body's velocity is applied."""
    from adaptivemerging_gb300 import abi, native
    sc = scenes.wall(cols=8, rows=6, seed=13)
    P = params(enable_merging=1, friction=0.5, iterations=80)
    g = native.System(sc, P)
    h = native.System(sc, P)
    g.step(0.005, 97)
    h.step(0.005, 97)
    assert any(isinstance(t, tuple) for t in h.topology()), "no collection"
    st = abi.BodyState(h.n)
    h.get_bodies_struct(st.struct())
    h.put_bodies_struct(st.struct())
    for _ in range(20):
        g.step(0.005)
        h.step(0.005)
    assert np.array_equal(g.bodies()["x"], h.bodies()["x"])
    assert np.array_equal(g.bodies()["v"], h.bodies()["v"])
    free = [t for t in h.topology() if not isinstance(t, tuple) and sc.a["pinned"][t] == 0]
    assert free
    st = abi.BodyState(h.n)
    h.get_bodies_struct(st.struct())
    st.v.reshape(-1, 3)[free[0], 0] += 1.0
    h.put_bodies_struct(st.struct())
    assert h.bodies()["v"][free[0], 0] == g.bodies()["v"][free[0], 0] + 1.0
