"""The benchmark's own configurations, device path against the oracle.

- Config 1: the 25-box tower (1.0 x 0.5 x 1.0 m, density 1000, seed 1),
  mu 0.6, dt 0.01, 100 PGS iterations, merging on, 500 steps, reference order:
  bit-exact every 10 steps (topology, contacts with multipliers, bodies,
  merge / unmerge counts).
- Config 2: the 40 x 25 brick wall with the 50 kg projectile, mu 0.5,
  dt 0.005, 200 iterations, merging on, reference order: bit-exact every 10
  steps for 300 steps.
- Config 3: the 512-bin batch the benchmark times.  Contact sets of every bin
  equal the per-scene oracle's at the bin's first contact step (all earlier
  steps are free flight, so both sides hold the same state).  Later, with
  piles formed and the largest bins solved by thread-block clusters, the
  device state is handed to the oracle: the contact sets of the bins solved
  by clusters of 2, 4 and 8 CTAs (and the largest bins) are bit-exact, and
  the FP32 fixed point gives the FP64 one's body velocities.
"""
import concurrent.futures as cf

import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scenes
from helpers import compare_bodies, compare_contacts, params
from oracle_binding import Oracle

pytestmark = pytest.mark.gpu

GEOMETRY = ("body1", "body2", "bv1", "bv2", "info", "frame", "jac")


def _run_lockstep(sc, P, dt, steps, every=10):
    from adaptivemerging_gb300 import native
    g = native.System(sc, P)
    o = Oracle(sc, P)
    merged = 0
    for s in range(steps):
        g.step(dt)
        o.step(dt)
        if s % every == every - 1 or s == steps - 1:
            tg, to = g.topology(), o.topology()
            assert tg == to, f"step {s}: topology differs"
            cg, co = g.contacts(), o.contacts()
            assert len(cg["body1"]) == len(co["body1"]), f"step {s}: {len(cg['body1'])} vs {len(co['body1'])}"
            msg = compare_contacts(cg, co)
            assert msg is None, f"step {s}: {msg}"
            msg = compare_bodies(g.bodies(), o.bodies())
            assert msg is None, f"step {s}: {msg}"
            c = o.counters()
            pg = g.perf()
            assert (pg.merge_events, pg.unmerge_events) == (c["merges"], c["unmerges"]), f"step {s}"
            merged = max(merged, sum(1 for t in to if isinstance(t, tuple)))
    return o.counters(), merged


def test_config1_tower25_merging_500_steps(gpu_lib):
    sc = scenes.tower(25, seed=1)            # density 1000 kg/m3
    P = params(enable_merging=1, friction=0.6, iterations=100)
    c, merged = _run_lockstep(sc, P, 0.01, 500)
    print(f"config 1: {c['merges']} merges, {c['unmerges']} unmerges")
    assert c["merges"] > 0 and c["unmerges"] > 0 and merged > 0


def test_config2_wall_projectile_merging_300_steps(gpu_lib):
    sc = scenes.wall(cols=40, rows=25, seed=2)
    P = params(enable_merging=1, friction=0.5, iterations=200)
    c, merged = _run_lockstep(sc, P, 0.005, 300)
    print(f"config 2: {c['merges']} merges, {c['unmerges']} unmerges")
    assert c["merges"] > 1000 and c["unmerges"] > 100 and merged > 0


# ---------------------------------------------------------------------------
# config 3: the benchmark batch
BATCH_DT = 0.005


def _batch_params(**over):
    base = dict(gravity_amount=9.81, friction_override=0, restitution_override=1, restitution=0.0,
                iterations=5000, enable_merging=0)
    base.update(over)
    return abi.default_params(**base)


def _local(part, off, node_off):
    out = dict(part)
    out["body1"] = part["body1"] - off
    out["body2"] = part["body2"] - off
    for k in ("bv1", "bv2"):
        v = part[k].copy()
        v[v >= 0] -= node_off
        pl = v <= -2
        v[pl] = -2 - ((-2 - v[pl]) - off)
        out[k] = v
    return out


def _split(cg, sc_list):
    offs = np.cumsum([0] + [s.n for s in sc_list])
    node_offs = np.cumsum([0] + [s.n_nodes for s in sc_list])
    order = np.argsort(cg["body1"], kind="stable")
    b1 = cg["body1"][order]
    out = []
    for k in range(len(sc_list)):
        lo, hi = np.searchsorted(b1, [offs[k], offs[k + 1]])
        sel = order[lo:hi]
        sel.sort()
        out.append(_local({f: v[sel] for f, v in cg.items()}, offs[k], node_offs[k]))
    return out


def test_config3_first_contact_sets_all_bins(gpu_lib):
    """Every one of the 512 bins: its contact set at its first contact step
    equals the oracle's, bit for bit (keys, frames, Jacobians, violation)."""
    from adaptivemerging_gb300 import native
    sc = scenes.batch_scenes(512, seed=3)
    P = _batch_params()
    g = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    ors = [Oracle(s, P) for s in sc]
    todo = set(range(len(sc)))
    checked = 0
    for step in range(40):
        g.step(BATCH_DT)
        parts = None
        for k in sorted(todo):
            o = ors[k]
            o.step(BATCH_DT)
            if o.num_contacts() == 0:
                continue
            if parts is None:
                parts = _split(g.contacts(), sc)
            co = o.contacts()
            assert len(parts[k]["body1"]) == len(co["body1"]), f"bin {k} step {step}"
            msg = compare_contacts(parts[k], co, fields=GEOMETRY + ("violation",))
            assert msg is None, f"bin {k} step {step}: {msg}"
            todo.discard(k)
            ors[k] = None
            checked += 1
        if not todo:
            break
    assert not todo, f"{len(todo)} bins never touched"
    assert checked == 512


def _inject(scene, x, R, v, w):
    """The scene with the device's body state (planes keep their point)."""
    a = {k: np.array(val, copy=True) for k, val in scene.a.items()}
    body = a["type"] != abi.AM_PLANE
    for key, src, m in (("x", x, 3), ("R", R, 9), ("v", v, 3), ("omega", w, 3)):
        arr = a[key].reshape(-1, m)
        arr[body] = src[body]
        a[key] = arr.reshape(-1)
    return abi.SceneArrays(**a)


def _oracle_converged(scene, P):
    o = Oracle(scene, P)
    o.set_residual_target(1e-10, 10)
    o.step(BATCH_DT)
    return o.contacts(), o.counters()["sweeps"], o.bodies()["v"]


def test_config3_cluster_bins_against_oracle(gpu_lib):
    """With piles formed (step 50) the batch solves its large bins with
    clusters of 2 and 4 CTAs.  The device state of the largest bins and of
    bins on each cluster size is handed to the oracle: their contact sets are
    the oracle's bit for bit.  The same states, loaded into fresh batches whose
    CTAs hold at most 2048, 640 and 320 records (clusters of 2, 4 and 8 CTAs),
    are solved from the same cold start as the oracle to a fixed point (60000
    FP32 sweeps; residual 1e-10 in FP64): multipliers within 2e-4 relative,
    body velocities within 1e-4.  (Box friction makes the problem non-monotone,
    so a frictional pile can hold several solutions: from its own warm start
    the batch settles on another one, converged as tightly; cold start against
    cold start is the comparison that pins the solver.)"""
    from adaptivemerging_gb300 import native
    sc = scenes.batch_scenes(512, seed=3)
    P = _batch_params(enable_sleeping=0)
    g = native.BatchSystem(sc, P, threads=0, residual_target=1e-6, check_every=10)
    for _ in range(50):
        g.step(BATCH_DT)
    b = g.bodies()
    offs = g.offsets
    g.step(BATCH_DT)
    ctas = g.scene_ctas()
    ks = {int(k): int((ctas == k).sum()) for k in np.unique(ctas)}
    print("CTAs per scene at step 51:", ks)
    assert ks.get(2, 0) > 0 and ks.get(4, 0) > 0, ks
    parts = _split(g.contacts(), sc)
    nc = np.array([len(p["body1"]) for p in parts])
    pick = set(np.argsort(-nc)[:8].tolist())
    for k in (4, 2):
        pick.update(np.nonzero(ctas == k)[0][:3].tolist())
    pick = sorted(pick)
    inj = {}
    for k in pick:
        lo, hi = offs[k], offs[k + 1]
        inj[k] = _inject(sc[k], b["x"][lo:hi], b["R"][lo:hi], b["v"][lo:hi], b["omega"][lo:hi])
    Po = _batch_params(enable_sleeping=0, iterations=400000, tolerance=0.0)
    with cf.ThreadPoolExecutor(max_workers=16) as ex:
        jobs = {k: ex.submit(_oracle_converged, inj[k], Po) for k in pick}
    res = {k: jobs[k].result() for k in pick}
    for k in pick:   # the batch's own contact sets at step 51
        co = res[k][0]
        assert len(parts[k]["body1"]) == len(co["body1"]) > 0, f"bin {k}"
        msg = compare_contacts(parts[k], co, fields=GEOMETRY)
        assert msg is None, f"bin {k} ({ctas[k]} CTAs): {msg}"
    big = [k for k in pick if ctas[k] > 1]
    seen = set()
    errs, verrs = [], []
    Pfix = _batch_params(enable_sleeping=0, iterations=60000)
    for stage in (0, 640, 320):
        h = native.BatchSystem([inj[k] for k in big], Pfix, threads=0, residual_target=0.0, check_every=0,
                               cluster_stage=stage)
        h.step(BATCH_DT)
        hct = h.scene_ctas()
        seen.update(int(x) for x in hct)
        hparts = _split(h.contacts(), [inj[k] for k in big])
        hb = h.bodies()["v"]
        hoffs = np.cumsum([0] + [inj[k].n for k in big])
        for i, k in enumerate(big):
            co, sweeps, vo = res[k]
            assert sweeps < 400000, f"bin {k}: oracle did not converge"
            pk = hparts[i]
            msg = compare_contacts(pk, co, fields=GEOMETRY)
            assert msg is None, f"bin {k} ({hct[i]} CTAs): {msg}"
            assert np.array_equal(pk["violation"][:, 0], co["violation"][:, 0]), f"bin {k}"
            err = float(np.abs(pk["lambda"] - co["lambda"]).max()) / max(1.0, float(np.abs(co["lambda"]).max()))
            verr = float(np.abs(hb[hoffs[i]:hoffs[i + 1]] - vo).max()) / max(1.0, float(np.abs(vo).max()))
            print(f"bin {k}: {sc[k].n} bodies, {len(co['body1'])} contacts, {hct[i]} CTAs, oracle sweeps {sweeps}, "
                  f"lambda rel err {err:.2e}, velocity rel err {verr:.2e}")
            errs.append(err)
            verrs.append(verr)
            assert err <= 2e-4 and verr <= 1e-4, f"bin {k} ({hct[i]} CTAs): {err} {verr}"
        h.close()
    print(f"cluster sizes {sorted(seen)}; worst lambda {max(errs):.2e}, worst velocity {max(verrs):.2e}")
    assert {2, 4, 8} <= seen, seen
