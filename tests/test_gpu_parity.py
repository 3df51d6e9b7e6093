"""Device path vs the oracle, bit for bit, in reference order.

Scenes are seeded; both sides start from the same am_scene and the same
parameters.  In AM_ORDER_REFERENCE mode every kernel evaluates the reference's
arithmetic in the reference's order (no fused multiply-add), so contact lists
(pair indices, counts, info ids), contact frames, Jacobians, multipliers and
body states must be identical to the last bit after every step.
"""
import numpy as np
import pytest

from adaptivemerging_gb300 import abi, scenes
from helpers import DT, compare_bodies, compare_contacts, params
from oracle_binding import Oracle

pytestmark = pytest.mark.gpu

SCENES = {
    "tower6": lambda: scenes.tower(6, seed=1),
    "tower25": lambda: scenes.tower(25, seed=3),
    "pile_box_sphere": lambda: scenes.random_pile(24, seed=5, kinds=("box", "sphere")),
    "pile_clumps": lambda: scenes.random_pile(16, seed=7, kinds=("box", "sphere", "clump")),
    "wall_small": lambda: scenes.wall(cols=8, rows=5, seed=11),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_contacts_first_step(gpu_lib, name):
    from adaptivemerging_gb300 import native
    sc = SCENES[name]()
    P = params()
    g = native.System(sc, P)
    o = Oracle(sc, P)
    g.collision_detection(DT)
    o.begin_step()
    o.collide()
    cg, co = g.contacts(), o.contacts()
    assert len(cg["body1"]) == len(co["body1"])
    msg = compare_contacts(cg, co, fields=("body1", "body2", "bv1", "bv2", "info", "frame", "jac", "violation"))
    assert msg is None, msg


@pytest.mark.parametrize("name", list(SCENES))
def test_trajectory_bit_exact(gpu_lib, name):
    from adaptivemerging_gb300 import native
    sc = SCENES[name]()
    P = params()
    g = native.System(sc, P)
    o = Oracle(sc, P)
    steps = 60 if name != "tower25" else 40
    total = 0
    for s in range(steps):
        g.step(DT)
        o.step(DT)
        cg, co = g.contacts(), o.contacts()
        total += len(co["body1"])
        assert len(cg["body1"]) == len(co["body1"]), f"step {s}: {len(cg['body1'])} vs {len(co['body1'])}"
        msg = compare_contacts(cg, co)
        assert msg is None, f"step {s}: {msg}"
        msg = compare_bodies(g.bodies(), o.bodies())
        assert msg is None, f"step {s}: {msg}"
    assert total > 0


def test_phase_by_phase(gpu_lib):
    """collide / warm start / solve compared after each phase of one step (tower25, step 3)."""
    from adaptivemerging_gb300 import native
    sc = scenes.tower(25, seed=3)
    P = params(iterations=30)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    g.step(DT, 2)
    o.step(DT, 2)
    g.collision_detection(DT)
    o.begin_step()
    o.collide()
    assert compare_contacts(g.contacts(), o.contacts(), fields=("body1", "info", "frame", "jac")) is None
    g.warm_start()
    o.warm_start()
    msg = compare_contacts(g.contacts(), o.contacts(), fields=("lambda", "violation", "fresh"))
    assert msg is None, f"warm start: {msg}"
    st = g.solve_lcp(DT)
    o.solve(DT)
    msg = compare_contacts(g.contacts(), o.contacts(), fields=("lambda", "state"))
    assert msg is None, f"solve: {msg}"
    assert st.sweeps == o.counters()["sweeps"]


# (solver order, form of the mixed kernel: -1 chosen per step, 0 grid, 1 one
# block, 2 one block with the contact records in shared memory)
ORDERS = pytest.mark.parametrize("order,form", [(abi.AM_ORDER_COLOURED, -1), (abi.AM_ORDER_MIXED, -1),
                                                (abi.AM_ORDER_MIXED, 0), (abi.AM_ORDER_MIXED, 1),
                                                (abi.AM_ORDER_MIXED, 2)],
                                 ids=["fp64", "mixed", "mixed-grid", "mixed-block", "mixed-shared"])


@ORDERS
@pytest.mark.parametrize("name", ["tower6", "pile_box_sphere", "wall_small"])
def test_coloured_converged(gpu_lib, name, order, form):
    """AM_ORDER_COLOURED reorders Gauss-Seidel, so multipliers match only at
    convergence: from an identical state (reference-order steps first), both
    sides iterate to a fixed point and must agree within 1e-6 relative
    (compliance 1e-3 makes the regularised LCP's solution unique).
    AM_ORDER_MIXED (FP32 sweeps on the correction, FP64 refinement) must
    reach the same fixed point to the same bound."""
    from adaptivemerging_gb300 import native
    sc = SCENES[name]()
    P = params(iterations=100)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    warm = {"tower6": 15, "pile_box_sphere": 90, "wall_small": 15}[name]
    g.step(DT, warm)
    o.step(DT, warm)
    assert compare_bodies(g.bodies(), o.bodies()) is None
    iters = {"tower6": 6000, "pile_box_sphere": 6000, "wall_small": 60000}[name]
    g.set_params(params(iterations=iters, tolerance=1e-13, solver_order=order))
    g.set_mixed_form(form)
    o.set_params(params(iterations=iters, tolerance=1e-13))
    g.step(DT)
    o.step(DT)
    if order == abi.AM_ORDER_MIXED and form >= 0:
        assert g.mixed_form() == form
    lg, lo = g.contacts()["lambda"], o.contacts()["lambda"]
    assert lg.shape == lo.shape and lo.size > 0
    scale = max(1.0, float(np.abs(lo).max()))
    err = float(np.abs(lg - lo).max()) / scale
    st = g.stats()
    print(f"{name}: contacts {lo.shape[0]} rel err {err:.2e} sweeps {st.sweeps} residual_rel {st.residual_rel:.2e}")
    assert err <= 1e-6, err
    assert st.residual_rel <= 1e-6


@ORDERS
def test_coloured_residual_target_stops_at_target(gpu_lib, order, form):
    """am_set_residual_target: the coloured FP64 solve stops as soon as the
    relative natural-map residual is <= the target (the reference's
    max-change tolerance switched off), well before the sweep cap, and the
    multipliers agree with the oracle run to a fixed point."""
    from adaptivemerging_gb300 import native
    sc = SCENES["pile_box_sphere"]()
    P = params(iterations=100)
    g = native.System(sc, P)
    o = Oracle(sc, P)
    g.step(DT, 90)
    o.step(DT, 90)
    g.set_params(params(iterations=60000, tolerance=0.0, solver_order=order))
    g.set_mixed_form(form)
    g.set_residual_target(1e-7, 10)
    o.set_params(params(iterations=60000, tolerance=1e-13))
    g.step(DT)
    o.step(DT)
    st = g.stats()
    lg, lo = g.contacts()["lambda"], o.contacts()["lambda"]
    assert lg.shape == lo.shape and lo.size > 0
    err = float(np.abs(lg - lo).max()) / max(1.0, float(np.abs(lo).max()))
    print(f"residual target 1e-7: sweeps {st.sweeps} residual_rel {st.residual_rel:.2e} rel err {err:.2e}")
    assert st.residual_rel <= 1e-7 and st.sweeps % 10 == 0 and st.sweeps < 60000
    assert err <= 1e-5


def test_nonfinite_velocity_is_reported(gpu_lib):
    """A NaN body velocity in the input is reported as AM_E_NONFINITE by the
    step that integrates it (the arithmetic itself is not altered)."""
    from adaptivemerging_gb300 import native
    sc = scenes.tower(3, seed=2)
    sc.a["v"][3] = np.nan            # body 1 (the lowest box), x velocity
    g = native.System(sc, params(iterations=20))
    with pytest.raises(native.AmError) as e:
        g.step(DT)
    assert e.value.code == -3


def test_context_reused_for_new_scenes(gpu_lib):
    """One context given a second scene (and then a batch) steps it exactly
    as a fresh context does: every device buffer of the first scene is
    released and allocated anew."""
    import ctypes as C
    from adaptivemerging_gb300 import native
    P = params(friction=0.6, iterations=40)
    first = scenes.tower(6, seed=1)
    second = scenes.random_pile(14, seed=3, kinds=("box", "sphere"))
    g = native.System(first, P)
    for _ in range(20):
        g.step(0.01)
    s2 = second.struct()
    g._check(native.lib().am_set_scene(g.h, C.byref(s2)))
    g._s, g.n, g.scene = s2, second.n, second
    fresh = native.System(second, P)
    for _ in range(30):
        g.step(0.01)
        fresh.step(0.01)
    assert np.array_equal(g.bodies()["x"], fresh.bodies()["x"])
    assert np.array_equal(g.contacts()["lambda"], fresh.contacts()["lambda"])
    # the same context loaded with a batch afterwards
    bins = [scenes.bin_scene(n, 70 + n, gap=-0.001) for n in (25, 60)]
    arr = (native.abi.am_scene * len(bins))(*[b.struct() for b in bins])
    g._check(native.lib().am_set_batch(g.h, arr, len(bins)))
    g._check(native.lib().am_set_batch_options(g.h, 0, 1e-6, 10))
    g.n = sum(b.n for b in bins)
    ref = native.BatchSystem(bins, P, threads=0, residual_target=1e-6, check_every=10)
    for _ in range(5):
        g.step(0.005)
        ref.step(0.005)
    assert np.array_equal(g.bodies()["x"], ref.bodies()["x"])
