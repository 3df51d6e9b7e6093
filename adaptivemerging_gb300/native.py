"""ctypes binding of libam.so and a host-side mirror of the reference's
system / collision-processor call surface.

`System` follows RigidBodySystem (step = advanceTime) and exposes the
CollisionProcessor phases (collisionDetection, warmStart, solveLCP) with the
reference's names.  Errors from the C ABI raise `AmError` with the context's
last error string; there is no CPU fallback: if libam.so cannot be loaded the
import fails loudly.
"""
import ctypes as C
import os

import numpy as np

from . import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libam.so")

EXPORTS = [
    "am_params_default", "am_create", "am_destroy", "am_last_error", "am_set_params", "am_set_scene",
    "am_step", "am_collide", "am_warm_start", "am_solve", "am_integrate", "am_get_bodies",
    "am_num_contacts", "am_get_contacts", "am_get_stats", "am_get_perf", "am_reset_perf", "am_get_stream", "am_get_step_phases", "am_get_state", "am_put_state", "am_merge_tests", "am_step_phase", "am_single_sweep_order", "am_single_sweep", "am_check_barrier_timeout", "am_put_bodies", "am_get_topology", "am_set_batch", "am_set_batch_options", "am_get_batch_stats", "am_get_batch_scene_stats", "am_get_batch_scene_times", "am_get_batch_scene_ctas", "am_get_batch_scene_chain", "am_set_residual_target", "am_set_mixed_form", "am_get_mixed_form", "am_set_kinematic",
    "am_set_batch_local_sweeps", "am_set_batch_accel", "am_set_batch_critical", "am_set_batch_clusters", "am_set_batch_stage", "am_set_batch_relaxation",
    "am_set_batch_cluster_stage", "am_set_batch_size_classes", "am_set_phase_timing", "am_get_phase_times",
    "am_learned_collect", "am_learned_train", "am_learned_use", "am_learned_scope", "am_learned_weights", "am_learned_info",
    "am_learned_grad", "am_learned_infer", "am_learned_infer_noalloc",
]

_lib = None


class AmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"am status {code}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m adaptivemerging_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.am_params_default.argtypes = [C.POINTER(abi.am_params)]
        L.am_params_default.restype = None
        L.am_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(vp)]
        L.am_destroy.argtypes = [vp]
        L.am_last_error.argtypes = [vp]
        L.am_last_error.restype = C.c_char_p
        L.am_set_params.argtypes = [vp, C.POINTER(abi.am_params)]
        L.am_set_scene.argtypes = [vp, C.POINTER(abi.am_scene)]
        L.am_step.argtypes = [vp, C.c_double]
        L.am_collide.argtypes = [vp, C.c_double]
        L.am_warm_start.argtypes = [vp]
        L.am_solve.argtypes = [vp, C.c_double, C.POINTER(abi.am_solve_stats)]
        L.am_integrate.argtypes = [vp, C.c_double]
        L.am_get_bodies.argtypes = [vp, C.POINTER(abi.am_body_state)]
        L.am_num_contacts.argtypes = [vp, C.POINTER(C.c_int32)]
        L.am_get_contacts.argtypes = [vp, C.POINTER(abi.am_contacts), C.c_int32, C.POINTER(C.c_int32)]
        L.am_get_stats.argtypes = [vp, C.POINTER(abi.am_solve_stats)]
        L.am_get_perf.argtypes = [vp, C.POINTER(abi.am_perf)]
        L.am_put_bodies.argtypes = [vp, C.POINTER(abi.am_body_state)]
        L.am_set_batch.argtypes = [vp, C.POINTER(abi.am_scene), C.c_int32]
        L.am_set_batch_options.argtypes = [vp, C.c_int32, C.c_double, C.c_int32]
        L.am_get_batch_stats.argtypes = [vp, C.POINTER(abi.am_batch_stats)]
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int32)
        L.am_get_batch_scene_stats.argtypes = [vp, ip, fp, ip, ip]
        L.am_get_batch_scene_times.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), ip]
        L.am_get_batch_scene_ctas.argtypes = [vp, ip]
        L.am_get_batch_scene_chain.argtypes = [vp, ip]
        L.am_set_residual_target.argtypes = [vp, C.c_double, C.c_int32]
        L.am_set_mixed_form.argtypes = [vp, C.c_int32, C.c_int32]
        L.am_get_mixed_form.argtypes = [vp, C.POINTER(C.c_int32)]
        L.am_set_kinematic.argtypes = [vp, C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double]
        L.am_set_batch_local_sweeps.argtypes = [vp, C.c_int32]
        L.am_set_batch_accel.argtypes = [vp, C.c_int32]
        L.am_set_batch_critical.argtypes = [vp, C.c_double, C.c_int32]
        L.am_set_batch_clusters.argtypes = [vp, C.c_int32]
        L.am_set_batch_size_classes.argtypes = [vp, C.c_int32]
        L.am_set_batch_stage.argtypes = [vp, C.c_int32]
        L.am_set_batch_cluster_stage.argtypes = [vp, C.c_int32]
        L.am_set_batch_relaxation.argtypes = [vp, C.c_double, C.c_int32]
        L.am_learned_collect.argtypes = [vp, C.c_int32, C.c_int32]
        L.am_learned_train.argtypes = [vp, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_double)]
        L.am_learned_use.argtypes = [vp, C.c_int32]
        L.am_learned_scope.argtypes = [vp, C.c_int32]
        L.am_learned_weights.argtypes = [vp, fp, fp, fp, fp]
        L.am_learned_info.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.am_learned_grad.argtypes = [vp, fp, fp, C.c_int32, fp, fp]
        L.am_learned_infer.argtypes = [vp, fp, C.c_int32, fp, C.c_int32]
        L.am_learned_infer_noalloc.argtypes = [vp, fp, C.c_int32, fp, C.c_int32]
        L.am_get_topology.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.am_reset_perf.argtypes = [vp]
        L.am_set_phase_timing.argtypes = [vp, C.c_int32]
        L.am_get_phase_times.argtypes = [vp, C.POINTER(C.c_double)]
        L.am_get_stream.argtypes = [vp, C.POINTER(vp)]
        L.am_get_step_phases.argtypes = [vp, C.POINTER(C.c_double)]
        L.am_get_state.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64)]
        L.am_put_state.argtypes = [vp, vp, C.c_int64]
        L.am_merge_tests.argtypes = [vp, C.POINTER(abi.am_bpc_tests), C.c_int32, C.POINTER(C.c_int32)]
        L.am_step_phase.argtypes = [vp, C.c_int32, C.c_double]
        L.am_single_sweep_order.argtypes = [vp, ip, C.c_int32, ip]
        L.am_single_sweep.argtypes = [vp, ip, C.c_int32, C.c_double]
        L.am_check_barrier_timeout.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
        for f in EXPORTS:
            if f not in ("am_params_default", "am_last_error"):
                getattr(L, f).restype = C.c_int32
        _lib = L
    return _lib


class BatchSystem:
    """Many independent scenes in one context (merging off); am_step advances all."""

    def __init__(self, scene_list, params, threads=0, residual_target=1e-6, check_every=10, cluster_stage=0):
        self.params = params
        self.scenes = scene_list
        self.h = C.c_void_p()
        self._check(lib().am_create(C.byref(params), C.byref(self.h)))
        if cluster_stage:
            self._check(lib().am_set_batch_cluster_stage(self.h, cluster_stage))
        arr = (abi.am_scene * len(scene_list))()
        for k, s in enumerate(scene_list):
            arr[k] = s.struct()
        self._arr = arr
        self._check(lib().am_set_batch(self.h, arr, len(scene_list)))
        self._check(lib().am_set_batch_options(self.h, threads, residual_target, check_every))
        self.n = sum(s.n for s in scene_list)
        self.offsets = np.cumsum([0] + [s.n for s in scene_list])

    _check = None  # filled below

    def batch_stats(self):
        st = abi.am_batch_stats()
        self._check(lib().am_get_batch_stats(self.h, C.byref(st)))
        return st

    def set_relaxation(self, relax=1.0, symmetric=False):
        self._check(lib().am_set_batch_relaxation(self.h, relax, int(symmetric)))

    def set_stage(self, slots):
        self._check(lib().am_set_batch_stage(self.h, slots))

    def set_clusters(self, enable=True):
        self._check(lib().am_set_batch_clusters(self.h, int(enable)))

    def set_size_classes(self, enable=True):
        self._check(lib().am_set_batch_size_classes(self.h, int(enable)))

    def set_accel(self, mode=1):
        """1: conjugate-gradient (NNCG) acceleration of the batched sweep; 0: plain PGS."""
        self._check(lib().am_set_batch_accel(self.h, int(mode)))

    def set_critical(self, frac=0.75, cap=640):
        """Scenes within `frac` of the costliest solve get clusters of at most `cap` records per CTA."""
        self._check(lib().am_set_batch_critical(self.h, frac, cap))

    def set_local_sweeps(self, passes):
        self._check(lib().am_set_batch_local_sweeps(self.h, passes))

    def scene_stats(self):
        n = len(self.scenes)
        sw = np.zeros(n, np.int32)
        rs = np.zeros(n, np.float32)
        fb = np.zeros(n, np.int32)
        nc = np.zeros(n, np.int32)
        ip = C.POINTER(C.c_int32)
        self._check(lib().am_get_batch_scene_stats(self.h, sw.ctypes.data_as(ip), rs.ctypes.data_as(C.POINTER(C.c_float)),
                                                   fb.ctypes.data_as(ip), nc.ctypes.data_as(ip)))
        return {"sweeps": sw, "residual": rs, "fell_back": fb, "colours": nc}

    def scene_times(self):
        """Per scene, last solve: start and end of its sweep CTA in ns
        (relative to the earliest start) and the SM it ran on."""
        n = len(self.scenes)
        t0 = np.zeros(n, np.int64)
        t1 = np.zeros(n, np.int64)
        sm = np.zeros(n, np.int32)
        i64 = C.POINTER(C.c_int64)
        self._check(lib().am_get_batch_scene_times(self.h, t0.ctypes.data_as(i64), t1.ctypes.data_as(i64),
                                                   sm.ctypes.data_as(C.POINTER(C.c_int32))))
        return {"start_ns": t0, "end_ns": t1, "sm": sm}

    def scene_ctas(self):
        """Per scene, last solve: CTAs that solved it (1, or the cluster size)."""
        out = np.zeros(len(self.scenes), np.int32)
        self._check(lib().am_get_batch_scene_ctas(self.h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def scene_chain(self):
        """Per scene, last solve: contacts on one sweep's critical path."""
        out = np.zeros(len(self.scenes), np.int32)
        self._check(lib().am_get_batch_scene_chain(self.h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    # learned warm start
    def learned_collect(self, enable=True, capacity=2_000_000):
        self._check(lib().am_learned_collect(self.h, int(enable), int(capacity)))

    def learned_train(self, epochs=20, batch=8192, lr=3e-3, normalise=True):
        loss = C.c_double()
        self._check(lib().am_learned_train(self.h, epochs, batch, lr, int(normalise), C.byref(loss)))
        return loss.value

    def learned_use(self, mode=1):
        self._check(lib().am_learned_use(self.h, mode))

    def learned_scope(self, all_contacts=False):
        self._check(lib().am_learned_scope(self.h, int(all_contacts)))

    def learned_info(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(lib().am_learned_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"n_params": a.value, "n_samples": b.value, "fallback_scenes": c.value}

    def learned_weights(self, set_w=None, set_norm=None):
        info = self.learned_info()
        w = np.zeros(info["n_params"], np.float32)
        nm = np.zeros(48, np.float32)
        fp = C.POINTER(C.c_float)
        sw = None if set_w is None else np.ascontiguousarray(set_w, np.float32)
        sn = None if set_norm is None else np.ascontiguousarray(set_norm, np.float32)
        self._check(lib().am_learned_weights(self.h, w.ctypes.data_as(fp),
                                             None if sw is None else sw.ctypes.data_as(fp),
                                             nm.ctypes.data_as(fp), None if sn is None else sn.ctypes.data_as(fp)))
        return w, nm

    def learned_grad(self, X, Y):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(self.learned_info()["n_params"], np.float32)
        loss = np.zeros(1, np.float32)
        fp = C.POINTER(C.c_float)
        self._check(lib().am_learned_grad(self.h, X.ctypes.data_as(fp), Y.ctypes.data_as(fp), len(X),
                                          g.ctypes.data_as(fp), loss.ctypes.data_as(fp)))
        return float(loss[0]), g

    def learned_infer(self, X, tensor_cores=True):
        X = np.ascontiguousarray(X, np.float32)
        out = np.zeros((len(X), 3), np.float32)
        fp = C.POINTER(C.c_float)
        self._check(lib().am_learned_infer(self.h, X.ctypes.data_as(fp), len(X), out.ctypes.data_as(fp),
                                           int(tensor_cores)))
        return out


class System:
    """One simulation context on the current CUDA device."""

    def __init__(self, scene, params):
        self.params = params
        self.scene = scene
        self.h = C.c_void_p()
        self._check(lib().am_create(C.byref(params), C.byref(self.h)))
        self._s = scene.struct()
        self._check(lib().am_set_scene(self.h, C.byref(self._s)))
        self.n = scene.n

    def _check(self, r):
        if r != 0:
            msg = lib().am_last_error(self.h).decode() if self.h else ""
            raise AmError(r, msg)

    def close(self):
        if self.h:
            lib().am_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # RigidBodySystem.advanceTime
    def advance_time(self, dt, n=1):
        for _ in range(n):
            self._check(lib().am_step(self.h, dt))

    step = advance_time

    # CollisionProcessor phases
    def collision_detection(self, dt=0.0):
        self._check(lib().am_collide(self.h, dt))

    def warm_start(self):
        self._check(lib().am_warm_start(self.h))

    def solve_lcp(self, dt):
        st = abi.am_solve_stats()
        self._check(lib().am_solve(self.h, dt, C.byref(st)))
        return st

    def integrate(self, dt):
        self._check(lib().am_integrate(self.h, dt))

    def stats(self):
        st = abi.am_solve_stats()
        self._check(lib().am_get_stats(self.h, C.byref(st)))
        return st

    def perf(self):
        p = abi.am_perf()
        self._check(lib().am_get_perf(self.h, C.byref(p)))
        return p

    def reset_perf(self):
        self._check(lib().am_reset_perf(self.h))

    def set_phase_timing(self, enable=True):
        """Per-phase wall times of each step (the reference's CSV columns)."""
        self._check(lib().am_set_phase_timing(self.h, int(enable)))

    def phase_times(self):
        """Seconds per phase of the last step, in abi.PHASES order."""
        out = np.zeros(abi.AM_NUM_PHASES, np.float64)
        self._check(lib().am_get_phase_times(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def step_phases(self):
        """Batched steps: device ms per phase (abi.STEP_PHASES order) summed
        since reset_perf."""
        out = np.zeros(len(abi.STEP_PHASES), np.float64)
        self._check(lib().am_get_step_phases(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return dict(zip(abi.STEP_PHASES, out.tolist()))

    def step_phase(self, phase, dt):
        """One phase of the merging step (abi.MPHASES); phases 0..7 in order make one step."""
        self._check(lib().am_step_phase(self.h, int(phase), dt))

    def single_sweep_order(self):
        n = C.c_int32(0)
        r = lib().am_single_sweep_order(self.h, None, 0, C.byref(n))
        if r not in (0, -2):
            self._check(r)
        out = np.zeros(max(1, n.value), np.int32)
        self._check(lib().am_single_sweep_order(self.h, out.ctypes.data_as(C.POINTER(C.c_int32)), len(out),
                                                C.byref(n)))
        return out[:n.value]

    def single_sweep(self, refs, dt):
        refs = np.ascontiguousarray(refs, np.int32)
        self._check(lib().am_single_sweep(self.h, refs.ctypes.data_as(C.POINTER(C.c_int32)), len(refs), dt))

    def merge_tests(self):
        """Merge / unmerge predicates on the current state (am_merge_tests):
        dict of arrays body1, body2, kind, result, metric."""
        n = C.c_int32(0)
        r = lib().am_merge_tests(self.h, None, 0, C.byref(n))
        if r not in (0, -2):
            self._check(r)
        m = max(1, n.value)
        arr = {k: np.zeros(m, np.int32) for k in ("body1", "body2", "kind", "result")}
        arr["metric"] = np.zeros(m)
        s = abi.am_bpc_tests()
        for k in ("body1", "body2", "kind", "result"):
            setattr(s, k, arr[k].ctypes.data_as(C.POINTER(C.c_int32)))
        s.metric = arr["metric"].ctypes.data_as(C.POINTER(C.c_double))
        self._check(lib().am_merge_tests(self.h, C.byref(s), m, C.byref(n)))
        return {k: v[:n.value] for k, v in arr.items()}

    def get_state(self):
        """Snapshot of the simulation state (bytes) for put_state."""
        n = C.c_int64(0)
        r = lib().am_get_state(self.h, None, 0, C.byref(n))
        if r not in (0, -2):
            self._check(r)
        buf = C.create_string_buffer(max(1, n.value))
        self._check(lib().am_get_state(self.h, buf, n.value, C.byref(n)))
        return buf.raw[:n.value]

    def put_state(self, blob):
        buf = C.create_string_buffer(bytes(blob), len(blob))
        self._check(lib().am_put_state(self.h, buf, len(blob)))

    def stream_handle(self):
        s = C.c_void_p()
        self._check(lib().am_get_stream(self.h, C.byref(s)))
        return s.value

    def set_params(self, params):
        self._check(lib().am_set_params(self.h, C.byref(params)))
        self.params = params

    def set_residual_target(self, target, check_every=10):
        self._check(lib().am_set_residual_target(self.h, target, check_every))

    def set_mixed_form(self, form=-1, refine=0):
        """AM_ORDER_MIXED: kernel form (-1 auto, 0 grid, 1 one block, 2 one
        block with the contact records in shared memory) and refinement interval."""
        self._check(lib().am_set_mixed_form(self.h, form, refine))

    def set_kinematic(self, body, axis, amplitude, frequency_hz, dt):
        """Prescribed oscillation of pinned body `body` (am_set_kinematic)."""
        ax = (C.c_double * 3)(*[float(a) for a in axis])
        self._check(lib().am_set_kinematic(self.h, int(body), ax, float(amplitude), float(frequency_hz), float(dt)))

    def mixed_form(self):
        """Form of the last AM_ORDER_MIXED solve (-1 before the first)."""
        f = C.c_int32()
        self._check(lib().am_get_mixed_form(self.h, C.byref(f)))
        return f.value

    def num_contacts(self):
        n = C.c_int32()
        self._check(lib().am_num_contacts(self.h, C.byref(n)))
        return n.value

    def contacts(self):
        n = self.num_contacts()
        buf = abi.Contacts(n)
        s = buf.struct()
        got = C.c_int32()
        self._check(lib().am_get_contacts(self.h, C.byref(s), buf.n, C.byref(got)))
        return buf.view(got.value)

    def put_bodies_struct(self, st_struct):
        self._check(lib().am_put_bodies(self.h, C.byref(st_struct)))

    def get_bodies_struct(self, st_struct):
        self._check(lib().am_get_bodies(self.h, C.byref(st_struct)))

    def topology(self):
        """RigidBodySystem.bodies: ints for free bodies, tuples of members for collections."""
        cap = 4 * self.n + 64
        items = np.zeros(cap, np.int32)
        off = np.zeros(2 * self.n + 8, np.int32)
        nt, ni = C.c_int32(), C.c_int32()
        P32 = C.POINTER(C.c_int32)
        self._check(lib().am_get_topology(self.h, items.ctypes.data_as(P32), off.ctypes.data_as(P32), cap,
                                          C.byref(nt), C.byref(ni)))
        out = []
        for t in range(nt.value):
            seg = [int(x) for x in items[off[t]:off[t + 1]]]
            out.append(tuple(seg[1:]) if seg[0] == -1 else seg[0])
        return out

    def bodies(self):
        st = abi.BodyState(self.n)
        s = st.struct()
        self._check(lib().am_get_bodies(self.h, C.byref(s)))
        return {"x": st.x.reshape(-1, 3), "R": st.R.reshape(-1, 9), "v": st.v.reshape(-1, 3),
                "omega": st.omega.reshape(-1, 3), "sleeping": st.sleeping, "parent": st.parent}


for _name in ("_check", "close", "__del__", "step", "advance_time", "stats", "num_contacts", "contacts", "bodies",
              "perf", "reset_perf", "set_phase_timing", "phase_times", "step_phases", "get_state", "put_state", "merge_tests",
              "step_phase", "single_sweep_order", "single_sweep", "stream_handle", "set_params", "topology",
              "put_bodies_struct",
              "get_bodies_struct", "collision_detection", "warm_start", "solve_lcp", "integrate"):
    setattr(BatchSystem, _name, getattr(System, _name))
