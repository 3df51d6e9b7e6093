"""ctypes mirror of include/am.h (the C ABI of libam.so).

The structures below must stay field-for-field identical to am.h; the
`test_abi_*` tests check every exported symbol and the struct sizes against a
C probe compiled from the header.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))

AM_OK = 0
AM_E_ARG = -1
AM_E_CAPACITY = -2
AM_E_NONFINITE = -3
AM_E_TIMEOUT = -4
AM_E_CUDA = -5
AM_E_STATE = -6

AM_BOX, AM_SPHERE, AM_PLANE, AM_TREE, AM_COMPOSITE = 0, 1, 2, 3, 4
AM_STATE_BROKEN, AM_STATE_ONEDGE, AM_STATE_CLEAR = 0, 1, 2
AM_BV_NULL = -1
# phases of the merging step (am_step_phase, AM_MPHASE_*)
MPHASES = ("collide", "warm_start", "single_sweep", "unmerge", "solve", "advance", "merge", "finish")
# device phases of a batched step (am_get_step_phases)
STEP_PHASES = ("detection", "warm_start", "solve_setup", "sweeps", "integration", "statistics")
AM_ORDER_REFERENCE, AM_ORDER_COLOURED, AM_ORDER_MIXED = 0, 1, 2
# am_get_phase_times order: the reference's CSV time columns
# (RigidBodySystem.exportDataToFile, RigidBodySystem.java:495-542)
PHASES = ("detection", "warmstart", "LCPSolve", "updateCollections", "contactOrdering", "singleItPGS",
          "merging", "mergingBuild", "unmerging", "unmergingBuild", "computeTime")
AM_NUM_PHASES = len(PHASES)


def AM_BV_PLANE(b):
    return -2 - b


_i32, _f64 = C.c_int32, C.c_double


class am_params(C.Structure):
    _fields_ = [
        ("iterations", _i32), ("tolerance", _f64), ("omega", _f64),
        ("iterations_in_collection", _i32), ("feedback_stiffness", _f64),
        ("enable_compliance", _i32), ("compliance", _f64),
        ("restitution_override", _i32), ("restitution", _f64),
        ("friction_override", _i32), ("friction", _f64), ("warm_start", _i32),
        ("use_gravity", _i32), ("gravity_amount", _f64), ("gravity_angle", _f64),
        ("viscous_linear", _f64), ("viscous_angular", _f64),
        ("enable_merging", _i32), ("enable_merge_pinned", _i32), ("enable_merge_cycle", _i32),
        ("enable_merge_stable_contact", _i32), ("enable_merge_let_it_breathe", _i32),
        ("enable_unmerging", _i32), ("enable_unmerge_friction", _i32),
        ("enable_unmerge_normal", _i32), ("enable_unmerge_relative_motion", _i32),
        ("update_contacts_in_collections", _i32), ("organize_contacts", _i32),
        ("metric_position_level", _i32), ("step_accum_merging", _i32),
        ("step_accum_unmerging", _i32), ("steps_between_merge_events", _i32),
        ("threshold_merge", _f64), ("threshold_unmerge", _f64), ("threshold_breath", _f64),
        ("enable_sleeping", _i32), ("sleep_step_accum", _i32), ("sleep_threshold", _f64),
        ("sliding_threshold", _f64), ("solver_order", _i32),
    ]


def default_params(**over):
    """am_params with the reference defaults (CollisionProcessor.java:1058-1083,
    Merging.java:30-54, Sleeping.java:25-30, Contact.java:518,
    RigidBodySystem.java:544-567), then `over` applied."""
    p = am_params()
    p.iterations = 30; p.tolerance = 1e-5; p.omega = 1.0; p.iterations_in_collection = 1
    p.feedback_stiffness = 0.5; p.enable_compliance = 1; p.compliance = 1e-3
    p.restitution_override = 0; p.restitution = 0.5; p.friction_override = 0; p.friction = 0.1
    p.warm_start = 1; p.use_gravity = 1; p.gravity_amount = 1.0; p.gravity_angle = 90.0
    p.viscous_linear = 1.0; p.viscous_angular = 1.0
    p.enable_merging = 1; p.enable_merge_pinned = 1; p.enable_merge_cycle = 0
    p.enable_merge_stable_contact = 1; p.enable_merge_let_it_breathe = 1
    p.enable_unmerging = 1; p.enable_unmerge_friction = 1; p.enable_unmerge_normal = 1
    p.enable_unmerge_relative_motion = 1; p.update_contacts_in_collections = 1
    p.organize_contacts = 1; p.metric_position_level = 0; p.step_accum_merging = 3
    p.step_accum_unmerging = 3; p.steps_between_merge_events = 10
    p.threshold_merge = 1e-2; p.threshold_unmerge = 2e-2; p.threshold_breath = 1e-5
    p.enable_sleeping = 1; p.sleep_step_accum = 10; p.sleep_threshold = 1e-5
    p.sliding_threshold = 0.01; p.solver_order = AM_ORDER_REFERENCE
    for k, v in over.items():
        setattr(p, k, v)
    return p


_P = C.POINTER


class am_scene(C.Structure):
    _fields_ = [
        ("n_bodies", _i32), ("type", _P(_i32)), ("pinned", _P(_i32)), ("x", _P(_f64)),
        ("R", _P(_f64)), ("v", _P(_f64)), ("omega", _P(_f64)), ("mass", _P(_f64)),
        ("inertia", _P(_f64)), ("friction", _P(_f64)), ("restitution", _P(_f64)),
        ("shape", _P(_f64)), ("n_nodes", _i32), ("body_root", _P(_i32)), ("node_c", _P(_f64)),
        ("node_r", _P(_f64)), ("node_child0", _P(_i32)), ("node_nchild", _P(_i32)),
        ("bbox", _P(_f64)),
        ("n_subs", _i32), ("sub_parent", _P(_i32)), ("sub_type", _P(_i32)), ("sub_shape", _P(_f64)),
        ("sub_R", _P(_f64)), ("sub_t", _P(_f64)),
    ]


class am_body_state(C.Structure):
    _fields_ = [("x", _P(_f64)), ("R", _P(_f64)), ("v", _P(_f64)), ("omega", _P(_f64)),
                ("sleeping", _P(_i32)), ("parent", _P(_i32))]


class am_contacts(C.Structure):
    _fields_ = [("body1", _P(_i32)), ("body2", _P(_i32)), ("bv1", _P(_i32)), ("bv2", _P(_i32)),
                ("info", _P(_i32)), ("frame", _P(_f64)), ("jac", _P(_f64)),
                ("violation", _P(_f64)), ("lambda_", _P(_f64)), ("bD", _P(_f64)),
                ("state", _P(_i32)), ("fresh", _P(_i32))]


class am_solve_stats(C.Structure):
    _fields_ = [("n_contacts", _i32), ("sweeps", _i32), ("last_change", _f64),
                ("residual_abs", _f64), ("residual_rel", _f64)]


class am_perf(C.Structure):
    _fields_ = [("launches", C.c_int64), ("pgs_launches", C.c_int64), ("pgs_ms", _f64),
                ("contact_sweeps", C.c_int64), ("steps", C.c_int64), ("merge_events", C.c_int64),
                ("unmerge_events", C.c_int64)]


class am_batch_stats(C.Structure):
    _fields_ = [("n_scenes", _i32), ("converged", _i32), ("sweeps_max", _i32), ("threads", _i32),
                ("stage_slots", _i32), ("resident_scenes", _i32), ("cluster_scenes", _i32), ("cluster_size", _i32),
                ("sweeps_sum", C.c_int64), ("contact_sweeps", C.c_int64), ("residual_max", _f64)]


def ptr(a, ctype):
    """Borrowed pointer to a contiguous numpy array (None -> NULL)."""
    if a is None:
        return C.cast(None, _P(ctype))
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P(ctype))


class SceneArrays:
    """Owns the numpy arrays behind one am_scene (keeps them alive)."""

    FIELDS_I = ("type", "pinned", "body_root", "node_child0", "node_nchild", "sub_parent", "sub_type")

    def __init__(self, **arrays):
        self.a = {}
        for k, v in arrays.items():
            dt = np.int32 if k in self.FIELDS_I else np.float64
            self.a[k] = np.ascontiguousarray(np.asarray(v, dtype=dt))
        self.n = len(self.a["type"])
        self.n_nodes = len(self.a["node_r"])

    def __getitem__(self, k):
        return self.a[k]

    def struct(self):
        s = am_scene()
        s.n_bodies = self.n
        s.n_nodes = self.n_nodes
        s.n_subs = len(self.a["sub_parent"]) if "sub_parent" in self.a else 0
        for k, v in self.a.items():
            setattr(s, k, ptr(v, _i32 if k in self.FIELDS_I else _f64))
        return s


class am_bpc_tests(C.Structure):
    _fields_ = [("body1", _P(_i32)), ("body2", _P(_i32)), ("kind", _P(_i32)), ("result", _P(_i32)),
                ("metric", _P(_f64))]


class Contacts:
    """numpy buffers for am_contacts of capacity n."""

    def __init__(self, n):
        n = max(int(n), 1)
        self.n = n
        self.body1 = np.zeros(n, np.int32); self.body2 = np.zeros(n, np.int32)
        self.bv1 = np.zeros(n, np.int32); self.bv2 = np.zeros(n, np.int32)
        self.info = np.zeros(n, np.int32)
        self.frame = np.zeros(12 * n); self.jac = np.zeros(36 * n)
        self.violation = np.zeros(2 * n); self.lam = np.zeros(3 * n); self.bD = np.zeros(6 * n)
        self.state = np.zeros(n, np.int32); self.fresh = np.zeros(n, np.int32)

    def struct(self):
        s = am_contacts()
        for k in ("body1", "body2", "bv1", "bv2", "info", "state", "fresh"):
            setattr(s, k, ptr(getattr(self, k), _i32))
        s.frame = ptr(self.frame, _f64); s.jac = ptr(self.jac, _f64)
        s.violation = ptr(self.violation, _f64); s.lambda_ = ptr(self.lam, _f64)
        s.bD = ptr(self.bD, _f64)
        return s

    def view(self, n):
        """dict of arrays trimmed to the first n contacts."""
        return {
            "body1": self.body1[:n].copy(), "body2": self.body2[:n].copy(),
            "bv1": self.bv1[:n].copy(), "bv2": self.bv2[:n].copy(), "info": self.info[:n].copy(),
            "frame": self.frame[:12 * n].reshape(n, 12).copy(),
            "jac": self.jac[:36 * n].reshape(n, 36).copy(),
            "violation": self.violation[:2 * n].reshape(n, 2).copy(),
            "lambda": self.lam[:3 * n].reshape(n, 3).copy(),
            "bD": self.bD[:6 * n].reshape(n, 6).copy(),
            "state": self.state[:n].copy(), "fresh": self.fresh[:n].copy(),
        }


class BodyState:
    def __init__(self, n):
        self.x = np.zeros(3 * n); self.R = np.zeros(9 * n); self.v = np.zeros(3 * n)
        self.omega = np.zeros(3 * n); self.sleeping = np.zeros(n, np.int32)
        self.parent = np.zeros(n, np.int32)

    def struct(self):
        s = am_body_state()
        s.x = ptr(self.x, _f64); s.R = ptr(self.R, _f64); s.v = ptr(self.v, _f64)
        s.omega = ptr(self.omega, _f64); s.sleeping = ptr(self.sleeping, _i32)
        s.parent = ptr(self.parent, _i32)
        return s
