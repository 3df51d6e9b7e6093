"""Test-side ctypes binding of the oracle (oracle/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load the
oracle; the product never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from adaptivemerging_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "liboracle.so")


def build():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(abi.am_scene)]
        for f in ("or_destroy", "or_begin_step", "or_collide", "or_warm_start"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.or_step.argtypes = [C.c_void_p, C.c_double]
        L.or_set_params.argtypes = [C.c_void_p, C.POINTER(abi.am_params)]
        L.or_set_residual_target.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.or_solve.argtypes = [C.c_void_p, C.c_double]
        L.or_run.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.or_num_contacts.argtypes = [C.c_void_p]
        L.or_num_contacts.restype = C.c_int
        L.or_get_contacts.argtypes = [C.c_void_p, C.POINTER(abi.am_contacts)]
        L.or_get_bodies.argtypes = [C.c_void_p, C.POINTER(abi.am_body_state)]
        L.or_get_counters.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.or_top_ids.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int]
        L.or_top_ids.restype = C.c_int
        L.or_topology.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int,
                                  C.POINTER(C.c_int32)]
        L.or_topology.restype = C.c_int
        ip = C.POINTER(C.c_int32)
        L.or_merge_tests.argtypes = [C.c_void_p, ip, ip, ip, ip, C.POINTER(C.c_double), C.c_int]
        L.or_merge_tests.restype = C.c_int
        L.or_set_kinematic.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_double, C.c_double,
                                       C.c_double]
        L.or_set_kinematic.restype = C.c_int
        _lib = L
    return _lib


def decode_topology(items, off):
    out = []
    for t in range(len(off) - 1):
        seg = [int(x) for x in items[off[t]:off[t + 1]]]
        out.append(tuple(seg[1:]) if seg[0] == -1 else seg[0])
    return out


class Oracle:
    def __init__(self, scene, params):
        self.scene = scene
        self.params = params
        self._s = scene.struct()
        self.h = lib().or_create(C.byref(params), C.byref(self._s))
        assert self.h, "the oracle refused the scene"
        self.n = scene.n

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    def set_params(self, params):
        self.params = params
        lib().or_set_params(self.h, C.byref(params))

    def set_residual_target(self, target, check=10):
        lib().or_set_residual_target(self.h, target, check)

    def step(self, dt, n=1):
        lib().or_run(self.h, dt, n)

    def begin_step(self):
        lib().or_begin_step(self.h)

    def collide(self):
        lib().or_collide(self.h)

    def warm_start(self):
        lib().or_warm_start(self.h)

    def solve(self, dt):
        lib().or_solve(self.h, dt)

    def num_contacts(self):
        return lib().or_num_contacts(self.h)

    def contacts(self):
        n = self.num_contacts()
        buf = abi.Contacts(n)
        s = buf.struct()
        lib().or_get_contacts(self.h, C.byref(s))
        return buf.view(n)

    def bodies(self):
        st = abi.BodyState(self.n)
        s = st.struct()
        lib().or_get_bodies(self.h, C.byref(s))
        return {"x": st.x.reshape(-1, 3), "R": st.R.reshape(-1, 9), "v": st.v.reshape(-1, 3),
                "omega": st.omega.reshape(-1, 3), "sleeping": st.sleeping, "parent": st.parent}

    def counters(self):
        out = (C.c_int64 * 6)()
        ch = C.c_double()
        lib().or_get_counters(self.h, out, C.byref(ch))
        return {"sweeps": out[0], "merges": out[1], "unmerges": out[2], "top": out[3],
                "bpcs": out[4], "collections": out[5], "last_change": ch.value}

    def topology(self):
        """Top-level list: ints for free bodies, tuples of member ids for collections."""
        cap = 4 * self.n + 64
        items = np.zeros(cap, np.int32)
        off = np.zeros(2 * self.n + 8, np.int32)
        nt = C.c_int32()
        k = lib().or_topology(self.h, items.ctypes.data_as(C.POINTER(C.c_int32)),
                              off.ctypes.data_as(C.POINTER(C.c_int32)), cap, C.byref(nt))
        return decode_topology(items[:k], off[:nt.value + 1])

    def set_kinematic(self, body, axis, amplitude, frequency_hz, dt):
        ax = (C.c_double * 3)(*[float(a) for a in axis])
        r = lib().or_set_kinematic(self.h, int(body), ax, float(amplitude), float(frequency_hz), float(dt))
        assert r == 0, "the oracle refused the kinematic body"

    def merge_tests(self):
        """Merge / unmerge predicates on the current state, reference order."""
        ip = C.POINTER(C.c_int32)
        for cap in (256, 1 << 20):
            arr = {k: np.zeros(cap, np.int32) for k in ("body1", "body2", "kind", "result")}
            arr["metric"] = np.zeros(cap)
            n = lib().or_merge_tests(self.h, *(arr[k].ctypes.data_as(ip) for k in ("body1", "body2", "kind", "result")),
                                     arr["metric"].ctypes.data_as(C.POINTER(C.c_double)), cap)
            if n <= cap:
                return {k: v[:n].copy() for k, v in arr.items()}
        raise RuntimeError("too many body-pair contacts")

    def top_ids(self):
        buf = np.zeros(self.n * 2 + 16, np.int32)
        k = lib().or_top_ids(self.h, buf.ctypes.data_as(C.POINTER(C.c_int32)), len(buf))
        return buf[:k].copy()
