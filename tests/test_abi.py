"""The C ABI library loads, exports every entry point declared in
include/am.h, and its structures have the layout the ctypes mirror assumes
(checked against a probe compiled from the header with gcc).  No compute
call is made, so this runs without a GPU."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from adaptivemerging_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "am.h")


def declared():
    src = open(HDR).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|void|const char\*)\s+(am_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from adaptivemerging_gb300 import build
    build.build()
    return C.CDLL(os.path.join(ROOT, "adaptivemerging_gb300", "libam.so"))


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_declared_symbols():
    from adaptivemerging_gb300 import native
    assert set(declared()) == set(native.EXPORTS)


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "am.h"
int main(void) {
  printf("am_params %zu %zu %zu %zu\n", sizeof(am_params), offsetof(am_params, tolerance),
         offsetof(am_params, threshold_breath), offsetof(am_params, solver_order));
  printf("am_scene %zu %zu\n", sizeof(am_scene), offsetof(am_scene, node_nchild));
  printf("am_contacts %zu %zu\n", sizeof(am_contacts), offsetof(am_contacts, fresh));
  printf("am_body_state %zu\n", sizeof(am_body_state));
  printf("am_solve_stats %zu %zu\n", sizeof(am_solve_stats), offsetof(am_solve_stats, residual_rel));
  printf("am_perf %zu %zu\n", sizeof(am_perf), offsetof(am_perf, unmerge_events));
  return 0;
}
"""


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict((l.split()[0], [int(x) for x in l.split()[1:]]) for l in
               subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    assert out["am_params"] == [C.sizeof(abi.am_params), abi.am_params.tolerance.offset,
                                abi.am_params.threshold_breath.offset, abi.am_params.solver_order.offset]
    assert out["am_scene"] == [C.sizeof(abi.am_scene), abi.am_scene.node_nchild.offset]
    assert out["am_contacts"] == [C.sizeof(abi.am_contacts), abi.am_contacts.fresh.offset]
    assert out["am_body_state"] == [C.sizeof(abi.am_body_state)]
    assert out["am_solve_stats"] == [C.sizeof(abi.am_solve_stats), abi.am_solve_stats.residual_rel.offset]
    assert out["am_perf"] == [C.sizeof(abi.am_perf), abi.am_perf.unmerge_events.offset]


def test_defaults_match_reference(lib):
    p = abi.am_params()
    lib.am_params_default(C.byref(p))
    q = abi.default_params()
    for f, _ in abi.am_params._fields_:
        assert getattr(p, f) == getattr(q, f), f
    assert (p.iterations, p.tolerance, p.feedback_stiffness, p.compliance) == (30, 1e-5, 0.5, 1e-3)
    assert (p.step_accum_merging, p.steps_between_merge_events, p.threshold_merge) == (3, 10, 1e-2)


def test_argument_errors_without_gpu(lib):
    """Invalid arguments are rejected with a status code, never a crash."""
    lib.am_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    h = C.c_void_p()
    assert lib.am_create(None, C.byref(h)) == abi.AM_E_ARG
    p = abi.default_params(enable_merge_cycle=1)
    lib.am_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(C.c_void_p)]
    assert lib.am_create(C.byref(p), C.byref(h)) == abi.AM_E_ARG
    lib.am_step.argtypes = [C.c_void_p, C.c_double]
    assert lib.am_step(None, 0.01) == abi.AM_E_ARG


def test_malformed_sphere_trees_are_refused_on_the_host(lib):
    """am_set_scene checks the node arrays before anything reaches the
    device: a node that lists itself (or an earlier node) as a child would
    never end a traversal, and a child range past the node array would read
    out of bounds.  Both come back as AM_E_ARG, with no CUDA call made."""
    from adaptivemerging_gb300 import scenes
    lib.am_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(C.c_void_p)]
    lib.am_set_scene.argtypes = [C.c_void_p, C.POINTER(abi.am_scene)]
    lib.am_set_batch.argtypes = [C.c_void_p, C.POINTER(abi.am_scene), C.c_int32]
    lib.am_destroy.argtypes = [C.c_void_p]
    lib.am_last_error.argtypes = [C.c_void_p]
    lib.am_last_error.restype = C.c_char_p
    good = scenes.funnel_clumps(2, seed=5)
    root = int(good.a["body_root"][good.a["type"].tolist().index(abi.AM_TREE)])
    h = C.c_void_p()
    assert lib.am_create(C.byref(abi.default_params(enable_merging=0)), C.byref(h)) == 0
    try:
        for child0, nchild in ((root, 1), (root + 1, len(good.a["node_r"]))):
            arr = {k: np.array(v, copy=True) for k, v in good.a.items()}
            arr["node_child0"][root] = child0
            arr["node_nchild"][root] = nchild
            bad = abi.SceneArrays(**arr)
            s = bad.struct()
            assert lib.am_set_scene(h, C.byref(s)) == abi.AM_E_ARG
            assert b"children must follow it" in lib.am_last_error(h)
            batch = (abi.am_scene * 2)(good.struct(), s)
            assert lib.am_set_batch(h, batch, 2) == abi.AM_E_ARG
    finally:
        lib.am_destroy(h)


def test_composite_bodies_are_refused_on_the_host(lib):
    """The library has no composite path yet: a scene with a composite body
    (AM_COMPOSITE, with its sub-bodies in am_scene) is refused with AM_E_ARG
    before any device work."""
    from adaptivemerging_gb300 import scenes
    lib.am_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(C.c_void_p)]
    lib.am_set_scene.argtypes = [C.c_void_p, C.POINTER(abi.am_scene)]
    lib.am_destroy.argtypes = [C.c_void_p]
    lib.am_last_error.argtypes = [C.c_void_p]
    lib.am_last_error.restype = C.c_char_p
    b = scenes.Builder()
    b.composite((0.0, 1.0, 0.0), 1.0, np.eye(3) / 6, [-0.5, -0.5, -0.5, 0.5, 0.5, 0.5],
                [(abi.AM_BOX, [1.0, 1.0, 1.0, 0.0], scenes.IDENT, [0.0, 0.0, 0.0])])
    b.plane((0, 0, 0), (0, 1, 0))
    s = b.build().struct()
    h = C.c_void_p()
    assert lib.am_create(C.byref(abi.default_params(enable_merging=0)), C.byref(h)) == 0
    try:
        assert lib.am_set_scene(h, C.byref(s)) == abi.AM_E_ARG
        assert lib.am_last_error(h) == b"composite bodies have no device path yet"
    finally:
        lib.am_destroy(h)


_SWEEP_CALLS = {
 "am_step": "(h, 0.01)", "am_collide": "(h, 0.01)", "am_warm_start": "(h,)", "am_solve": "(h, 0.01, None)",
 "am_integrate": "(h, 0.01)", "am_step_phase": "(h, 0, 0.01)", "am_step_phase_bad": "(h, 99, 0.01)",
 "am_single_sweep_order": "(h, None, 0, C.byref(i32))", "am_single_sweep": "(h, None, 0, 0.01)",
 "am_merge_tests": "(h, None, 0, C.byref(i32))", "am_get_state": "(h, None, 0, C.byref(i64))",
 "am_put_state": "(h, None, 0)", "am_get_bodies": "(h, None)", "am_put_bodies": "(h, None)",
 "am_num_contacts": "(h, C.byref(i32))", "am_get_contacts": "(h, None, 0, C.byref(i32))", "am_get_stats": "(h, None)",
 "am_set_batch": "(h, None, 0)", "am_set_batch_options": "(h, 0, 1e-6, 10)", "am_get_batch_stats": "(h, None)",
 "am_set_batch_local_sweeps": "(h, 1)", "am_set_batch_clusters": "(h, 1)", "am_set_batch_size_classes": "(h, 1)",
 "am_set_batch_stage": "(h, 64)", "am_set_batch_cluster_stage": "(h, 64)", "am_set_batch_relaxation": "(h, 1.0, 0)",
 "am_set_batch_accel": "(h, 1)", "am_set_batch_critical": "(h, 0.5, 640)", "am_set_residual_target": "(h, 1e-6, 10)",
 "am_set_kinematic": "(h, 0, None, 0.1, 1.0, 0.01)", "am_set_mixed_form": "(h, -1, 0)", "am_get_mixed_form": "(h, C.byref(i32))",
 "am_get_batch_scene_stats": "(h, None, None, None, None)", "am_get_batch_scene_times": "(h, None, None, None)",
 "am_get_batch_scene_ctas": "(h, None)", "am_get_batch_scene_chain": "(h, None)",
 "am_learned_collect": "(h, 1, 100)", "am_learned_train": "(h, 1, 32, 1e-3, 1, None)", "am_learned_use": "(h, 1)",
 "am_learned_scope": "(h, 0)", "am_learned_weights": "(h, None, None, None, None)",
 "am_learned_info": "(h, None, None, None)", "am_learned_grad": "(h, None, None, 0, None, None)",
 "am_learned_infer": "(h, None, 0, None, 1)", "am_learned_infer_noalloc": "(h, None, 0, None, 1)",
 "am_get_topology": "(h, None, None, 0, C.byref(i32), C.byref(i32))", "am_get_perf": "(h, None)", "am_reset_perf": "(h,)",
 "am_set_phase_timing": "(h, 1)", "am_get_phase_times": "(h, None)", "am_get_step_phases": "(h, None)",
 "am_check_barrier_timeout": "(h, 4, C.byref(i32))", "am_get_stream": "(h, None)",
}

_SWEEP_CHILD = r"""
import ctypes as C, sys
sys.path.insert(0, sys.argv[1])
from adaptivemerging_gb300 import abi
from tests.test_abi import _SWEEP_CALLS
L = C.CDLL(sys.argv[2])
L.am_create.argtypes = [C.POINTER(abi.am_params), C.POINTER(C.c_void_p)]
L.am_destroy.argtypes = [C.c_void_p]
h = C.c_void_p()
assert L.am_create(C.byref(abi.default_params()), C.byref(h)) == 0
i32 = C.c_int32(0); i64 = C.c_int64(0)
for name, args in _SWEEP_CALLS.items():
    fn = getattr(L, name.replace("_bad", ""))
    fn.restype = C.c_int32
    a = tuple(C.c_void_p(x.value) if isinstance(x, C.c_void_p) else (C.c_double(x) if isinstance(x, float) else x)
              for x in eval(args))
    print(name, fn(*a), flush=True)
L.am_destroy(h)
"""


def test_every_entry_point_answers_without_a_scene(lib):
    """Every entry point on a context with no scene loaded, with null
    pointers and zero sizes, returns a status (AM_OK, AM_E_ARG or
    AM_E_STATE): nothing crashes, and nothing reaches a CUDA call (no GPU
    is needed).  The calls run in a child process, so a crash fails the
    test instead of the test session."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = os.path.join(root, "adaptivemerging_gb300", "libam.so")
    r = subprocess.run([sys.executable, "-c", _SWEEP_CHILD, root, so], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = dict(line.rsplit(" ", 1) for line in r.stdout.split("\n") if line.strip())
    assert set(got) == set(_SWEEP_CALLS)
    allowed = {str(abi.AM_OK), str(abi.AM_E_ARG), str(abi.AM_E_STATE)}
    assert all(v in allowed for v in got.values()), got
