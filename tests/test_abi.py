"""The C ABI library loads, exports every entry point declared in
include/am.h, and its structures have the layout the ctypes mirror assumes
(checked against a probe compiled from the header with gcc).  No compute
call is made, so this runs without a GPU."""
import ctypes as C
import os
import re
import subprocess

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
    (the oracle's type 4) is refused with AM_E_ARG before any device work."""
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
        assert lib.am_last_error(h) == b"unknown body type"
    finally:
        lib.am_destroy(h)
