"""am_learned_infer_noalloc, the inference call that passes its rows through a
fixed device scratch instead of per-call temporaries, against the allocating
am_learned_infer on the same weights and rows, two calls in a row each."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from adaptivemerging_gb300 import scenes
from helpers import params

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NIN, NOUT = 24, 3
FP = C.POINTER(C.c_float)


def _max_rows():
    with open(os.path.join(ROOT, "include", "am.h")) as f:
        return int(re.search(r"#define AM_NOALLOC_MAX_ROWS (\d+)", f.read()).group(1))


def _system():
    from adaptivemerging_gb300 import native
    return native.BatchSystem([scenes.bin_scene(30, 7, gap=-0.001)], params(friction_override=0), threads=128,
                              residual_target=1e-6, check_every=10)


def _noalloc(L, g, X, tc):
    out = np.full((len(X), NOUT), np.nan, np.float32)
    X = np.ascontiguousarray(X, np.float32)
    r = L.am_learned_infer_noalloc(g.h, X.ctypes.data_as(FP), len(X), out.ctypes.data_as(FP), tc)
    return r, out


def test_noalloc_inference_matches_allocating_call(gpu_lib):
    L = gpu_lib
    g = _system()
    rng = np.random.default_rng(3)
    n_par = g.learned_info()["n_params"]
    w = (rng.standard_normal(n_par) * 0.3).astype(np.float32)
    nm = np.concatenate([rng.standard_normal(NIN) * 0.1, 0.5 + rng.random(NIN)]).astype(np.float32)
    g.learned_weights(set_w=w, set_norm=nm)       # setup: the weights are allocated here
    for tc in (1, 0):
        for n in (1000, 4099):                    # two calls in a row, different sizes
            X = rng.standard_normal((n, NIN)).astype(np.float32)
            ref = g.learned_infer(X, tensor_cores=bool(tc))
            r, out = _noalloc(L, g, X, tc)
            assert r == 0
            # same kernels and weights: equal within the inference tests' FP32 tolerance
            np.testing.assert_allclose(out, ref, rtol=1e-6, atol=1e-6)
    # the largest accepted size, then one row more
    m = _max_rows()
    X = rng.standard_normal((m + 1, NIN)).astype(np.float32)
    r, out = _noalloc(L, g, X[:m], 1)
    assert r == 0
    np.testing.assert_allclose(out[-5:], g.learned_infer(X[m - 5:m], tensor_cores=True), rtol=1e-6, atol=1e-6)
    r, _ = _noalloc(L, g, X, 1)
    assert r == -2                                 # AM_E_CAPACITY
    r, _ = _noalloc(L, g, X[:0], 1)
    assert r == -1                                 # AM_E_ARG


def test_noalloc_inference_takes_no_device_memory(gpu_lib):
    """After the first call, calls of several sizes leave the device's free
    memory where it was: nothing is allocated per call."""
    import torch
    L = gpu_lib
    g = _system()
    rng = np.random.default_rng(5)
    n_par = g.learned_info()["n_params"]
    g.learned_weights(set_w=(rng.standard_normal(n_par) * 0.3).astype(np.float32))
    X = rng.standard_normal((_max_rows(), NIN)).astype(np.float32)
    assert _noalloc(L, g, X[:10], 1)[0] == 0       # first call: looks up the scratch
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for n in (1, 777, 4096, 30000, _max_rows()):
        for tc in (1, 0):
            assert _noalloc(L, g, X[:n], tc)[0] == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_inference_needs_weights(gpu_lib):
    g = _system()
    r, _ = _noalloc(gpu_lib, g, np.zeros((4, NIN), np.float32), 1)
    assert r == -6                                 # AM_E_STATE: no weights set up yet
    # recording samples initialises the network but sets up no weights either
    g.learned_collect(True, 1000)
    r, _ = _noalloc(gpu_lib, g, np.zeros((4, NIN), np.float32), 1)
    assert r == -6
    g.learned_use(1)                               # the default weights, packed for inference
    r, out = _noalloc(gpu_lib, g, np.zeros((4, NIN), np.float32), 1)
    assert r == 0 and np.isfinite(out).all()
