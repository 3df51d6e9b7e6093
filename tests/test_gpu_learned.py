"""Learned warm start: the device MLP's loss and gradients against a float64
PyTorch restatement of the same network, BF16 tensor-core inference against
FP32, and what the learned start gains over the plain previous-frame start on
batched scenes solved to a relative LCP residual of 1e-6."""
import ctypes as C

import numpy as np
import pytest

from adaptivemerging_gb300 import scenes
from helpers import params

pytestmark = pytest.mark.gpu

DT = 0.005
NIN, NH, NOUT = 24, 64, 3


def _unpack(w):
    o = 0
    out = {}
    for name, shape in (("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)),
                        ("b3", (NOUT,))):
        n = int(np.prod(shape))
        out[name] = (o, shape)
        o += n
    assert o == len(w)
    return out


def _torch_loss_grad(w, nm, X, Y):
    """float64 forward / backward of the MLP 24 -> 64 -> 64 -> 3, erf GELU, MSE"""
    torch = pytest.importorskip("torch")
    lay = _unpack(w)
    t = torch.tensor(w, dtype=torch.float64, requires_grad=True)
    p = {k: t[o:o + int(np.prod(s))].view(*s) for k, (o, s) in lay.items()}
    x = (torch.tensor(X, dtype=torch.float64) - torch.tensor(nm[:NIN], dtype=torch.float64)) * \
        torch.tensor(nm[NIN:], dtype=torch.float64)
    gelu = torch.nn.functional.gelu
    a1 = gelu(x @ p["W1"].T + p["b1"])
    a2 = gelu(a1 @ p["W2"].T + p["b2"])
    y = a2 @ p["W3"].T + p["b3"]
    loss = ((y - torch.tensor(Y, dtype=torch.float64)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), t.grad.numpy(), y.detach().numpy()


def _system(n_scenes=8, seed=11, sizes=(20, 120), gap=-0.001, **kw):
    from adaptivemerging_gb300 import native
    sc = [scenes.bin_scene(n, seed * 1000 + n, gap=gap) for n in np.linspace(*sizes, n_scenes).astype(int)]
    P = params(friction_override=0, iterations=kw.pop("iterations", 500))
    return native.BatchSystem(sc, P, threads=kw.pop("threads", 128), residual_target=kw.pop("residual_target", 1e-6),
                              check_every=kw.pop("check_every", 10))


def _random_net(g, rng, scale=0.3):
    n = g.learned_info()["n_params"]
    w = (rng.standard_normal(n) * scale).astype(np.float32)
    nm = np.concatenate([rng.standard_normal(NIN) * 0.1, 0.5 + rng.random(NIN)]).astype(np.float32)
    g.learned_weights(set_w=w, set_norm=nm)
    return w, nm


def test_learned_gradients_match_torch_fp64(gpu_lib):
    g = _system()
    rng = np.random.default_rng(5)
    w, nm = _random_net(g, rng)
    for n in (1, 37, 256, 1000):   # ragged sizes: partial blocks
        X = rng.standard_normal((n, NIN)).astype(np.float32)
        Y = rng.standard_normal((n, NOUT)).astype(np.float32)
        loss, grad = g.learned_grad(X, Y)
        lr, gr, _ = _torch_loss_grad(w, nm, X, Y)
        # FP32 kernels (FMA, shared-memory atomics) against float64
        assert abs(loss - lr) <= 1e-5 * max(1.0, abs(lr)), (n, loss, lr)
        err = np.abs(grad - gr).max() / max(1e-12, np.abs(gr).max())
        assert err <= 1e-4, (n, err)
        # every block of the parameter vector carries gradient
        for name, (o, s) in _unpack(w).items():
            assert np.abs(gr[o:o + int(np.prod(s))]).max() > 0, name


def test_learned_gradient_finite_differences(gpu_lib):
    """central differences of the float64 restatement confirm the analytic
    gradient that the device gradient is checked against"""
    g = _system()
    rng = np.random.default_rng(6)
    w, nm = _random_net(g, rng)
    X = rng.standard_normal((64, NIN)).astype(np.float32)
    Y = rng.standard_normal((64, NOUT)).astype(np.float32)
    _, grad = g.learned_grad(X, Y)
    for k in rng.choice(len(w), 24, replace=False):
        h = 1e-3
        wp, wm = w.astype(np.float64).copy(), w.astype(np.float64).copy()
        wp[k] += h
        wm[k] -= h
        fd = (_torch_loss_grad(wp, nm, X, Y)[0] - _torch_loss_grad(wm, nm, X, Y)[0]) / (2 * h)
        assert abs(grad[k] - fd) <= 2e-4 * max(1.0, abs(fd)) + 1e-5, (k, grad[k], fd)


def test_bf16_tensor_core_inference_matches_fp32(gpu_lib):
    g = _system()
    rng = np.random.default_rng(7)
    w, nm = _random_net(g, rng)
    for n in (1, 15, 16, 17, 1000, 4099):
        X = rng.standard_normal((n, NIN)).astype(np.float32)
        yt = g.learned_infer(X, tensor_cores=True)
        yf = g.learned_infer(X, tensor_cores=False)
        _, _, yr = _torch_loss_grad(w, nm, X, np.zeros((n, NOUT), np.float32))
        scale = max(1.0, np.abs(yr).max())
        assert np.abs(yf - yr).max() <= 1e-5 * scale, n
        # BF16 operands (8-bit mantissa), FP32 accumulation, three layers
        assert np.abs(yt - yr).max() <= 3e-2 * scale, (n, np.abs(yt - yr).max(), scale)


def test_training_reduces_loss(gpu_lib):
    g = _system(sizes=(100, 400), gap=0.01)   # falling bodies: fresh contacts to record
    g.learned_collect(True, 200_000)
    for _ in range(160):
        g.step(DT)
    n = g.learned_info()["n_samples"]
    assert n >= 256, n
    l0 = g.learned_train(epochs=1, batch=n // 8, lr=1e-3)
    l1 = g.learned_train(epochs=60, batch=n // 8, lr=1e-3, normalise=False)
    assert np.isfinite(l1) and l1 < 0.5 * l0, (l0, l1)


def test_learned_start_meets_residual_target_and_reports_gain(gpu_lib):
    """One batch records (features, converged impulse) pairs and trains the
    network; then, for 40 steps, a second context loads the first one's state
    before each step (am_put_state) and solves the same step from the learned
    start.  Both solve identical problems, so the learned start must reach the
    residual target on at least every scene the plain start does (a scene
    whose learned start falls short is solved again from the plain start in
    the same CTA); the contact-sweeps ratio is the learned start's net gain on
    equal problems."""
    # bodies dropped from a grid: contacts keep appearing while the piles form
    a = _system(n_scenes=16, seed=21, sizes=(100, 400), gap=0.01)
    b = _system(n_scenes=16, seed=21, sizes=(100, 400), gap=0.01)
    a.learned_collect(True, 500_000)
    for _ in range(150):
        a.step(DT)
    n = a.learned_info()["n_samples"]
    assert n >= 256, n
    a.learned_train(epochs=40, batch=min(1024, n // 4), lr=2e-3)
    w, nm = a.learned_weights()
    b.learned_weights(set_w=w, set_norm=nm)
    b.learned_use(1)
    a.learned_collect(False)
    cs_plain = cs_learned = 0
    conv_plain = conv_learned = 0
    falls = 0
    for _ in range(40):
        b.put_state(a.get_state())
        a.step(DT)
        b.step(DT)
        sa, sb = a.batch_stats(), b.batch_stats()
        cs_plain += sa.contact_sweeps
        cs_learned += sb.contact_sweeps
        conv_plain += sa.converged
        conv_learned += sb.converged
        falls += b.learned_info()["fallback_scenes"]
    gain = cs_plain / max(1, cs_learned)
    print(f"learned start on equal problems: contact-sweeps plain {cs_plain}, learned {cs_learned} (x{gain:.2f}); "
          f"converged scene-steps plain {conv_plain}, learned {conv_learned} of {40 * 16}; "
          f"fallback scene-steps {falls}")
    assert cs_learned > 0
    assert conv_learned >= conv_plain


def test_grid_barrier_wait_gives_up(gpu_lib):
    """The bounded grid barrier of the FP64 sweeps: a barrier that cannot
    complete (one arrival short) ends every block's wait after the poll limit
    with AM_E_TIMEOUT in the status word, and the context keeps working."""
    from adaptivemerging_gb300 import native
    g = native.System(scenes.tower(4, seed=1), params(iterations=20))
    st = C.c_int32(0)
    g._check(native.lib().am_check_barrier_timeout(g.h, 12, C.byref(st)))
    assert st.value == -4                          # AM_E_TIMEOUT
    g.step(0.01)                                   # the context still steps
    assert g.num_contacts() > 0
