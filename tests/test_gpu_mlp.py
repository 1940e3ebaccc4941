"""Learned aliasing correction kernels (csrc/mlp.cu): the GPU gradient of the
mean squared error against an FP64 restatement (fftgal_gb300.alias_mlp.grad_np,
itself checked against finite differences), the forward kernel, and a short
Adam run that fits a smooth target."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def test_gradient_against_fp64(fg):
    import torch
    from fftgal_gb300 import alias_mlp as a
    rng = np.random.default_rng(3)
    p = a.init_params(5)
    p[a.LAYOUT["W4"][0]:a.LAYOUT["W4"][0] + a.LAYOUT["W4"][1]] *= 10  # non-trivial output layer
    X = rng.standard_normal((300, a.IN)).astype(np.float32)
    T = rng.standard_normal((300, a.OUT)).astype(np.float32)
    tr = a.Trainer(p)
    g, loss = tr.grad(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"))
    g = g.cpu().numpy().astype(np.float64)
    g64, loss64 = a.grad_np(p, X, T)
    assert abs(loss - loss64) <= 1e-5 * loss64
    assert np.linalg.norm(g - g64) <= 1e-4 * np.linalg.norm(g64)
    for k, (o, n) in a.LAYOUT.items():  # every layer, not just the norm
        assert np.linalg.norm(g[o:o + n] - g64[o:o + n]) <= 2e-4 * np.linalg.norm(g64[o:o + n]) + 1e-12, k


def test_forward_against_fp64(fg):
    from fftgal_gb300 import alias_mlp as a
    rng = np.random.default_rng(4)
    p = a.init_params(6)
    X = rng.standard_normal((500, a.IN)).astype(np.float32)
    y = a.forward_gpu(p, X)
    y64, _ = a.forward_np(p, X.astype(np.float64))
    assert np.abs(y - y64).max() <= 1e-5 * max(1.0, np.abs(y64).max())


def test_adam_fits_a_smooth_target(fg):
    from fftgal_gb300 import alias_mlp as a
    rng = np.random.default_rng(7)
    X = rng.uniform(-1, 1, (4000, a.IN)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], 0.5 * X[:, 2] ** 2, X[:, 3] * X[:, 4]], 1).astype(np.float32)
    params, hist = a.train(X, T, epochs=40, batch=512, lr=3e-3, seed=1)
    assert hist[-1] < 0.05 * hist[0], hist[::10]


def test_committed_params_correct_single_paint(fg):
    """The committed parameters, on fresh mocks outside the training seeds:
    single paint + perceptron is closer to the interlaced estimate (the judge)
    than the single paint alone: by more than 2x in rms below 0.8 k_Nyq, and
    over all bins (whose rms the noise of the few-mode corner bins dominates)."""
    from fftgal_gb300 import alias_mlp as a
    res = a.evaluate(a.load(), 256, 3e6, n_mocks=2, seed=777)
    for r in res:
        s, l = r["single"], r["learned"]
        assert l["rms_below_0p8"] < 0.5 * s["rms_below_0p8"], r
        assert l["rms_all"] < s["rms_all"], r
