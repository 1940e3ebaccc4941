"""Learned aliasing correction kernels (csrc/mlp.cu): the GPU gradient of the
mean squared error against the FP64 restatement oracle/mlp.py (itself checked
against finite differences in tests/test_mlp_oracle.py), the forward kernel,
a short Adam run that fits a smooth target, the committed parameters, and
the learned mode checked against the interlaced estimator."""
import numpy as np
import pytest

from oracle import mlp as mlp_ref

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
    g64, loss64 = mlp_ref.grad(p, X, T)
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
    y64, _ = mlp_ref.forward(p, X.astype(np.float64))
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
    single paint + perceptron is closer to the interlaced estimate
    than the single paint alone: by more than 2x in rms below 0.8 k_Nyq, and
    over all bins (whose rms the noise of the few-mode corner bins dominates)."""
    from fftgal_gb300 import alias_mlp as a
    res = a.evaluate(a.load(), 256, 3e6, n_mocks=2, seed=777)
    for r in res:
        s, l = r["single"], r["learned"]
        assert l["rms_below_0p8"] < 0.5 * s["rms_below_0p8"], r
        assert l["rms_all"] < s["rms_all"], r


def _err(a, b, Pshot):
    den = np.abs(np.nan_to_num(b["P"][:, :1])) + Pshot
    ok = np.isfinite(b["P"]) & (b["N"][:, None] > 0)
    return float((np.abs(a["P"] - b["P"]) / den)[ok].max())


def test_learned_checked_and_fallback(fg):
    """fftgal_power_learned_checked_f32: held-out catalogs report the
    interlaced estimate and their disagreement, the others the learned one;
    a disagreement above tol switches every later catalog to interlaced.
    Two runs of one estimator agree to 1e-6 of (|P_0| + Pshot) (the bin sums'
    atomic order varies); learned ones to 1e-4, as the network's local-slope
    feature differences neighbouring bins."""
    import torch
    from fftgal_gb300 import alias_mlp as a, mocks
    Ng, L = 128, 1000.0
    dK, V, los = 2 * np.pi / L, L ** 3, (0.0, 0.0, 1.0)
    cats = []
    for seed in range(5):
        x, y, z, vx, vy, vz = mocks.lognormal_catalog(Ng, L, 3e5, 900 + seed, axes=(2,))
        cats.append((x.cpu().numpy(), y.cpu().numpy(), (z + vz).cpu().numpy()))
    torch.cuda.synchronize()
    params = a.load()
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    res, used, dis = g.power_learned_checked_f32(cats, V, los, dK, params, 2, 1e9)
    assert list(used) == [1, 0, 1, 0, 1]
    for c, cat in enumerate(cats):
        Pshot = V / len(cat[0])
        learned = g.power_learned_f32(*cat, V, los, dK, params)
        if used[c] == 1:
            inter = g.power_f32(*cat, V, los, dK)
            assert _err(res[c], inter, Pshot) <= 1e-6
            ok = (inter["N"] > 0) & (inter["K"] < 0.8 * np.pi * Ng / L)
            den = np.abs(inter["P"][:, 0]) + Pshot
            want = (np.abs(learned["P"][:, :3] - inter["P"][:, :3]) / den[:, None])[ok].max()
            print("checked", c, dis[c], want)
            assert abs(dis[c] - want) <= 1e-4
        else:
            assert np.isnan(dis[c])
            e = _err(res[c], learned, Pshot)
            print("learned", c, e)
            assert e <= 1e-4
    res, used, dis = g.power_learned_checked_f32(cats, V, los, dK, params, 2, 0.0)
    assert list(used) == [1, 2, 2, 2, 2] and dis[0] > 0 and np.all(np.isnan(dis[1:]))
    assert _err(res[3], g.power_f32(*cats[3], V, los, dK), V / len(cats[3][0])) <= 1e-6
    res, used, dis = g.power_learned_checked_f32(cats, V, los, dK, params, 0, 0.0)
    assert list(used) == [0] * 5 and np.all(np.isnan(dis))
