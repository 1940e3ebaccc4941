"""The FP64 perceptron restatement (oracle/mlp.py) that the GPU gradient and
forward kernels are checked against: its gradient against central finite
differences of its own loss, and its parameter layout against the library's
(fftgal_mlp_nparams) and the trainer's.  CPU only."""
import numpy as np

from oracle import mlp as ref


def test_gradient_against_finite_differences():
    rng = np.random.default_rng(11)
    p = rng.normal(0, 0.3, ref.NPARAMS)
    X = rng.standard_normal((40, ref.IN))
    T = rng.standard_normal((40, ref.OUT))
    g, loss = ref.grad(p, X, T)
    idx = np.concatenate([rng.choice(np.arange(o, o + n), size=min(n, 12), replace=False)
                          for o, n in ref.LAYOUT.values()])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (ref.grad(p + e, X, T)[1] - ref.grad(p - e, X, T)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    y, _ = ref.forward(p, X)
    assert abs(loss - ((y - T) ** 2).sum() / len(X)) <= 1e-12 * loss


def test_layout_matches_library_and_trainer():
    from fftgal_gb300 import alias_mlp, lib
    assert lib().fftgal_mlp_nparams() == ref.NPARAMS == alias_mlp.NPARAMS
    assert alias_mlp.LAYOUT == ref.LAYOUT
