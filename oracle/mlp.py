"""FP64 restatement of the learned-correction perceptron (TEST INFRASTRUCTURE
ONLY): the forward pass of mlp_forward_kernel and the gradient of
mlp_grad_kernel (fftgal_gb300/csrc/mlp.cu), as the reference for their
parity tests.  Only tests/ import it.

Network: 5 -> 64 -> 64 -> 64 -> 3, tanh hidden units, linear output; loss =
mean over samples of |y - t|^2.  Parameter layout (floats, the kernels'):
W1[5][64] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64][3] b4[3].
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 5, 64, 3
SHAPES = {"W1": (IN, HID), "b1": (HID,), "W2": (HID, HID), "b2": (HID,), "W3": (HID, HID), "b3": (HID,),
          "W4": (HID, OUT), "b4": (OUT,)}


def _layout():
    off, out = 0, {}
    for name, shape in SHAPES.items():
        n = int(np.prod(shape))
        out[name] = (off, n)
        off += n
    return out, off


LAYOUT, NPARAMS = _layout()


def unpack(p):
    return {k: np.asarray(p[o:o + n], dtype=np.float64).reshape(SHAPES[k]) for k, (o, n) in LAYOUT.items()}


def forward(p, X):
    """Outputs y[n][3] and the hidden activations, in FP64."""
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = np.tanh(X @ w["W1"] + w["b1"])
    a2 = np.tanh(a1 @ w["W2"] + w["b2"])
    a3 = np.tanh(a2 @ w["W3"] + w["b3"])
    return a3 @ w["W4"] + w["b4"], (a1, a2, a3)


def grad(p, X, T):
    """Gradient (flat, the kernels' layout) and value of the mean over
    samples of |y - t|^2, in FP64."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    n = len(X)
    w = unpack(p)
    y, (a1, a2, a3) = forward(p, X)
    r = y - T
    loss = float((r * r).sum() / n)
    d4 = 2.0 * r / n
    d3 = (d4 @ w["W4"].T) * (1 - a3 * a3)
    d2 = (d3 @ w["W3"].T) * (1 - a2 * a2)
    d1 = (d2 @ w["W2"].T) * (1 - a1 * a1)
    g = {"W4": a3.T @ d4, "b4": d4.sum(0), "W3": a2.T @ d3, "b3": d3.sum(0), "W2": a1.T @ d2, "b2": d2.sum(0),
         "W1": X.T @ d1, "b1": d1.sum(0)}
    out = np.zeros(NPARAMS)
    for k, (o, n_) in LAYOUT.items():
        out[o:o + n_] = g[k].ravel()
    return out, loss
