"""Test infrastructure only: an FP64 restatement of the cost model's network.

The library's tuner trains a multilayer perceptron with its own CUDA kernels
(compute.scala_gb300/csrc/mlp.cu).  This module computes the same forward pass,
mean-squared-error loss, gradients and Adam update in float64 with numpy, so the
tests can check the kernels' gradients and steps.  It is pinned against central
finite differences in tests/test_tuner.py.  The network has no counterpart in
the reference (which has no tuner).

Parameter layout (shared with the kernels): for each layer, W (inputs x
outputs, row-major) then b.  Hidden layers apply ReLU; the last is linear.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def unpack(params: np.ndarray, dims: Sequence[int]) -> List[Tuple[np.ndarray, np.ndarray]]:
    out, off = [], 0
    for k, n in zip(dims[:-1], dims[1:]):
        w = params[off:off + k * n].reshape(k, n)
        off += k * n
        b = params[off:off + n]
        off += n
        out.append((w, b))
    if off != params.size:
        raise ValueError("parameter count does not match the widths")
    return out


def forward(params: np.ndarray, dims: Sequence[int], x: np.ndarray):
    """Returns the output (batch,) and the activations [x, h_1, ..., h_L]."""
    layers = unpack(np.asarray(params, dtype=np.float64), dims)
    h = np.asarray(x, dtype=np.float64)
    acts = [h]
    for i, (w, b) in enumerate(layers):
        h = h @ w + b
        if i < len(layers) - 1:
            h = np.maximum(h, 0.0)
        acts.append(h)
    return h[:, 0], acts


def loss_and_gradients(params: np.ndarray, dims: Sequence[int], x: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient with respect to every parameter."""
    y, acts = forward(params, dims, x)
    t = np.asarray(t, dtype=np.float64)
    n = y.shape[0]
    e = y - t
    loss = float(np.mean(e * e))
    layers = unpack(np.asarray(params, dtype=np.float64), dims)
    delta = (2.0 / n) * e[:, None]
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        w, _ = layers[l]
        gw = acts[l].T @ delta
        gb = delta.sum(axis=0)
        grads.append((gw, gb))
        if l > 0:
            delta = (delta @ w.T) * (acts[l] > 0.0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return loss, flat


def adam_step(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015) with bias correction; returns (params, m, v)."""
    m = beta1 * m + (1.0 - beta1) * grads
    v = beta2 * v + (1.0 - beta2) * grads * grads
    c1 = 1.0 - beta1 ** step
    c2 = 1.0 - beta2 ** step
    params = params - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return params, m, v
