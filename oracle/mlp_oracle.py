"""fp64 restatements of the schedule-search pieces, for tests only.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker, never by the
product.

* the MLP cost model (dense tanh layers, one linear output, mean-squared
  error, Adam): forward pass, backpropagated gradient and one Adam step, in
  float64 with the library's flat parameter layout -- for each layer l
  (din -> dout) the weights W_l (dout x din, row-major) then the bias b_l;
* the reference's analytic tiling objective ``objective2D``
  (include/PSkelStencil.hpp:1883-1895) and the phenotype bounds of
  ``solve2D`` (include/PSkelStencil.hpp:1897-1913), with the memory budget a
  parameter.
"""
from __future__ import annotations

import math

import numpy as np


def dims_of(in_dim: int, hidden: int, layers: int):
    return [in_dim] + [hidden] * (layers - 1) + [1]


def num_params(dims) -> int:
    return sum(dims[l] * dims[l + 1] + dims[l + 1] for l in range(len(dims) - 1))


def unpack(params: np.ndarray, dims):
    p = np.asarray(params, dtype=np.float64)
    out, off = [], 0
    for l in range(len(dims) - 1):
        din, dout = dims[l], dims[l + 1]
        W = p[off:off + din * dout].reshape(dout, din)
        off += din * dout
        b = p[off:off + dout]
        off += dout
        out.append((W, b))
    assert off == p.size
    return out


def forward(params, X, dims):
    """Activations of every layer (last = linear output, shape (n,))."""
    a = np.asarray(X, dtype=np.float64)
    acts = [a]
    layers = unpack(params, dims)
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = np.tanh(z) if l < len(layers) - 1 else z
        acts.append(a)
    return acts


def predict(params, X, dims):
    return forward(params, X, dims)[-1][:, 0]


def loss(params, X, y, dims) -> float:
    e = predict(params, X, dims) - np.asarray(y, dtype=np.float64)
    return float(np.mean(e * e))


def gradient(params, X, y, dims):
    """(flat gradient of mean((yhat - y)^2), loss) by backpropagation."""
    acts = forward(params, X, dims)
    layers = unpack(params, dims)
    n = acts[0].shape[0]
    e = acts[-1][:, 0] - np.asarray(y, dtype=np.float64)
    delta = (2.0 * e / n)[:, None]
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        if l < len(layers) - 1:
            delta = delta * (1.0 - acts[l + 1] ** 2)
        grads[l] = (delta.T @ acts[l], delta.sum(axis=0))
        delta = delta @ W
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return flat, float(np.mean(e * e))


def adam(params, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return params - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def objective2d(h: float, it: float, width: float, height: float, iterations: float, rng: int, type_size: float,
                mem_free: float, depth: float = 1.0) -> float:
    """objective2D (include/PSkelStencil.hpp:1883-1895); tileHeight is a size_t there."""
    tile_h = float(math.floor(min(height, 2 * it * rng + h)))
    if 2 * (width * depth * tile_h * type_size) > mem_free:
        return 0.0
    return (h / tile_h) * ((it * h) / (height * iterations))


def max_height(width, height, type_size, mem_free, depth=1.0) -> int:
    """solve2D's phenotype bound for h (include/PSkelStencil.hpp:1903-1904)."""
    div = (2.0 * (width * depth * height * type_size)) / (mem_free * 1.1)
    return max(1, math.ceil(height / div))
