"""FP64 numpy restatement of the warm-start network (TEST INFRASTRUCTURE ONLY).

The network has no counterpart in the reference; this is the CPU gradient
oracle its CUDA forward/backward kernels are checked against.  Same layout as
the library: layers (4->64, d1), (64->64, d2), (64->64, d4), (64->1, d8),
kernel 5, zero padding, tanh on hidden layers, parameters flattened as each
layer's weights [co][ci][k] followed by its bias [co].
"""
from __future__ import annotations

import numpy as np

GRID = 256
K = 5
LAYERS = [(5, 64, 1, True), (64, 64, 2, True), (64, 64, 4, True), (64, 1, 8, False)]
SCALE = 5.0


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    out, off = [], 0
    for ci, co, d, act in LAYERS:
        W = p[off:off + co * ci * K].reshape(co, ci, K)
        off += co * ci * K
        b = p[off:off + co]
        off += co
        out.append((W, b, d, act))
    assert off == p.size
    return out


def _shifted(x, d):
    xp = np.pad(x, ((0, 0), (0, 0), (2 * d, 2 * d)))
    return [xp[:, :, k * d:k * d + GRID] for k in range(K)]


def forward(params, features):
    """features (B, 5, 256) -> output (B, 256) and the activations."""
    acts = [np.asarray(features, dtype=np.float64)]
    for W, b, d, act in unpack(params):
        xs = _shifted(acts[-1], d)
        y = sum(np.einsum("oc,bcp->bop", W[:, :, k], xs[k]) for k in range(K)) + b[None, :, None]
        acts.append(np.tanh(y) if act else y)
    return acts[-1][:, 0, :], acts


def loss_grad(params, features, targets):
    out, acts = forward(params, features)
    t = np.asarray(targets, dtype=np.float64)
    n = out.size
    loss = float(np.mean((out - t) ** 2))
    g = (2.0 * (out - t) / n)[:, None, :]
    layers = unpack(params)
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, b, d, act = layers[li]
        x = acts[li]
        xs = _shifted(x, d)
        gW = np.stack([np.einsum("bop,bcp->oc", g, xs[k]) for k in range(K)], axis=2)
        gb = g.sum(axis=(0, 2))
        grads.append((gW, gb))
        if li > 0:
            gxp = np.zeros((x.shape[0], x.shape[1], GRID + 4 * d))
            for k in range(K):
                gxp[:, :, k * d:k * d + GRID] += np.einsum("oc,bop->bcp", W[:, :, k], g)
            gx = gxp[:, :, 2 * d:2 * d + GRID]
            g = gx * (1.0 - x ** 2)  # x = tanh activation of the previous layer
    flat = []
    for gW, gb in reversed(grads):
        flat += [gW.ravel(), gb]
    return loss, np.concatenate(flat)


def features(x, f0, nsteps, w=None):
    """Network input of one instance (5, 256) and the target w/5 on the grid: the
    grid coordinate, L, log2 of the contour steps, log f0 on the grid and the log
    of the mean element length."""
    x = np.asarray(x, dtype=np.float64)
    L = x[-1] - x[0]
    u = np.arange(GRID) / (GRID - 1)
    xq = x[0] + u * L
    fq = np.interp(xq, x, f0)
    f = np.stack([2 * u - 1, np.full(GRID, (L - 6.0) / 4.0), np.full(GRID, (np.log2(nsteps) - 10.5) / 1.5),
                  np.log(np.maximum(fq, 1e-8)) / 10.0, np.full(GRID, np.log(L / (len(x) - 1)) + 3.7)])
    t = None if w is None else np.interp(xq, x, w) / SCALE
    return f, t
