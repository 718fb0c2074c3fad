"""CPU restatement of the learned test-ordering network (test infrastructure only).

The GPU engine ranks each particle's in-range neighbours with a 13 -> 64 -> 64 -> 1 ReLU
network (rampack_gb300/csrc/rp_mlp.cuh) so that its move sweep can pre-test the partners
most likely to overlap.  rampack itself has no such ordering: it tests a mover against
its neighbour-grid cells in cell order (Packing::countParticleOverlaps,
core/Packing.cpp:373-430), so this module has no reference counterpart to follow and the
decisions it could change are pinned elsewhere (the ordered sweep's states equal the
plain sweep's).  What it pins is the network arithmetic itself:

* ``forward``: BF16 rounding of every layer input and weight (the tensor-core operands),
  biases in FP32, ReLU, the hidden layer rounded to BF16 before layer 2 and layer 3;
* ``loss_and_grad``: mean binary cross-entropy on the logits and its gradient with the
  BF16 roundings passed straight through (what the training kernels compute);
* the backward formulas are checked against finite differences of ``forward`` with the
  roundings off.

Parameter layout (FP32 vector of 5313): W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
from __future__ import annotations

import numpy as np

IN, H, FEATURES = 16, 64, 13
W1, B1 = 0, H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
NPARAM = B3 + 1
assert NPARAM == 5313


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(w, dtype=np.float32):
    w = np.asarray(w, dtype=dtype)
    return (w[W1:B1].reshape(H, IN), w[B1:W2], w[W2:B2].reshape(H, H), w[B2:W3], w[W3:B3], w[B3])


def features(d, ai, aj, inv_range) -> np.ndarray:
    """Pair features: d / range, the two unit axes, |d|^2, ai.aj, d.ai, d.aj (FP32), 3 zeros."""
    d = np.asarray(d, dtype=np.float32) * np.float32(inv_range)
    ai = np.asarray(ai, dtype=np.float32)
    aj = np.asarray(aj, dtype=np.float32)
    f = np.zeros(d.shape[:-1] + (IN,), dtype=np.float32)
    f[..., 0:3] = d
    f[..., 3:6] = ai
    f[..., 6:9] = aj
    f[..., 9] = (d * d).sum(-1)
    f[..., 10] = (ai * aj).sum(-1)
    f[..., 11] = (d * ai).sum(-1)
    f[..., 12] = (d * aj).sum(-1)
    return f


def forward(feats, w, rounding: bool = True):
    """Logits (float64) and the activations the backward pass needs."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(w, np.float32 if rounding else np.float64)
    x = r(feats).astype(np.float64)
    s1 = x @ r(w1).astype(np.float64).T + b1
    h1 = np.where(s1 > 0, s1, 0.0)
    if rounding:
        h1 = bf16(h1.astype(np.float32)).astype(np.float64)
    s2 = h1 @ r(w2).astype(np.float64).T + b2
    h2 = np.where(s2 > 0, s2, 0.0)
    h2r = bf16(h2.astype(np.float32)).astype(np.float64) if rounding else h2
    y = h2r @ r(w3).astype(np.float64) + float(b3)
    return y, (x, h1, h2, h2r)


def loss(feats, labels, w, rounding: bool = True) -> float:
    y, _ = forward(feats, w, rounding)
    lab = np.asarray(labels, dtype=np.float64)
    return float(np.mean(np.maximum(y, 0) - y * lab + np.log1p(np.exp(-np.abs(y)))))


def loss_and_grad(feats, labels, w, rounding: bool = True):
    """Mean BCE-with-logits and its gradient (float64, layout of the parameter vector)."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(w, np.float32 if rounding else np.float64)
    y, (x, h1, h2, h2r) = forward(feats, w, rounding)
    n = len(y)
    lab = np.asarray(labels, dtype=np.float64)
    lval = float(np.mean(np.maximum(y, 0) - y * lab + np.log1p(np.exp(-np.abs(y)))))
    dy = (1.0 / (1.0 + np.exp(-y)) - lab) / n
    g = np.zeros(NPARAM, dtype=np.float64)
    w3r = r(w3).astype(np.float64)
    g[W3:B3] = h2r.T @ dy
    g[B3] = dy.sum()
    dh2 = np.where(h2 > 0, dy[:, None] * w3r[None, :], 0.0)
    g[W2:B2] = (dh2.T @ h1).reshape(-1)
    g[B2:W3] = dh2.sum(0)
    dh1 = np.where(h1 > 0, dh2 @ r(w2).astype(np.float64), 0.0)
    g[W1:B1] = (dh1.T @ x).reshape(-1)
    g[B1:W2] = dh1.sum(0)
    return lval, g


def init_params(seed: int) -> np.ndarray:
    """A numpy initialisation of the same shape as the engine's (for tests)."""
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM, dtype=np.float32)
    a1, a2 = np.sqrt(6.0 / FEATURES), np.sqrt(6.0 / H)
    w1 = rng.uniform(-a1, a1, (H, IN)).astype(np.float32)
    w1[:, FEATURES:] = 0
    w[W1:B1] = w1.reshape(-1)
    w[B1:W2] = rng.uniform(-0.1, 0.1, H)
    w[W2:B2] = rng.uniform(-a2, a2, H * H)
    w[B2:W3] = rng.uniform(-0.1, 0.1, H)
    w[W3:B3] = rng.uniform(-a2, a2, H)
    w[B3] = 0.05
    return w
