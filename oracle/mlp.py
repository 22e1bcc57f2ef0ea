"""CPU restatement of the learned-relaxation network, for gradient checks.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Same network as the CUDA
kernels in tmp_gb300/csrc/k_mlp.cu: x^ = (x - mean) * scale, h1 = relu(W1 x^ +
b1), h2 = relu(W2 h1 + b2), o = W3 h2 + b3, with the weight matrices rounded to
bf16 (round to nearest even) and everything else in binary64.  The loss is
(1/n) sum_i sum_o m_io (o_io - t_io)^2 and the gradient is taken with respect
to the rounded weights.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 12, 64, 2
SIZES = [("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)  # finite inputs
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n]).reshape(shape)
        o += n
    return out


def forward(p, norm, X, quantize: bool = True):
    w = unpack(p)
    q = bf16 if quantize else (lambda a: a)
    W1, W2, W3 = (q(w[k]).astype(np.float64) for k in ("W1", "W2", "W3"))
    b1, b2, b3 = (w[k].astype(np.float64) for k in ("b1", "b2", "b3"))
    xh = (np.asarray(X, np.float64) - norm[:NI].astype(np.float64)) * norm[NI:].astype(np.float64)
    a1 = xh @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    o = h2 @ W3.T + b3
    return o, (xh, h1, h2, W2, W3)


def loss_grad(p, norm, X, T, M=None, quantize: bool = True):
    n = len(X)
    o, (xh, h1, h2, W2, W3) = forward(p, norm, X, quantize)
    m = np.ones_like(o) if M is None else np.asarray(M, np.float64)
    e = o - np.asarray(T, np.float64)
    loss = float((m * e * e).sum() / n)
    do = 2.0 * m * e / n
    g2 = (do @ W3) * (h2 > 0)
    g1 = (g2 @ W2) * (h1 > 0)
    grads = [g1.T @ xh, g1.sum(0), g2.T @ h1, g2.sum(0), do.T @ h2, do.sum(0)]
    return loss, np.concatenate([g.reshape(-1) for g in grads])
