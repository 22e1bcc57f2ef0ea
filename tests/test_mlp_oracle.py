"""The CPU restatement of the relaxation network (oracle/mlp.py) checked on its own.

Its analytic gradient is compared with central finite differences (weights
taken as exact, no bf16 rounding, so the loss is smooth in them), and its bf16
rounding with a bit-level definition of round-to-nearest-even.  The GPU
kernels are then checked against this oracle (tests/test_gpu_learn.py).
"""
from __future__ import annotations

import numpy as np

from oracle import mlp as om


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.3e-5, 65504.0, 1e-30], np.float32)
    r = om.bf16(x)
    assert np.all(r.view(np.uint32) & 0xFFFF == 0)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)  # ties to even, then up
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8 + 1e-45)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.3, om.NPARAM).astype(np.float64)
    norm = np.concatenate([rng.normal(0, 1, 12), rng.uniform(0.5, 2, 12)])
    X = rng.normal(0, 1, (40, 12))
    T = rng.normal(0, 1, (40, 2))
    M = rng.uniform(0.2, 1, (40, 2))
    _, g = om.loss_grad(p, norm, X, T, M, quantize=False)

    def f(q):
        o, _ = om.forward(q, norm, X, quantize=False)
        return float((M * (o - T) ** 2).sum() / len(X))

    idx = rng.choice(om.NPARAM, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (f(p + e) - f(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
