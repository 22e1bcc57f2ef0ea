"""The learned relaxation on the GPU: the network's kernels against the CPU
oracle (oracle/mlp.py), training, the features of a case, and the gain of the
trained network over the plain LU-SGS update on held-out cases.

Tolerances: the kernels accumulate in fp32 (fused multiply-add) while the
oracle sums in binary64 with the same bf16-rounded weights, so outputs agree
to 1e-5 relative and gradients to 1e-4 relative in norm.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp as om

pytestmark = pytest.mark.gpu


def _net(abi, seed=3):
    rng = np.random.default_rng(seed)
    m = abi.Mlp(seed)
    p, _ = m.params()
    p[-2:] = rng.normal(0, 1, 2)
    norm = np.concatenate([rng.normal(0, 1, 12), rng.uniform(0.5, 2, 12)]).astype(np.float32)
    m.set_params(p, norm)
    return m, p, norm


def test_forward_and_gradient_match_oracle(built_lib):
    import torch

    from tmp_gb300 import abi

    m, p, norm = _net(abi)
    rng = np.random.default_rng(1)
    n = 5000
    X = rng.normal(0, 2, (n, 12)).astype(np.float32)
    T = rng.normal(0, 1, (n, 2)).astype(np.float32)
    M = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    dx, dt, dm = (torch.tensor(a, device="cuda") for a in (X, T, M))
    dy = torch.empty(2 * n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    m.forward(dx.data_ptr(), n, dy.data_ptr())
    torch.cuda.synchronize()
    o_ref, _ = om.forward(p, norm, X)
    y = dy.cpu().numpy().reshape(n, 2)
    assert np.max(np.abs(y - o_ref)) <= 1e-5 * max(1.0, np.abs(o_ref).max())
    loss, g = m.loss_grad(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), n)
    lref, gref = om.loss_grad(p, norm, X, T, M)
    assert abs(loss - lref) <= 1e-5 * lref
    assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)
    # the gradient is a fixed-order sum: bitwise repeatable
    _, g2 = m.loss_grad(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), n)
    assert np.array_equal(g, g2)


def test_training_fits_a_teacher(built_lib):
    import torch

    from tmp_gb300 import abi

    teacher, _, _ = _net(abi, seed=11)
    rng = np.random.default_rng(2)
    n = 20000
    X = rng.normal(0, 1, (n, 12)).astype(np.float32)
    dx = torch.tensor(X, device="cuda")
    dt = torch.empty(2 * n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    teacher.forward(dx.data_ptr(), n, dt.data_ptr())
    student = abi.Mlp(5)
    p, _ = student.params()
    student.set_params(p, np.concatenate([np.zeros(12), np.ones(12)]).astype(np.float32))
    torch.cuda.synchronize()
    l0, _ = student.loss_grad(dx.data_ptr(), dt.data_ptr(), None, n)
    hist = student.train(dx.data_ptr(), dt.data_ptr(), None, n, 600, 2048, 3e-3, seed=4)
    l1, _ = student.loss_grad(dx.data_ptr(), dt.data_ptr(), None, n)
    assert np.all(np.isfinite(hist)) and l1 < 0.1 * l0


def test_case_features_and_learned_step(built_lib):
    import torch

    from tmp_gb300 import abi, learn

    spec = learn.CaseSpec(nbody=48, nlayer=10, seed=3)
    mesh = spec.mesh()
    case = spec.case(mesh)
    abi.case_track(case, True)
    case.step_graph(30)
    nc = case.ncell
    f = torch.empty(nc * 12, dtype=torch.float32, device="cuda")
    case.sync()
    abi.case_features(case, f.data_ptr())
    case.sync()
    X = f.view(nc, 12).cpu().numpy()
    assert np.isfinite(X).all()
    # features 10 and 11 are rho - 1 and p - 1 of the state
    U = case.get("U")
    assert np.allclose(X[:, 10], U[:, 0] - 1, atol=1e-6) and np.allclose(X[:, 11], U[:, 1] - 1, atol=1e-6)
    # an untrained network relaxes by ~1.04: the learned step stays close to the plain one
    plain = spec.case(mesh)
    plain.put("U", U)
    case.put("U", U)
    m = abi.Mlp(0)
    abi.case_set_mlp(case, m)
    case.step(1)
    plain.step(1)
    a, b = case.get("U"), plain.get("U")
    abi.case_set_mlp(case, None)
    assert np.isfinite(a).all() and np.max(np.abs(a - b)) < 0.2 * np.max(np.abs(b - U)) + 1e-12
