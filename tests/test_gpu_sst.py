"""SST k-omega kernels against the reference's own SST functions.

tests/golden/{mixed,omesh}_lam_sst.npz were dumped by the compiled reference
(oracle/ref_driver.cpp, SST phase): one laminar residual from a perturbed
state, then SolveTurbulenceEquation, SolveDiag and UpdatePrimitiveVariables on
non-uniform k, omega and mu_t.  The GPU evaluates the same functions from the
same inputs.  Tolerance 1e-12 relative (the residual bound): the flow inputs
(face viscosity, far-field states) carry pow()'s last-bit differences and F1 /
F2 tanh's; the face values, gradients and fluxes that depend on neither are
also checked bit for bit.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = {"mixed_lam_sst": ("mixed.grd", 0.4, 5.0, 1000.0), "omesh_lam_sst": ("omesh.grd", 0.2, 0.0, 40.0)}


def _close(a, b, rtol=1e-12):
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    scale = np.maximum(np.abs(b), np.abs(b).max() * 1e-3)
    return np.max(np.abs(a - b) / scale) <= rtol


@pytest.mark.parametrize("name", list(CASES))
def test_sst_residual_matches_reference(built_lib, name):
    from tmp_gb300 import abi

    mesh_file, ma, aoa, re = CASES[name]
    g = np.load(GOLDEN / f"{name}.npz")
    mesh = abi.Mesh.load_grd(GOLDEN / mesh_file, -1, -2)
    case = abi.Case([mesh], [dict(mach=ma, aoa_deg=aoa, reynolds=re)], abi.FLOW_LAMINAR, abi.ADV_LUSGS,
                    abi.PREC_FP64, cfl=50.0)
    case.put("U", g["init_U"])
    case.residual(0)
    case.local_dt(50.0)
    assert _close(case.get("DT"), g["res0_dt"])
    inf = abi.sst_enable(case)
    assert np.array_equal(inf, g["sst_inf"])  # InitializeturbulenceVariable, bit for bit
    assert np.array_equal(case.get("SST_T").reshape(-1), np.repeat(inf[None, :2], mesh.ncell, 0).reshape(-1))
    case.put("SST_T", g["sst_T_in"])
    case.put("SST_MUT", g["sst_mut_in"])
    abi.sst_residual(case)
    for field, key in (("SST_TFACE", "sst_tface"), ("SST_TGRAD", "sst_tgrad"), ("SST_F1", "sst_f1"),
                       ("SST_F2", "sst_f2"), ("SST_MUTF", "sst_mutf"), ("SST_FCONV", "sst_fconv"),
                       ("SST_FVISC", "sst_fvisc"), ("SST_R", "sst_R"), ("SST_DIAG", "sst_diag")):
        assert _close(case.get(field), g[key]), field
    # k face values and their gradient involve no pow / tanh: bit for bit
    tf = case.get("SST_TFACE").reshape(-1, 2)
    assert np.array_equal(tf[:, 0], g["sst_tface"].reshape(-1, 2)[:, 0])
    assert np.array_equal(case.get("SST_TGRAD").reshape(-1, 4)[:, :2], g["sst_tgrad"].reshape(-1, 4)[:, :2])
    abi.sst_update_mut(case)
    assert np.array_equal(case.get("SST_T").reshape(-1), g["sst_T2"])
    assert _close(case.get("SST_MUT"), g["sst_mut"])
    # the blending functions span both regimes on these states
    f1 = case.get("SST_F1")
    assert f1.min() < 0.5 < f1.max()
