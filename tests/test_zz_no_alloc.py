"""The allocation-free residual norm (cfd_residual_norm_noalloc).

Callers such as a host solver that reserves all device memory at start-up, a
host whose own pool owns the device, or a time loop being captured into a CUDA
graph cannot call cudaMalloc while they step; this entry point reduces a
caller-owned device array using only a static device scratch array.  The test
calls it through the C ABI on two consecutive steps and checks each result
against the case-based norm (cfd_residual_norm), within the 1e-12 relative
tolerance the residual tests use.  It lives in its own file, collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, golden, manifest

pytestmark = pytest.mark.gpu


def _fn(lib):
    f = lib.cfd_residual_norm_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_norm_matches_case_norm(built_lib):
    import torch

    from tmp_gb300 import abi

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    mesh = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    case = abi.Case([mesh], [dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])], abi.FLOW_LAMINAR,
                    abi.ADV_LUSGS, abi.PREC_FP64, cfl=c["cfl"])
    case.put("U", g["init_U"])
    f = _fn(abi.lib())
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row, each after a fresh step
        case.step(1)
        want = case.norm("DW_RHO2")
        dw = torch.from_numpy(case.get("DW").copy()).cuda()
        rc = f(dw.data_ptr(), mesh.ncell, 0, out.data_ptr(), None)
        assert rc == 0, abi.lib().cfd_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        assert want > 0
        assert abs(got - want) <= 1e-12 * abs(want), (call, got, want)
        want_l2 = case.norm("L2_R_RHO")
        r = torch.from_numpy(case.get("R").copy()).cuda()
        rc = f(r.data_ptr(), mesh.ncell, 2, out.data_ptr(), None)
        assert rc == 0, abi.lib().cfd_last_error()
        torch.cuda.synchronize()
        assert abs(float(out.item()) - want_l2) <= 1e-12 * abs(want_l2)


def test_noalloc_rejects_oversize_and_bad_args(built_lib):
    import torch

    from tmp_gb300 import abi

    f = _fn(abi.lib())
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # rejected before any launch: the record count is above the static array's limit
    rc = f(buf.data_ptr(), 33554433, 0, out.data_ptr(), None)
    assert rc == -1
    assert b"limit" in abi.lib().cfd_last_error()
    assert f(buf.data_ptr(), 2, 1, out.data_ptr(), None) == -1   # RK norm needs two arrays
    assert f(None, 2, 0, out.data_ptr(), None) == -1
