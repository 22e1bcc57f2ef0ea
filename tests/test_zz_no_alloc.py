"""The allocation-free residual norm (cfd_residual_norm_noalloc).

Callers such as a host solver that reserves all of its device memory at
start-up, or a host whose own memory pool owns the device, cannot call
cudaMalloc while they step; this entry point reduces a caller-owned device
array using only a static device scratch array.  The tests call it through the
C ABI: on two consecutive steps against the case-based norm
(cfd_residual_norm), on arrays of several chunks (the last one partly full)
and at the record limit against a float64 sum, all within the 1e-12 relative
tolerance the residual tests use, and check that calls after the first leave
the device's free memory unchanged.  They live in their own file, collected
last.
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


CHUNK = 8192          # records per partial sum in k_noalloc.cu
LIMIT = 4096 * CHUNK  # records the static scratch array can serve


def test_noalloc_several_chunks_and_limit(built_lib):
    """Several partial sums, a partly full last chunk and the largest accepted
    size, against float64 sums of the same records."""
    import torch

    from tmp_gb300 import abi

    f = _fn(abi.lib())
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(7)
    for n in (1, CHUNK, CHUNK + 1, 3 * CHUNK + 17, 37 * CHUNK - 5):
        rec = rng.standard_normal((n, 4))
        d = torch.from_numpy(rec).cuda()
        for which, want in ((0, float(np.sum(rec[:, 0] ** 2))), (2, float(np.sqrt(np.sum(rec[:, 0] ** 2) / n)))):
            assert f(d.data_ptr(), n, which, out.data_ptr(), None) == 0, abi.lib().cfd_last_error()
            torch.cuda.synchronize()
            assert abs(float(out.item()) - want) <= 1e-12 * want, (n, which)
    # the limit itself (1 GiB of records) is accepted; one record more is not
    big = torch.empty((LIMIT, 4), dtype=torch.float64, device="cuda")
    big[:, 0].uniform_(-1.0, 1.0, generator=torch.Generator(device="cuda").manual_seed(11))
    want = float((big[:, 0] * big[:, 0]).sum())
    assert f(big.data_ptr(), LIMIT, 0, out.data_ptr(), None) == 0, abi.lib().cfd_last_error()
    torch.cuda.synchronize()
    assert abs(float(out.item()) - want) <= 1e-12 * want
    assert f(big.data_ptr(), LIMIT + 1, 0, out.data_ptr(), None) == -1
    del big
    torch.cuda.empty_cache()


def test_noalloc_calls_allocate_nothing(built_lib):
    """After a first call (which looks up the scratch array's address and
    loads the kernels), further calls leave the device's free memory as it
    was: nothing is allocated per call."""
    import torch

    from tmp_gb300 import abi

    f = _fn(abi.lib())
    rec = torch.rand((3 * CHUNK + 17, 4), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert f(rec.data_ptr(), rec.shape[0], 0, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for which in (0, 2, 0, 2):
        assert f(rec.data_ptr(), rec.shape[0], which, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
