"""The MIXFF form: the residual in float-float pairs, the rest as the mixed form.

Its residual passes are the same kernels as the binary64 residual, instantiated
on hi + lo pairs of binary32 numbers (48-bit significands, sums and products
within about 2^-46, quotients 2^-44; tests/test_ff_arith.py pins the arithmetic
on the host).  So every residual-phase array agrees with the reference's
binary64 dumps to FF_RES_TOL normwise, steps agree with the mixed form (same
binary32 sweep, same binary64 update) to FF_FIELD_TOL, and a long run follows
the mixed form's residual history.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, golden, manifest
from test_gpu_parity import make_case, rel

pytestmark = pytest.mark.gpu

CASES = list(manifest())
FF_RES_TOL = 1e-11
FF_FIELD_TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("name", CASES)
def test_mixff_residual_phase(name):
    """Every residual-phase array of the float-float residual against the
    reference's binary64 dump of the same state."""
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    _, case = make_case(c, precision=abi.PREC_MIXFF)
    case.put("U", g["init_U"])
    case.residual()
    case.sync()
    pairs = [("R", "res0_R"), ("UEDGE", "res0_Uedge"), ("GRAD", "res0_grad"), ("PHI", "res0_phi"),
             ("SPEC_C", "res0_specc")]
    if c["flow"] == "viscous":
        pairs += [("GRADT", "res0_gradT"), ("SPEC_V", "res0_specv"), ("MU", "res0_mu"), ("MUEDGE", "res0_muedge")]
    errs = {fld: rel(case.get(fld), g[key]) for fld, key in pairs}
    cfl = c["cfl"] if c["advance"] == "lusgs" else 0.8
    case.local_dt(cfl)
    errs["DT"] = rel(case.get("DT"), g["res0_dt"])
    bad = {k: v for k, v in errs.items() if not v <= FF_RES_TOL}
    assert not bad, f"normwise errors above {FF_RES_TOL}: {bad} (all: {errs})"
    case.close()


@pytest.mark.parametrize("name", [n for n in CASES if manifest()[n]["advance"] == "lusgs"])
def test_mixff_steps_follow_mixed(name):
    """LU-SGS steps: the same binary32 sweep and binary64 update as the mixed
    form, so the two differ only by the residual's rounding."""
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    out = {}
    for prec in (abi.PREC_MIXED, abi.PREC_MIXFF):
        _, case = make_case(c, precision=prec)
        case.put("U", g["init_U"])
        hist = []
        for _ in range(c["nsteps"]):
            case.step(1)
            hist.append(case.norm("DW_RHO2"))
        case.sync()
        out[prec] = (case.get("U"), case.get("R"), np.array(hist))
        case.close()
    (u0, r0, h0), (u1, r1, h1) = out[abi.PREC_MIXED], out[abi.PREC_MIXFF]
    assert rel(u1, u0) <= FF_FIELD_TOL
    assert rel(r1, r0) <= 1e-9
    np.testing.assert_allclose(h1, h0, rtol=1e-8)


@pytest.mark.parametrize("name", [n for n in CASES if manifest()[n]["advance"] == "rk5"])
def test_mixff_rk5_steps_match_reference(name):
    """RK5 with the float-float residual and the binary64 stage updates: within
    FF_FIELD_TOL of the reference's binary64 fields after the fixture's steps."""
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    _, case = make_case(c, precision=abi.PREC_MIXFF)
    case.put("U", g["init_U"])
    case.step(c["nsteps"])
    case.sync()
    assert rel(case.get("U"), g["end_U"]) <= FF_FIELD_TOL
    case.close()


def _cylinder():
    from tmp_gb300 import learn

    spec = learn.CaseSpec(nbody=96, nlayer=24, seed=12, dr1=5e-3, growth=1.05, rfar=30.0)
    return spec.mesh(), dict(mach=spec.mach, aoa_deg=spec.aoa, reynolds=spec.re)


@pytest.mark.parametrize("sweep_mode", [0, 5, 6])
def test_mixff_long_run_follows_mixed(sweep_mode):
    """600 graph-replayed LU-SGS steps from the freestream on a ~25k-cell
    cylinder mesh: the residual history and the final state of the MIXFF form
    stay on the mixed form's."""
    from tmp_gb300 import abi

    mesh, fs = _cylinder()
    res = {}
    for prec in (abi.PREC_MIXED, abi.PREC_MIXFF):
        case = abi.Case([mesh], [fs], abi.FLOW_LAMINAR, abi.ADV_LUSGS, prec, cfl=50.0, sweep_mode=sweep_mode)
        case.init_freestream()
        hist = []
        for _ in range(12):
            case.step_graph(50)
            hist.append(case.norm("L2_R_RHO"))
        case.sync()
        res[prec] = (case.get("U"), np.array(hist))
        case.close()
    (u0, h0), (u1, h1) = res[abi.PREC_MIXED], res[abi.PREC_MIXFF]
    assert np.all(np.isfinite(u1))
    np.testing.assert_allclose(h1, h0, rtol=1e-6)
    assert rel(u1, u0) <= 1e-8


def test_mixff_wall_force_matches_binary64():
    from tmp_gb300 import abi

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    f = {}
    for prec in (abi.PREC_FP64, abi.PREC_MIXFF):
        _, case = make_case(c, precision=prec)
        case.put("U", g["init_U"])
        f[prec] = case.wall_force()
        case.close()
    a, b = f[abi.PREC_MIXFF], f[abi.PREC_FP64]
    scale = max(abs(b["fx"]), abs(b["fy"]))
    assert abs(a["fx"] - b["fx"]) <= 1e-11 * scale and abs(a["fy"] - b["fy"]) <= 1e-11 * scale


def test_switch_from_fp32_to_mixff_follows_mixed():
    """A binary32-form case switched to MIXFF continues as the same case
    switched to the mixed form would (to 1e-8 normwise: the 80 steps from an
    impulsive start are a strong transient that amplifies the 1e-14 residual
    differences)."""
    from tmp_gb300 import abi

    mesh, fs = _cylinder()
    out = {}
    for target in (abi.PREC_MIXED, abi.PREC_MIXFF):
        case = abi.Case([mesh], [fs], abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_FP32, cfl=50.0, sweep_mode=5)
        case.init_freestream()
        case.step_graph(40)
        case.set_precision(target)
        case.step_graph(40)
        case.sync()
        out[target] = case.get("U")
        case.close()
    assert rel(out[abi.PREC_MIXFF], out[abi.PREC_MIXED]) <= 1e-8


def test_mixff_learned_relaxation_runs():
    """The learned update reads the float-float residual arrays' high parts as
    its features and runs on the MIXFF form.  It is not the mixed form's
    learned update to rounding: one feature is log10(|R_rho| dt / (vol rho)),
    and in cells still at the freestream |R_rho| is the residual's rounding
    floor — near 1e-17 in binary64, near 1e-14 in float-float — so those cells'
    features differ by about three decades and the pooled factor moves with
    them.  After 20 learned steps the two states agree to 5e-3 normwise."""
    from tmp_gb300 import abi, learn

    net = learn.load()
    if net is None:
        pytest.skip("no committed relaxation weights")
    mesh, fs = _cylinder()
    out = {}
    for prec in (abi.PREC_MIXED, abi.PREC_MIXFF):
        case = abi.Case([mesh], [fs], abi.FLOW_LAMINAR, abi.ADV_LUSGS, prec, cfl=50.0)
        case.init_freestream()
        case.step_graph(30)
        abi.case_track(case, True)
        abi.case_set_mlp(case, net, False)
        case.step_graph(20)
        case.sync()
        out[prec] = case.get("U")
        abi.case_set_mlp(case, None)
        case.close()
    assert np.all(np.isfinite(out[abi.PREC_MIXFF]))
    assert rel(out[abi.PREC_MIXFF], out[abi.PREC_MIXED]) <= 5e-3


def test_mixff_refuses_what_it_does_not_run():
    """Sweep modes 1 and 2 (per-level launches that read a binary64 viscosity)
    and the SST model (binary64 residual arrays) are refused for MIXFF."""
    from tmp_gb300 import abi

    c = manifest()["mixed_lam_lusgs"]
    m = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    fs = [dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])]
    for mode in (1, 2):
        with pytest.raises(abi.CfdError):
            abi.Case([m], fs, abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_MIXFF, cfl=c["cfl"], sweep_mode=mode)
    case = abi.Case([m], fs, abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_MIXFF, cfl=c["cfl"])
    with pytest.raises(abi.CfdError):
        abi.sst_enable(case)
    case.close()
    case = abi.Case([m], fs, abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_MIXED, cfl=c["cfl"], sweep_mode=1)
    with pytest.raises(abi.CfdError):
        case.set_precision(abi.PREC_MIXFF)
    case.close()
