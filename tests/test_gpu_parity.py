"""GPU parity of the CUDA path (through the C ABI) against the reference.

Fixtures in tests/golden/ were dumped by the reference's own serial code; the
larger cases compare against the C oracle (oracle/cfd_oracle.c), itself pinned
bit for bit to those fixtures by test_oracle_golden.py.

Tolerances (the benchmark spec): residual-phase arrays 1e-12 relative, fields after
steps 1e-10 relative, both normwise (max |a-b| / max |b|).  The binary64 path
reproduces the reference's operation order with -fmad=false, so most arrays
are bit-identical; pow() (far-field Riemann state, Sutherland's law) is the one
libm call whose last bit may differ between CUDA and glibc.
Binary32 form: residual within 5e-4 normwise of the binary64 reference.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, golden, manifest

pytestmark = pytest.mark.gpu

CASES = list(manifest())
RES_TOL = 1e-12
FIELD_TOL = 1e-10
FP32_RES_TOL = 5e-4


def rel(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    assert a.shape == b.shape
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def make_case(c: dict, precision: int | None = None, mesh=None):
    from tmp_gb300 import abi

    m = mesh or abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    flow = abi.FLOW_LAMINAR if c["flow"] == "viscous" else abi.FLOW_EULER
    adv = abi.ADV_LUSGS if c["advance"] == "lusgs" else abi.ADV_RK5
    prec = abi.PREC_FP64 if precision is None else precision
    case = abi.Case([m], [dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])], flow, adv, prec,
                    cfl=c["cfl"], first_order=bool(c["first_order"]))
    return m, case


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("name", CASES)
def test_geometry_bitexact(name):
    c, g = manifest()[name], golden(name)
    _, case = make_case(c)
    for fld, key in [("VOL", "geo_vol"), ("CENTER", "geo_cen"), ("NORMAL", "geo_nrm"), ("AREA", "geo_area"),
                     ("ECENTER", "geo_ecen")]:
        np.testing.assert_array_equal(case.get(fld).ravel(), g[key], err_msg=fld)


@pytest.mark.parametrize("name", CASES)
def test_residual_phase(name):
    c, g = manifest()[name], golden(name)
    _, case = make_case(c)
    case.put("U", g["init_U"])
    case.residual()
    case.sync()
    pairs = [("R", "res0_R"), ("UEDGE", "res0_Uedge"), ("GRAD", "res0_grad"), ("PHI", "res0_phi"),
             ("SPEC_C", "res0_specc"), ("UL", "res0_UL"), ("UR", "res0_UR")]
    if c["flow"] == "viscous":
        pairs += [("GRADT", "res0_gradT"), ("SPEC_V", "res0_specv"), ("MU", "res0_mu"), ("MUEDGE", "res0_muedge")]
    for fld, key in pairs:
        assert rel(case.get(fld), g[key]) <= RES_TOL, fld
    cfl = c["cfl"] if c["advance"] == "lusgs" else 0.8
    case.local_dt(cfl)
    assert rel(case.get("DT"), g["res0_dt"]) <= RES_TOL


@pytest.mark.parametrize("name", CASES)
def test_steps(name):
    c, g = manifest()[name], golden(name)
    _, case = make_case(c)
    case.put("U", g["init_U"])
    hist = []
    for _ in range(c["nsteps"]):
        case.step(1)
        if c["advance"] == "lusgs":
            hist.append(case.norm("DW_RHO2"))
    case.sync()
    assert rel(case.get("U"), g["end_U"]) <= FIELD_TOL
    if c["advance"] == "lusgs":
        assert rel(case.get("DIAG"), g["end_D"][::4]) <= FIELD_TOL
        for fld, key in [("DW1", "end_dW1"), ("DW", "end_dW"), ("W", "end_W"), ("R", "end_R")]:
            assert rel(case.get(fld), g[key]) <= FIELD_TOL, fld
        np.testing.assert_allclose(hist, g["hist"], rtol=1e-9)


@pytest.mark.parametrize("name", CASES)
def test_fp32_form_residual(name):
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    _, case = make_case(c, precision=abi.PREC_FP32)
    case.put("U", g["init_U"])
    case.residual()
    case.sync()
    assert rel(case.get("R"), g["res0_R"]) <= FP32_RES_TOL


def test_graph_replay_equals_eager():
    c = manifest()["mixed_lam_lusgs"]
    g = golden("mixed_lam_lusgs")
    _, a = make_case(c)
    _, b = make_case(c)
    a.put("U", g["init_U"])
    b.put("U", g["init_U"])
    a.step(4)
    b.step_graph(4)
    a.sync()
    b.sync()
    np.testing.assert_array_equal(a.get("U"), b.get("U"))


def test_deterministic_bits():
    c = manifest()["mixed_lam_rk5"]
    g = golden("mixed_lam_rk5")
    out = []
    for _ in range(2):
        _, case = make_case(c)
        case.put("U", g["init_U"])
        case.step(3)
        out.append(case.get("U"))
    np.testing.assert_array_equal(out[0], out[1])


def test_packed_meshes_match_separate():
    """Two meshes packed in one case give the same bits as two separate cases."""
    from tmp_gb300 import abi

    m = manifest()
    c1, c2 = m["omesh_euler_lusgs"], m["mixed_euler_lusgs_sup"]
    g1, g2 = golden("omesh_euler_lusgs"), golden("mixed_euler_lusgs_sup")
    m1 = abi.Mesh.load_grd(GOLDEN / c1["mesh"], c1["wall_tag"], c1["far_tag"])
    m2 = abi.Mesh.load_grd(GOLDEN / c2["mesh"], c2["wall_tag"], c2["far_tag"])
    fs = [dict(mach=c1["mach"], aoa_deg=c1["aoa"], reynolds=c1["re"]),
          dict(mach=c2["mach"], aoa_deg=c2["aoa"], reynolds=c2["re"])]
    packed = abi.Case([m1, m2], fs, abi.FLOW_EULER, abi.ADV_LUSGS, abi.PREC_FP64, cfl=c1["cfl"])
    packed.put("U", g1["init_U"], mesh=0)
    packed.put("U", g2["init_U"], mesh=1)
    packed.step(2)
    for k, (c, g, mm) in enumerate([(c1, g1, m1), (c2, g2, m2)]):
        single = abi.Case([mm], [fs[k]], abi.FLOW_EULER, abi.ADV_LUSGS, abi.PREC_FP64, cfl=c1["cfl"])
        single.put("U", g["init_U"])
        single.step(2)
        np.testing.assert_array_equal(packed.get("U", mesh=k), single.get("U"))


def _oracle_run(topo, mach, aoa, re, viscous, U0, advance, cfl, nsteps):
    import oracle

    o = oracle.Oracle(topo, mach, aoa, re, viscous)
    o.set_U(U0)
    for _ in range(nsteps):
        if advance == "lusgs":
            o.lusgs_step(cfl)
        else:
            o.rk_step()
    return o


@pytest.mark.parametrize("viscous,advance,cfl", [(True, "lusgs", 50.0), (False, "rk5", 0.8)])
def test_larger_mesh_vs_oracle(tmp_path, built_oracle, viscous, advance, cfl):
    """~20k-cell mixed quad/triangle mesh, several steps, against the C oracle."""
    from oracle import grd
    from tmp_gb300 import abi, meshgen

    gm = meshgen.mixed_mesh(meshgen.naca_body(96), nlayer=16, dr1=2e-3, growth=1.15, rfar=8.0, seed=3,
                            density=1.0, grade=1.0)
    path = tmp_path / "m.grd"
    meshgen.write_grd(path, gm)
    topo = grd.read_grd(path, gm.wall_tag, gm.far_tag)
    mesh = abi.Mesh.load_grd(path, gm.wall_tag, gm.far_tag)
    mach, aoa, re = 0.3, 2.0, 500.0
    a = 3.141593 * aoa / 180
    fs = np.array([1.0, 1.0, mach * np.sqrt(1.4) * np.cos(a), mach * np.sqrt(1.4) * np.sin(a)])
    import oracle

    o0 = oracle.Oracle(topo, mach, aoa, re, viscous)
    U0 = meshgen.perturbed_state(gm.ncell, o0.field("CENTER").copy(), fs, amp=0.04, seed=9)
    o = _oracle_run(topo, mach, aoa, re, viscous, U0, advance, cfl, 3)
    case = abi.Case([mesh], [dict(mach=mach, aoa_deg=aoa, reynolds=re)],
                    abi.FLOW_LAMINAR if viscous else abi.FLOW_EULER,
                    abi.ADV_LUSGS if advance == "lusgs" else abi.ADV_RK5, abi.PREC_FP64, cfl=cfl)
    case.put("U", U0)
    case.step(3)
    case.sync()
    assert rel(case.get("U"), o.field("U")) <= FIELD_TOL
    assert rel(case.get("R"), o.field("R")) <= FIELD_TOL


def test_nonphysical_state_is_reported():
    """A negative pressure in the input is reported as CFD_ERR_NONPHYSICAL (no GPU fault)."""
    from tmp_gb300 import abi

    c, g = manifest()["omesh_euler_lusgs"], golden("omesh_euler_lusgs")
    _, case = make_case(c)
    U = g["init_U"].reshape(-1, 4).copy()
    U[10, 1] = -1.0
    case.put("U", U)
    case.step(1)
    with pytest.raises(abi.CfdError) as ei:
        case.norm("DW_RHO2")
    assert ei.value.code in (-6, -5)
    # the handle stays usable after the error is reported
    case.put("U", g["init_U"])
    case.step(1)
    case.norm("DW_RHO2")


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_sweep_schedules_agree_bitwise(mode):
    """The dataflow sweep (default), the two-cells-per-warp dataflow sweep,
    per-level 16-lane and per-level direct sweeps give identical bits: all of
    them keep the reference's dependence exactly."""
    from tmp_gb300 import abi

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    m = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    out = []
    for sm in (0, mode):
        case = abi.Case([m], [dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])], abi.FLOW_LAMINAR,
                        abi.ADV_LUSGS, abi.PREC_FP64, cfl=c["cfl"], sweep_mode=sm)
        case.put("U", g["init_U"])
        case.step(3)
        case.sync()
        out.append((case.get("U"), case.get("DW1"), case.get("DW")))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", ["mixed_lam_lusgs", "omesh_euler_lusgs"])
def test_fp32_form_lusgs_steps(name):
    """Fast form (binary32 fluxes and sweep combination, binary64 update): fields
    after the fixture's steps within 1e-4 of the binary64 reference."""
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    _, case = make_case(c, precision=abi.PREC_FP32)
    case.put("U", g["init_U"])
    case.step(c["nsteps"])
    case.sync()
    assert rel(case.get("U"), g["end_U"]) <= 1e-4


def test_bounded_wait_reports_timeout_and_context_survives():
    """A device wait on a flag nothing sets gives up after its poll limit, the
    host reads CFD_ERR_TIMEOUT, and the same case keeps working (no GPU fault)."""
    from tmp_gb300 import abi

    c, g = manifest()["omesh_euler_lusgs"], golden("omesh_euler_lusgs")
    _, case = make_case(c)
    rc = abi.lib().cfd_selftest_bounded_wait(case.h, 1 << 16)
    assert rc == -7
    case.put("U", g["init_U"])
    case.step(1)
    assert case.norm("DW_RHO2") > 0


def test_graph_replay_dataflow_epochs():
    """Graph replays of the dataflow sweep use fresh epochs each time (the epoch
    lives in device memory): 5 replays equal 5 eager steps bit for bit."""
    c, g = manifest()["omesh_euler_lusgs"], golden("omesh_euler_lusgs")
    _, a = make_case(c)
    _, b = make_case(c)
    a.put("U", g["init_U"])
    b.put("U", g["init_U"])
    a.step(5)
    b.step_graph(5)
    np.testing.assert_array_equal(a.get("U"), b.get("U"))


@pytest.mark.parametrize("name", ["mixed_lam_lusgs", "omesh_euler_rk5", "mixed_euler_lusgs_sup"])
def test_wall_force_and_distance(name, built_oracle):
    """Wall force (CL/CD) against the oracle's wall-face flux sum; wall distance
    bit-exact against the reference's ComputeWallCellDistance dump."""
    import oracle
    from oracle import grd

    c, g = manifest()[name], golden(name)
    _, case = make_case(c)
    np.testing.assert_array_equal(case.get("WALLDIST"), g["geo_wall"])
    case.put("U", g["init_U"])
    f = case.wall_force()
    t = grd.read_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    o = oracle.Oracle(t, c["mach"], c["aoa"], c["re"], c["flow"] == "viscous")
    o.set_U(g["init_U"])
    o.residual(bool(c["first_order"]))
    fo = o.wall_force()
    scale = max(abs(fo[0]), abs(fo[1]))
    assert abs(f["fx"] - fo[0]) <= 1e-12 * scale and abs(f["fy"] - fo[1]) <= 1e-12 * scale
    assert np.isfinite(f["cl"]) and np.isfinite(f["cd"])


@pytest.mark.parametrize("prec", ["FP32", "MIXED"])
def test_fast_sweep_independent_halves_bitwise(prec):
    """The binary32 dataflow sweep with independently synchronising half-warps
    (sweep_mode 4) computes every cell with the same arithmetic as the default
    one: identical bits after the fixture's steps."""
    from tmp_gb300 import abi

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    m = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    out = []
    for sm in (0, 4):
        case = abi.Case([m], [dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])], abi.FLOW_LAMINAR,
                        abi.ADV_LUSGS, getattr(abi, f"PREC_{prec}"), cfl=c["cfl"], sweep_mode=sm)
        case.put("U", g["init_U"])
        case.step(3)
        case.sync()
        out.append((case.get("U"), case.get("DW1"), case.get("DW")))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("prec", ["FP32", "MIXED"])
@pytest.mark.parametrize("bpsm", [1, 4])
def test_fast_sweep_chain_schedule_bitwise(prec, bpsm):
    """The chain-scheduled binary32 sweeps (sweep_mode 5: cells dealt to
    half-warps so that a dependency on the previous cell of the same
    half-warp is taken from registers; sweep_mode 6: the same with a block's
    lists consecutive and same-block dependencies handed over in shared
    memory) give the same bits as the default dataflow sweep, on the fixture mesh and on a cylinder mesh of ~25k cells
    whose quad rows form long chains, at two grid sizes (two schedules), both
    through plain steps and through the graph-captured step.  Mode 6 also runs
    with its table capped to a block's first 5 and 24 positions (the later
    producers hand off through global memory only)."""
    from tmp_gb300 import abi, learn

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    fixture = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    spec = learn.CaseSpec(nbody=96, nlayer=24, seed=12, dr1=5e-3, growth=1.05, rfar=30.0)
    cyl = spec.mesh()
    fs_fix = dict(mach=c["mach"], aoa_deg=c["aoa"], reynolds=c["re"])
    fs_cyl = dict(mach=spec.mach, aoa_deg=spec.aoa, reynolds=spec.re)
    for mesh, fs, init in [(fixture, fs_fix, g["init_U"]), (cyl, fs_cyl, None)]:
        out = []
        for sm, cap in ((0, 0), (5, 0), (6, 0), (6, 5), (6, 24)):
            case = abi.Case([mesh], [fs], abi.FLOW_LAMINAR, abi.ADV_LUSGS, getattr(abi, f"PREC_{prec}"),
                            cfl=c["cfl"], sweep_mode=sm, sweep_blocks_per_sm=bpsm, chain_table_cap=cap)
            if init is None:
                case.init_freestream()
            else:
                case.put("U", init)
            case.step(2)
            case.step_graph(2)
            case.sync()
            out.append((case.get("U"), case.get("DW1"), case.get("DW")))
        for other in out[1:]:
            for a, b in zip(out[0], other):
                np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", ["mixed_lam_lusgs", "omesh_euler_rk5"])
def test_tecplot_cell_dump_matches_reference(tmp_path, name):
    """writeCellData: the state of the fixture's initial field, Cp and Mach
    formed on the device, written byte for byte as the reference writes it."""
    from tmp_gb300 import abi

    c, g = manifest()[name], golden(name)
    tec = np.load(GOLDEN / "tecplot.npz")
    _, case = make_case(c)
    case.put("U", g["init_U"])
    case.write_cell_data(str(tmp_path / "cells"))
    assert (tmp_path / "cells_1_1").read_bytes() == bytes(tec[f"{name}/cells"])


def test_step_io_equals_separate_calls():
    """cfd_step_io (field in, graph steps, norms out, one sync) gives the bits
    of the separate put / step_graph / norm calls."""
    from tmp_gb300 import abi

    c, g = manifest()["mixed_lam_lusgs"], golden("mixed_lam_lusgs")
    _, a = make_case(c)
    _, b = make_case(c)
    u = np.ascontiguousarray(g["init_U"], np.float64).reshape(-1)
    back = np.zeros_like(u)
    for _ in range(2):
        n1 = a.step_io(u, 3, "L2_R_RHO", u_out=back)
        b.put("U", u)
        b.step_graph(3)
        n2 = b.norm("L2_R_RHO")
        assert n1[0] == n2
        np.testing.assert_array_equal(a.get("U"), b.get("U"))
        np.testing.assert_array_equal(back.reshape(-1, 4), b.get("U").reshape(-1, 4))
