"""Pin the C oracle (oracle/cfd_oracle.c) to the reference's own dumps.

Every array the oracle produces must equal, bit for bit, the array the
reference's compiled serial path dumped for the same mesh and input
(tests/golden/make_golden.py).  Runs on CPU only.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, golden, manifest

CASES = list(manifest())


def _oracle(name):
    import oracle
    from oracle import grd

    c = manifest()[name]
    t = grd.read_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    return c, t, oracle.Oracle(t, c["mach"], c["aoa"], c["re"], c["flow"] == "viscous")


@pytest.mark.parametrize("name", CASES)
def test_topology_and_geometry(name, built_oracle):
    c, t, o = _oracle(name)
    g = golden(name)
    np.testing.assert_array_equal(t.lr, g["topo_lr"])
    np.testing.assert_array_equal(t.cell_edges, g["topo_cedges"])
    np.testing.assert_array_equal(t.cell_verts, g["topo_cverts"])
    for fld, key in [("VOL", "geo_vol"), ("CENTER", "geo_cen"), ("NORMAL", "geo_nrm"), ("AREA", "geo_area"),
                     ("ECENTER", "geo_ecen"), ("WALLDIST", "geo_wall")]:
        np.testing.assert_array_equal(o.field(fld).ravel(), g[key], err_msg=fld)


@pytest.mark.parametrize("name", CASES)
def test_residual_phase(name, built_oracle):
    c, t, o = _oracle(name)
    g = golden(name)
    o.set_U(g["init_U"])
    assert o.residual(bool(c["first_order"])) == 0
    pairs = [("R", "res0_R"), ("UEDGE", "res0_Uedge"), ("GRAD", "res0_grad"), ("PHI", "res0_phi"),
             ("SPEC_C", "res0_specc"), ("UL", "res0_UL"), ("UR", "res0_UR")]
    if c["flow"] == "viscous":
        pairs += [("GRADT", "res0_gradT"), ("SPEC_V", "res0_specv"), ("MU", "res0_mu"), ("MUEDGE", "res0_muedge")]
    for fld, key in pairs:
        np.testing.assert_array_equal(o.field(fld).ravel(), g[key], err_msg=fld)
    o.solve_time(c["cfl"] if c["advance"] == "lusgs" else 0.8)
    np.testing.assert_array_equal(o.field("DT"), g["res0_dt"])


@pytest.mark.parametrize("name", CASES)
def test_steps(name, built_oracle):
    c, t, o = _oracle(name)
    g = golden(name)
    o.set_U(g["init_U"])
    hist = []
    for _ in range(c["nsteps"]):
        if c["advance"] == "lusgs":
            o.lusgs_step(c["cfl"], bool(c["first_order"]))
            hist.append(float(np.sum(o.field("DW")[:, 0] ** 2)))
        else:
            o.rk_step(bool(c["first_order"]))
    np.testing.assert_array_equal(o.field("U").ravel(), g["end_U"])
    if c["advance"] == "lusgs":
        np.testing.assert_array_equal(o.field("DIAG"), g["end_D"][::4])
        for fld, key in [("DW1", "end_dW1"), ("DW", "end_dW"), ("W", "end_W"), ("R", "end_R")]:
            np.testing.assert_array_equal(o.field(fld).ravel(), g[key], err_msg=fld)
        np.testing.assert_allclose(hist, g["hist"], rtol=1e-12)
    else:
        np.testing.assert_array_equal(o.field("W").ravel(), g["end_W0"])


def test_planted_mistake_is_caught(built_oracle):
    """A one-ulp change in the oracle's output must fail the comparison."""
    c, t, o = _oracle("omesh_euler_rk5")
    g = golden("omesh_euler_rk5")
    o.set_U(g["init_U"])
    o.residual()
    r = o.field("R").ravel().copy()
    r[7] = np.nextafter(r[7], np.inf)
    assert not np.array_equal(r, g["res0_R"])


def test_reference_driver_matches_fixtures(tmp_path):
    """When the reference sources are present, rebuild its serial path and rerun one case."""
    import subprocess
    from pathlib import Path

    from oracle.build import build_ref

    drv = build_ref()
    if drv is None:
        pytest.skip("reference sources not present")
    c = manifest()["mixed_lam_lusgs"]
    g = golden("mixed_lam_lusgs")
    init = tmp_path / "u0.bin"
    g["init_U"].astype(np.float64).tofile(init)
    out = tmp_path / "out"
    subprocess.run([str(drv), str(GOLDEN / c["mesh"]), str(c["wall_tag"]), str(c["far_tag"]), "viscous", "lusgs",
                    repr(c["mach"]), repr(c["aoa"]), repr(c["re"]), repr(c["cfl"]), str(c["nsteps"]), str(out),
                    str(init), "0"], check=True, capture_output=True)
    np.testing.assert_array_equal(np.fromfile(out / "end_U.bin"), g["end_U"])
