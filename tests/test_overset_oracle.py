"""The overset restatement in oracle/ against the reference's own overset code.

tests/golden/overset.npz holds outputs of the reference's computeNodalWeight2D,
MeshBlock::search and getInterpolatedSolution/updateSolnData (compiled from
its sources, tests/golden/make_golden_overset.py).  The C restatement must
reproduce them bit for bit; the GPU kernels are then checked against both.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

import oracle
from oracle import grd


@pytest.fixture(scope="module")
def ov():
    return np.load(GOLDEN / "overset.npz")


def _meshes():
    return {"mx": grd.read_grd(GOLDEN / "mixed.grd", -1, -2), "om": grd.read_grd(GOLDEN / "omesh.grd", -1, -2)}


def test_weights_bitwise(ov):
    f, bad = oracle.nodal_weights(ov["w_nvert"], ov["w_xv"], ov["w_xp"])
    ref = ov["w_frac"]
    assert bad == int((ref[:, 0] == -1e300).sum()) and bad > 0
    assert np.array_equal(f.view(np.int64), ref.view(np.int64))
    # the cases cover both cell kinds, every findClockWise branch and Newton failures (u = 2)
    assert (ov["w_nvert"] == 3).sum() > 500 and (ov["w_nvert"] == 4).sum() > 1000
    quads = ov["w_nvert"] == 4
    assert np.any(np.abs(ref[quads].sum(1) - 1.0) < 1e-12)


def test_search_matches_reference_where_unique(ov):
    for name, m in _meshes().items():
        pts, ref = ov[f"s_{name}_pts"], ov[f"s_{name}_donor"]
        donor, cnt, _ = oracle.donor_search(m.xy, m.cell_verts, m.cell_nvert, pts)
        uniq = cnt <= 1
        assert np.array_equal(donor[uniq], ref[uniq])
        assert (ref >= 0).sum() > len(pts) // 2 and (ref < 0).sum() > 50
        # ties (points on shared vertices): the reference's donor is one of the containing cells
        tie = ~uniq
        assert tie.sum() > 0 and np.all(ref[tie] >= 0)


@pytest.mark.parametrize("nvar", [4, 6])
@pytest.mark.parametrize("layout", [0, 1])
def test_interp_update_bitwise(ov, nvar, layout):
    nn, nr = ov[f"i{nvar}_dims"]
    q = ov[f"i{nvar}_q"]
    qin = q.reshape(-1) if layout == 0 else np.ascontiguousarray(q.T).reshape(-1)
    qr = np.zeros(nr * nvar)
    oracle.interp_update(ov[f"i{nvar}_recv"], ov[f"i{nvar}_nw"], ov[f"i{nvar}_inode"], ov[f"i{nvar}_w"], qin,
                         nn, qr, nr, nvar, layout)
    ref = ov[f"i{nvar}_row" if layout == 0 else f"i{nvar}_col"]
    assert np.array_equal(qr.view(np.int64), ref.view(np.int64))
    assert len(np.unique(ov[f"i{nvar}_recv"])) < len(ov[f"i{nvar}_recv"])  # repeated receivers: last wins


@pytest.mark.parametrize("isym", [3, 1, 2])
def test_holemap_bitwise(ov, isym):
    for name, m in _meshes().items():
        nxy, geo, sam = oracle.holemap(m.xy, m.cell_verts, m.cell_nvert, oracle.wall_nodes(m), isym)
        assert np.array_equal(nxy, ov[f"h_{name}_{isym}_nx"])
        assert np.array_equal(geo.view(np.int64), ov[f"h_{name}_{isym}_ext"].view(np.int64))
        assert np.array_equal(sam, ov[f"h_{name}_{isym}_sam"])
        inside = oracle.holemap_check(nxy, geo, sam, ov[f"h_{name}_pts"])
        assert np.array_equal(inside, ov[f"h_{name}_{isym}_in"])
        assert 0 < inside.sum() < inside.size


def test_cell_iblank(ov):
    for name, m in _meshes().items():
        got = oracle.cell_iblank(m.cell_verts, m.cell_nvert, ov[f"c_{name}_node"])
        assert np.array_equal(got, ov[f"c_{name}_cell"])
        assert set(np.unique(got)) == {-1, 0, 1}


def test_connect_fixture_reproduces():
    """The assembly fixture is what the reference's own code gives today (run
    only where the reference's driver has been built)."""
    import subprocess
    from pathlib import Path

    drv = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "ref_overset"
    if not drv.exists():
        pytest.skip("reference overset driver not built here")
    import importlib.util

    spec = importlib.util.spec_from_file_location("mgc", GOLDEN / "make_golden_connect.py")
    mgc = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mgc)
    gc = np.load(GOLDEN / "overset_connect.npz")
    for name, meshes, nfringe, mexclude in mgc.cases():
        if name not in ("cyl", "three"):
            continue
        topos = [mgc.topo(g) for g in meshes]
        walls = [mgc.bnodes(t, -2) for t in topos]
        obcs = [np.zeros(0, np.int32)] + [mgc.bnodes(t, -3) for t in topos[1:]]
        ibl, iblc, interps = mgc.run_connect(topos, walls, obcs, nfringe, mexclude)
        for k in range(len(meshes)):
            p = f"{name}/{k}/"
            assert np.array_equal(ibl[k], gc[p + "iblank"])
            assert np.array_equal(iblc[k], gc[p + "cell_iblank"])
            assert np.array_equal(interps[k][0], gc[p + "interp_int"])
            assert np.array_equal(interps[k][1].view(np.int64), gc[p + "interp_w"].view(np.int64))
