"""Overset kernels on the GPU against the oracle and the reference's fixtures.

Weights and interpolated values are compared bit for bit.  Donors are
compared with the reference's own MeshBlock::search on every fixture point,
including points that lie in several cells (a shared edge or vertex, where the
first cell of the reference's tree walk donates), coincident points and cells
refused as donors (tests/golden/overset_ties.npz), and with the oracle's
literal restatement of that walk (orc_adt_search) on larger random sets.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

import oracle
from oracle import grd

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ov():
    return np.load(GOLDEN / "overset.npz")


def _eq(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


def _blocks(abi):
    out = {}
    for name, f in (("mx", "mixed.grd"), ("om", "omesh.grd")):
        mesh = abi.Mesh.load_grd(GOLDEN / f, -1, -2)
        out[name] = (mesh, abi.Block(mesh), grd.read_grd(GOLDEN / f, -1, -2))
    return out


def test_weights_match_reference(built_lib, ov):
    from tmp_gb300 import abi

    ok = ov["w_frac"][:, 0] != -1e300
    f = abi.nodal_weights(ov["w_nvert"][ok], ov["w_xv"][ok], ov["w_xp"][ok])
    assert _eq(f, ov["w_frac"][ok])
    with pytest.raises(abi.CfdError) as e:
        abi.nodal_weights(ov["w_nvert"][~ok][:3], ov["w_xv"][~ok][:3], ov["w_xp"][~ok][:3])
    assert e.value.code == -3


def test_weights_match_oracle_random(built_lib):
    from tmp_gb300 import abi

    rng = np.random.default_rng(7)
    n = 200_000
    nv = rng.choice([3, 4], n).astype(np.int32)
    xv = rng.normal(0, 1, (n, 4, 2)) * 10.0 ** rng.integers(-6, 3, (n, 1, 1))
    xp = xv[:, :3].mean(1) + rng.normal(0, 0.5, (n, 2)) * np.abs(xv).max((1, 2))[:, None]
    ref, bad = oracle.nodal_weights(nv, xv, xp)
    ok = ref[:, 0] != -1e300
    assert _eq(abi.nodal_weights(nv[ok], xv[ok], xp[ok]), ref[ok])


def _weights_in(topo, pts, donor):
    """The oracle's weights of each point in its donor cell (0 where there is none)."""
    xy = topo.xy.reshape(-1, 2)
    cv = topo.cell_verts.reshape(-1, 4)
    hit = donor >= 0
    w = np.zeros((len(pts), 4))
    c = donor[hit]
    nv = topo.cell_nvert[c]
    xv = np.zeros((c.size, 8))
    for m in range(4):
        xv[:, 2 * m:2 * m + 2] = xy[np.where(nv > m, cv[c, m], cv[c, 2])]
    f, bad = oracle.nodal_weights(nv, xv, pts[hit])
    assert bad == 0
    w[hit] = f
    return w


def test_search_matches_reference_and_oracle(built_lib, ov):
    from tmp_gb300 import abi

    for name, (mesh, blk, topo) in _blocks(abi).items():
        pts, ref = ov[f"s_{name}_pts"], ov[f"s_{name}_donor"]
        d, nodes, w = blk.search(pts)
        assert np.array_equal(d, ref)  # every point, the ties included
        od, _, _ = oracle.adt_search(topo.xy, topo.cell_verts, topo.cell_nvert, pts)
        assert np.array_equal(d, od)
        assert _eq(w, _weights_in(topo, pts, d))
        low, cnt, _ = oracle.donor_search(topo.xy, topo.cell_verts, topo.cell_nvert, pts)
        assert (cnt > 1).sum() >= 100 and (d != low).sum() > 50  # ties where the tree order matters
        cv = topo.cell_verts.reshape(-1, 4)
        hit = d >= 0
        assert np.array_equal(nodes[hit], cv[d[hit]])
        assert np.all(nodes[~hit] == -1)


@pytest.mark.parametrize("name", ["mx", "om", "ct"])
def test_search_ties_refusals_and_coincident_points(built_lib, name):
    """overset_ties.npz: every node, every edge midpoint, coincident copies (same and other tag), per-point
    resolutions and 30% of the cells refused as donors, against the reference's MeshBlock::search."""
    from tmp_gb300 import abi

    from tmp_gb300 import meshgen

    t = np.load(GOLDEN / "overset_ties.npz")
    if name == "ct":  # the fixture's Cartesian mesh, regenerated; its cells must be the ones the reference saw
        g = meshgen.cart_mesh(24, 20, (-1.0, -1.0), (1.0, 1.0))
        path = GOLDEN.parent / "_ct_tmp.grd"
        meshgen.write_grd(path, g)
        try:
            mesh = abi.Mesh.load_grd(path, g.wall_tag, g.far_tag)
            topo = grd.read_grd(path, g.wall_tag, g.far_tag)
        finally:
            path.unlink()
        assert np.array_equal(topo.xy, t["ct_mesh_xy"]) and np.array_equal(topo.cell_verts, t["ct_mesh_verts"])
        blk = abi.Block(mesh)
    else:
        mesh, blk, topo = _blocks(abi)[name]
    pts = t[f"{name}_pts"]
    d, nodes, w, xtag, res = blk.search_ex(pts, t[f"{name}_tags"], t[f"{name}_res"], t[f"{name}_unaccept"])
    assert np.array_equal(d, t[f"{name}_donor"])
    assert np.array_equal(xtag, t[f"{name}_xtag"])
    assert _eq(res, t[f"{name}_res_out"])
    assert _eq(w, _weights_in(topo, pts, d))  # merged points: their own weights in the first point's cell
    assert (xtag != np.arange(len(pts))).sum() > 100
    for k in range(3):  # one, two and three query points (findOBB's special cases)
        d, _, _ = blk.search(t[f"{name}_tiny{k}_pts"])
        assert np.array_equal(d, t[f"{name}_tiny{k}_donor"]), k


def test_search_large_sets_coincident_screen(built_lib):
    """Query sets of 2^16 points or more are screened for coincident pairs on the device before the reference's
    hash runs: with coincident copies (within 1e-10 in L1, same and other tag) the merges, donors and merged
    resolutions must be the oracle's; without any, every point keeps its own search."""
    from tmp_gb300 import abi

    mesh, blk, topo = _blocks(abi)["mx"]
    xy = topo.xy.reshape(-1, 2)
    lo, hi = xy.min(0), xy.max(0)
    rng = np.random.default_rng(17)
    base = np.concatenate([lo + rng.uniform(-0.02, 1.02, (70000, 2)) * (hi - lo), xy])
    for with_copies in (True, False):
        pts = base
        if with_copies:
            pick = rng.choice(len(base), 500, replace=False)
            pts = np.concatenate([base, base[pick] + rng.choice([0.0, 2e-11, -3e-11, 4e-11], (500, 2))])
        n = len(pts)
        tags = np.where(rng.random(n) < 0.3, 2, 1).astype(np.int32)
        res = rng.uniform(0.5, 2.0, n)
        unacc = (rng.random(topo.ncell) < 0.2).astype(np.uint8)
        d, _, w, xtag, r = blk.search_ex(pts, tags, res, unacc)
        od, oxt, orr = oracle.adt_search(topo.xy, topo.cell_verts, topo.cell_nvert, pts, unacc, tags, res)
        assert np.array_equal(xtag, oxt)
        assert np.array_equal(d, od)
        assert _eq(r, orr)
        merged = int((xtag != np.arange(n)).sum())
        assert (merged > 100) if with_copies else (merged == 0)


def test_search_larger_mesh_random_points(built_lib):
    from tmp_gb300 import abi, meshgen

    m = meshgen.mixed_mesh(meshgen.naca_body(96), nlayer=12, dr1=2e-3, growth=1.25, rfar=8.0, seed=3,
                           density=1.0, grade=1.0)
    path = GOLDEN.parent / "_ovs_tmp.grd"
    meshgen.write_grd(path, m)
    try:
        mesh = abi.Mesh.load_grd(path, -1, -2)
        topo = grd.read_grd(path, -1, -2)
    finally:
        path.unlink()
    blk = abi.Block(mesh)
    rng = np.random.default_rng(11)
    xy = topo.xy.reshape(-1, 2)
    lo, hi = xy.min(0), xy.max(0)
    pts = np.concatenate([lo + rng.uniform(-0.02, 1.02, (30000, 2)) * (hi - lo),
                          xy[rng.choice(len(xy), 2000, replace=False)],
                          rng.normal(0.5, 0.3, (8000, 2))])
    d, _, w = blk.search(pts)
    od, _, _ = oracle.adt_search(topo.xy, topo.cell_verts, topo.cell_nvert, pts)
    assert np.array_equal(d, od) and _eq(w, _weights_in(topo, pts, d))
    _, cnt, _ = oracle.donor_search(topo.xy, topo.cell_verts, topo.cell_nvert, pts)
    assert (cnt > 1).sum() > 100 and (d >= 0).sum() > 20000


@pytest.mark.parametrize("nvar", [4, 6])
@pytest.mark.parametrize("layout", [0, 1])
def test_interp_update_matches_reference(built_lib, ov, nvar, layout):
    import torch

    from tmp_gb300 import abi

    nn, nr = (int(x) for x in ov[f"i{nvar}_dims"])
    q = ov[f"i{nvar}_q"]
    qin = q.reshape(-1) if layout == 0 else np.ascontiguousarray(q.T).reshape(-1)
    it = abi.Interp.from_list(ov[f"i{nvar}_recv"], ov[f"i{nvar}_nw"], ov[f"i{nvar}_inode"], ov[f"i{nvar}_w"])
    dq = torch.tensor(qin, dtype=torch.float64, device="cuda")
    dr = torch.zeros(nr * nvar, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    it.update(dq.data_ptr(), nn, dr.data_ptr(), nr, nvar, layout)
    torch.cuda.synchronize()
    ref = ov[f"i{nvar}_row" if layout == 0 else f"i{nvar}_col"]
    assert _eq(dr.cpu().numpy(), ref)


def test_interp_in_place_and_edge_cases(built_lib):
    import torch

    from tmp_gb300 import abi

    rng = np.random.default_rng(5)
    nn, nvar, n = 500, 4, 300
    q = rng.normal(0, 1, nn * nvar)
    recv = rng.integers(0, nn, n).astype(np.int32)
    nw = rng.choice([3, 4], n).astype(np.int32)
    inode = rng.integers(0, nn, (n, 4)).astype(np.int32)
    w = np.zeros((n, 4))
    for i in range(n):
        w[i, :nw[i]] = rng.dirichlet(np.ones(nw[i]))
    expect = oracle.interp_update(recv, nw, inode, w, q, nn, q.copy(), nn, nvar, 0)
    it = abi.Interp.from_list(recv, nw, inode, w)
    dq = torch.tensor(q, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    it.update(dq.data_ptr(), nn, dq.data_ptr(), nn, nvar, abi.LAYOUT_ROW)
    torch.cuda.synchronize()
    assert _eq(dq.cpu().numpy(), expect)
    # empty list, non-convex weights, out-of-range nodes
    empty = abi.Interp.from_list(np.zeros(0), np.zeros(0), np.zeros((0, 4)), np.zeros((0, 4)))
    assert empty.info() == (0, 0)
    empty.update(dq.data_ptr(), nn, dq.data_ptr(), nn, nvar)
    bad_w = w.copy()
    bad_w[0, 0] = 1.5
    with pytest.raises(abi.CfdError) as e:
        abi.Interp.from_list(recv, nw, inode, bad_w)
    assert e.value.code == -3
    with pytest.raises(abi.CfdError):
        it.update(dq.data_ptr(), 10, dq.data_ptr(), nn, nvar)


def test_interp_from_search_and_node_to_cell(built_lib):
    import torch

    from tmp_gb300 import abi

    blocks = _blocks(abi)
    mesh_d, blk_d, topo_d = blocks["mx"]
    _, _, topo_r = blocks["om"]
    # receptors: the nodes of the other mesh, shifted into the donor's domain
    pts = topo_r.xy.reshape(-1, 2) * 0.9 + np.array([0.31, -0.17])
    recv = np.arange(len(pts), dtype=np.int32)
    it = abi.Interp.search(blk_d, pts, recv)
    nfound, nreq = it.info()
    d, nodes, w = blk_d.search(pts)
    assert nreq == len(pts) and nfound == (d >= 0).sum() > 0
    r, dc, inode, wl = it.get()
    hit = d >= 0
    assert np.array_equal(r, recv[hit]) and np.array_equal(dc, d[hit]) and _eq(wl, w[hit])
    nvar = 4
    rng = np.random.default_rng(9)
    qd = rng.normal(0, 1, topo_d.nnode * nvar)
    qr = rng.normal(0, 1, topo_r.nnode * nvar)
    nwl = np.where(inode[:, 3] < 0, 3, 4).astype(np.int32)
    expect = oracle.interp_update(r, nwl, np.where(inode < 0, 0, inode), wl, qd, topo_d.nnode, qr.copy(),
                                  topo_r.nnode, nvar, 0)
    dqd = torch.tensor(qd, dtype=torch.float64, device="cuda")
    dqr = torch.tensor(qr, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    it.update(dqd.data_ptr(), topo_d.nnode, dqr.data_ptr(), topo_r.nnode, nvar)
    torch.cuda.synchronize()
    assert _eq(dqr.cpu().numpy(), expect)
    # node -> cell mean (Orchestra.cpp:270-291), summed in vertex order then divided
    dc_out = torch.zeros(topo_d.ncell * nvar, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    blk_d.node_to_cell(dqd.data_ptr(), nvar, dc_out.data_ptr())
    torch.cuda.synchronize()
    cv = topo_d.cell_verts.reshape(-1, 4)
    qn = qd.reshape(-1, nvar)
    exp = np.zeros((topo_d.ncell, nvar))
    for c in range(topo_d.ncell):
        s = np.zeros(nvar)
        for j in range(topo_d.cell_nvert[c]):
            s = s + qn[cv[c, j]]
        exp[c] = s / topo_d.cell_nvert[c]
    assert _eq(dc_out.cpu().numpy(), exp.reshape(-1))


@pytest.mark.parametrize("isym", [3, 1, 2])
def test_holemap_matches_reference(built_lib, ov, isym):
    from tmp_gb300 import abi

    for name, (mesh, blk, topo) in _blocks(abi).items():
        hm = abi.HoleMap(blk, isym)
        nx, ext = hm.info()
        assert np.array_equal(nx, ov[f"h_{name}_{isym}_nx"]) and _eq(ext, ov[f"h_{name}_{isym}_ext"])
        assert np.array_equal(hm.get(), ov[f"h_{name}_{isym}_sam"])
        assert np.array_equal(hm.check(ov[f"h_{name}_pts"]), ov[f"h_{name}_{isym}_in"])


def test_overset_blank_matches_oracle(built_lib):
    from tmp_gb300 import abi

    blocks = _blocks(abi)
    _, blk_mx, topo_mx = blocks["mx"]
    _, blk_om, topo_om = blocks["om"]
    # mesh without walls of its own would not cut: both golden meshes have walls
    for nfringe in (0, 1, 2):
        ib, md = abi.overset_blank(blk_om, [blk_mx], [abi.HoleMap(blk_mx)], nfringe)
        eib, emd = oracle.blank(topo_om, [(topo_mx, oracle.wall_nodes(topo_mx), 3)], nfringe)
        assert np.array_equal(ib, eib) and np.array_equal(md, emd)
        assert (ib == 0).sum() > 0 and (nfringe == 0 or md.sum() > 0)
    ib, md = abi.overset_blank(blk_mx, [blk_om], [None], 1)
    assert np.all(ib == 1) and np.all(md == 0)


def test_overset_edge_cases(built_lib):
    from tmp_gb300 import abi, meshgen

    blocks = _blocks(abi)
    _, blk, topo = blocks["mx"]
    # no points, all points far outside, a block without walls
    d, nodes, w = blk.search(np.zeros((0, 2)))
    assert d.size == 0
    far = np.full((10, 2), 1e6)
    it = abi.Interp.search(blk, far, np.arange(10))
    assert it.info() == (0, 10)
    m = meshgen.cart_mesh(6, 5, (0.0, 0.0), (1.0, 1.0))
    path = GOLDEN.parent / "_cart_tmp.grd"
    meshgen.write_grd(path, m)
    try:
        mesh = abi.Mesh.load_grd(path, m.wall_tag, m.far_tag)
    finally:
        path.unlink()
    b2 = abi.Block(mesh)
    with pytest.raises(abi.CfdError) as e:
        abi.HoleMap(b2)
    assert e.value.code == -3
    # a Cartesian block donates to points inside it with bilinear weights
    pts = np.array([[0.31, 0.47], [0.999, 0.001], [0.5, 0.5]])
    d, nodes, w = b2.search(pts)
    assert np.all(d >= 0) and np.allclose(w.sum(1), 1.0, atol=1e-14)
    with pytest.raises(abi.CfdError):
        abi.HoleMap(blk, isym=7)


def test_cell_iblank_matches_reference(built_lib, ov):
    from tmp_gb300 import abi

    for name, (mesh, blk, topo) in _blocks(abi).items():
        assert np.array_equal(blk.cell_iblank(ov[f"c_{name}_node"]), ov[f"c_{name}_cell"])
