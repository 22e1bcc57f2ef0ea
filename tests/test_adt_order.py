"""The donor search's tree order, host half (tmp_gb300/csrc/adt.cpp), on the CPU.

The device search (k_donor_search) keeps, per point, the contained and
acceptable cell of lowest preorder number in the reference's search tree, else
the outcome of the highest-numbered cell it checks, and coincident points take
the first one's donor.  Here the product's host code (compiled with g++ into
tests/adt_check.cpp) gives the tree order and the coincident-point hash, the
same selection is evaluated in numpy with the oracle's weights, and the donors
must be the reference's own (tests/golden/overset.npz, overset_ties.npz, from
MeshBlock::search compiled from its sources) on every point, ties included.
"""
from __future__ import annotations

import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import oracle
from oracle import grd

TOL = 1e-10


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not present")
    exe = tmp_path_factory.mktemp("adt") / "adt_check"
    csrc = ROOT / "tmp_gb300" / "csrc"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", f"-I{csrc}", str(ROOT / "tests" / "adt_check.cpp"),
           str(csrc / "adt.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def run(exe, tmp, xy, cv, nv, pts, tags, res):
    inp, out = tmp / "in.bin", tmp / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(xy.reshape(-1)) // 2, len(nv)], np.int32).tofile(f)
        np.asarray(xy, np.float64).tofile(f)
        np.asarray(nv, np.int32).tofile(f)
        np.asarray(cv, np.int32).reshape(-1).tofile(f)
        np.array([len(pts)], np.int32).tofile(f)
        np.asarray(pts, np.float64).tofile(f)
        np.asarray(tags, np.int32).tofile(f)
        np.asarray(res, np.float64).tofile(f)
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    raw = out.read_bytes()
    nc, n = len(nv), len(pts)
    rank = np.frombuffer(raw[:4 * nc], np.int32)
    xtag = np.frombuffer(raw[4 * nc:4 * (nc + n)], np.int32)
    rout = np.frombuffer(raw[4 * (nc + n):], np.float64)
    return rank, xtag, rout


def select(xy, cv, nv, pts, rank, unacc, xtag, amb=None):
    """k_donor_search's choice per point, then k_take_coincident's; amb (optional, filled): the points whose
    choice depends on the order of the tree cells (several cells stop the walk, or none does and a refused one
    contains the point)."""
    xy = np.asarray(xy).reshape(-1, 2)
    cv = np.asarray(cv).reshape(-1, 4)
    lo = np.full((len(nv), 2), 1e15)
    hi = np.full((len(nv), 2), -1e15)
    for m in range(4):
        has = nv > m
        v = xy[cv[has, m]]
        lo[has] = np.minimum(lo[has], v)
        hi[has] = np.maximum(hi[has], v)
    n = len(pts)
    donor = np.full(n, -1, np.int32)
    for i in range(n):
        if xtag[i] != i:
            continue
        p = pts[i]
        cand = np.flatnonzero((rank >= 0) & (p[0] >= lo[:, 0] - TOL) & (p[1] >= lo[:, 1] - TOL) &
                              (p[0] <= hi[:, 0] + TOL) & (p[1] <= hi[:, 1] + TOL))
        if cand.size == 0:
            continue
        xv = np.zeros((cand.size, 8))
        for m in range(4):
            idx = np.where(nv[cand] > m, cv[cand, m], cv[cand, 2])
            xv[:, 2 * m:2 * m + 2] = xy[idx]
        f, bad = oracle.nodal_weights(nv[cand], xv, np.repeat(p[None], cand.size, 0))
        assert bad == 0
        used = np.arange(4)[None, :] < nv[cand][:, None]
        inside = np.all(~used | ((f + TOL) * (f - 1.0 - TOL) <= 0), axis=1)
        refused = unacc[cand].astype(bool) & np.any(used & (np.abs(f) < TOL), axis=1)
        good = inside & ~refused
        if amb is not None:
            amb[i] = good.sum() > 1 or (good.sum() == 0 and (inside & refused).any())
        if good.any():
            donor[i] = cand[good][np.argmin(rank[cand][good])]
        else:
            k = np.argmax(rank[cand])
            donor[i] = cand[k] if inside[k] else -1
    for i in range(n):  # xtag[i] <= i: the group's first point is already final
        if xtag[i] != i:
            donor[i] = donor[xtag[i]]
    return donor


def _golden_meshes():
    return {"mx": grd.read_grd(GOLDEN / "mixed.grd", -1, -2), "om": grd.read_grd(GOLDEN / "omesh.grd", -1, -2)}


@pytest.mark.parametrize("name", ["mx", "om"])
def test_tree_order_gives_reference_donors(harness, tmp_path, name):
    ov = np.load(GOLDEN / "overset.npz")
    m = _golden_meshes()[name]
    pts, ref = ov[f"s_{name}_pts"], ov[f"s_{name}_donor"]
    n = len(pts)
    rank, xtag, _ = run(harness, tmp_path, m.xy, m.cell_verts, m.cell_nvert, pts, np.ones(n), np.ones(n))
    donor = select(m.xy, m.cell_verts, m.cell_nvert, pts, rank, np.zeros(m.ncell, np.uint8), xtag)
    assert np.array_equal(donor, ref)
    _, cnt, _ = oracle.donor_search(m.xy, m.cell_verts, m.cell_nvert, pts)
    assert (cnt > 1).sum() >= 100  # ties: points in several cells


@pytest.mark.parametrize("name", ["mx", "om", "ct"])
def test_tree_order_ties_refusals_and_coincident_points(harness, tmp_path, name):
    t = np.load(GOLDEN / "overset_ties.npz")
    if name == "ct":
        xy, cv, nv = t["ct_mesh_xy"], t["ct_mesh_verts"], t["ct_mesh_nvert"]
    else:
        m = _golden_meshes()[name]
        xy, cv, nv = m.xy, m.cell_verts, m.cell_nvert
    pts = t[f"{name}_pts"]
    rank, xtag, rout = run(harness, tmp_path, xy, cv, nv, pts, t[f"{name}_tags"], t[f"{name}_res"])
    assert np.array_equal(xtag, t[f"{name}_xtag"])
    assert np.array_equal(rout.view(np.int64), t[f"{name}_res_out"].view(np.int64))
    assert (xtag != np.arange(len(pts))).sum() > 100
    donor = select(xy, cv, nv, pts, rank, t[f"{name}_unaccept"], xtag)
    assert np.array_equal(donor, t[f"{name}_donor"])
    # the device's first pass gives every tree cell one rank: it is exact wherever the choice does not depend on
    # the order, and it flags the rest
    amb = np.zeros(len(pts), bool)
    first = select(xy, cv, nv, pts, np.where(rank >= 0, 0, -1), t[f"{name}_unaccept"], np.arange(len(pts)), amb)
    assert amb.sum() > 50
    assert np.array_equal(first[~amb], select(xy, cv, nv, pts, rank, t[f"{name}_unaccept"], np.arange(len(pts)))[~amb])


@pytest.mark.parametrize("name", ["mx", "om", "ct"])
def test_tree_order_tiny_query_sets(harness, tmp_path, name):
    """One, two and three query points: findOBB's special cases for one and two points."""
    t = np.load(GOLDEN / "overset_ties.npz")
    if name == "ct":
        xy, cv, nv = t["ct_mesh_xy"], t["ct_mesh_verts"], t["ct_mesh_nvert"]
    else:
        m = _golden_meshes()[name]
        xy, cv, nv = m.xy, m.cell_verts, m.cell_nvert
    for k in range(3):
        pts = t[f"{name}_tiny{k}_pts"]
        n = len(pts)
        rank, xtag, _ = run(harness, tmp_path, xy, cv, nv, pts, np.ones(n), np.ones(n))
        donor = select(xy, cv, nv, pts, rank, np.zeros(len(nv), np.uint8), xtag)
        assert np.array_equal(donor, t[f"{name}_tiny{k}_donor"]), k
        d, _, _ = oracle.adt_search(xy, cv, nv, pts)
        assert np.array_equal(d, t[f"{name}_tiny{k}_donor"]), k


@pytest.mark.parametrize("name", ["mx", "om", "ct"])
def test_oracle_walk_matches_reference(name):
    """The oracle's literal restatement of the tree walk (oracle/cfd_oracle.c, orc_adt_search)."""
    t = np.load(GOLDEN / "overset_ties.npz")
    if name == "ct":
        xy, cv, nv = t["ct_mesh_xy"], t["ct_mesh_verts"], t["ct_mesh_nvert"]
    else:
        m = _golden_meshes()[name]
        xy, cv, nv = m.xy, m.cell_verts, m.cell_nvert
    d, xt, r = oracle.adt_search(xy, cv, nv, t[f"{name}_pts"], t[f"{name}_unaccept"], t[f"{name}_tags"],
                                 t[f"{name}_res"])
    assert np.array_equal(d, t[f"{name}_donor"])
    assert np.array_equal(xt, t[f"{name}_xtag"])
    assert np.array_equal(r.view(np.int64), t[f"{name}_res_out"].view(np.int64))
    ov = np.load(GOLDEN / "overset.npz")
    if name != "ct":
        d, _, _ = oracle.adt_search(xy, cv, nv, ov[f"s_{name}_pts"])
        assert np.array_equal(d, ov[f"s_{name}_donor"])


def _screen(pts, tags, tol=TOL):
    """The device screen's logic (k_coinc_scan) on the host: sort by (tag, x, y); each point against its
    successor and against the nearest y of every following x within tol of its tag."""
    x = pts[:, 0] + 0.0  # -0.0 as +0.0
    y = pts[:, 1]
    order = np.lexsort((y, x, tags))
    sx, sy, st = x[order], y[order], tags[order]
    n = len(sx)
    for i in range(n):
        if i + 1 < n and st[i + 1] == st[i] and abs(sx[i] - sx[i + 1]) + abs(sy[i] - sy[i + 1]) < tol:
            return True
        run = np.flatnonzero(st == st[i])
        lo, hi = run[0], run[-1] + 1
        g = lo + np.searchsorted(sx[lo:hi], sx[i], side="right")
        while g < hi and sx[g] - sx[i] < tol:
            e = lo + np.searchsorted(sx[lo:hi], sx[g], side="right")
            a = g + np.searchsorted(sy[g:e], sy[i], side="left")
            for k in (a, a - 1):
                if g <= k < e and abs(sx[i] - sx[k]) + abs(sy[i] - sy[k]) < tol:
                    return True
            g = e
    return False


def _brute(pts, tags, tol=TOL):
    n = len(pts)
    for i in range(n):
        d = np.abs(pts[i + 1:] - pts[i]).sum(1)
        if np.any((d < tol) & (tags[i + 1:] == tags[i])):
            return True
    return False


def test_coincident_screen_logic():
    """The device screen for coincident query points (k_overset.cu, k_coinc_scan) finds a pair closer than TOL
    in L1 with one tag exactly when one exists: its logic, restated in numpy, against all pairs on sets built to
    defeat it (whole columns of equal x, x values within TOL of each other, signed zeros, pairs across tags)."""
    rng = np.random.default_rng(5)
    positives = 0
    for trial in range(100):
        kind = trial % 5
        if kind == 0:  # a Cartesian lattice (columns of equal x) plus a few stray points
            g = np.stack(np.meshgrid(np.arange(12) * 0.1, np.arange(9) * 0.1), -1).reshape(-1, 2)
            pts = np.concatenate([g, rng.uniform(0, 1, (20, 2))])
        elif kind in (1, 2):  # columns whose x differ by less than TOL, sharing (1) or shifting (2) their y values
            cols = [0.5, 0.5 + 4e-11, 0.5 + 2e-10]
            ys = np.arange(10) * 0.07
            pts = np.concatenate([np.stack([np.full(10, c), ys + (7e-11 * k if kind == 2 else 0.0)], 1)
                                  for k, c in enumerate(cols)])
        elif kind == 3:  # signed zeros
            pts = np.stack([np.where(rng.random(40) < 0.5, -0.0, 0.0), rng.uniform(-1, 1, 40)], 1)
        else:
            pts = rng.uniform(-1, 1, (60, 2))
        tags = rng.integers(1, 3, len(pts)).astype(np.int32)
        if trial % 3 == 0:  # plant one near-coincident pair, sometimes across tags only
            i, j = rng.choice(len(pts), 2, replace=False)
            pts[j] = pts[i] + rng.choice([0.0, 3e-11, -4e-11], 2)
            if trial % 2:
                tags[j] = 3 - tags[i]
        want = _brute(pts, tags)
        positives += want
        assert _screen(pts, tags) == want, trial
    assert 20 <= positives <= 80
