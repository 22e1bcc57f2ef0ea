"""Generate tests/golden/overset.npz from the reference's own overset code.

Runs oracle/_ref/ref_overset (built from the reference's UniTioga and
mathTools sources by oracle/build_ref.sh) on seeded inputs:

  weights   computeNodalWeight2D on random triangles and quadrilaterals (every
            vertex order, tiny and rotated cells that take solvec's row
            exchange, points inside, on edges and outside) and on the cells of
            the two golden meshes
  search    MeshBlock::search of random points, of the nodes of the other
            golden mesh (shifted, as an overset pair) and of the donor's own
            cell centres, in mixed.grd (triangles + quadrilaterals) and in
            omesh.grd (quadrilaterals)
  interp    getInterpolatedSolution + updateSolnData, ROW and COLUMN, with
            repeated receivers, nvar = 4 and 6
  holemap   tioga::getHoleMap (markWallBoundary + fillHoleMap) of each golden
            mesh's walls for isym = 3, 1, 2, and checkHoleMap of random points
            and of the other mesh's nodes
  celliblank MeshBlock::getCellIblanks of random node blanking (holes,
            receptors, field nodes in clusters) on both golden meshes

and tests/golden/overset_ties.npz, MeshBlock::search where several cells
contain a point: every mesh node, every edge midpoint, cell centres and random
points, coincident copies (within the 1e-10 L1 tolerance, same and other mesh
tag), per-point resolutions and a random 30% of the cells refused as donors
(cellRes = BIGVALUE), on both golden meshes and on a mesh whose edges carry
the nodes of a second Cartesian mesh shifted by half a cell.

usage: python tests/golden/make_golden_overset.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import grd  # noqa: E402

DRV = ROOT / "oracle" / "_ref" / "ref_overset"


def _run(*args, cwd):
    subprocess.run([str(DRV), *map(str, args)], check=True, cwd=cwd, stdout=subprocess.DEVNULL)


def weights_cases(rng: np.random.Generator, meshes):
    nv, xv, xp = [], [], []

    def add(n, x, p):
        nv.append(n)
        v = np.zeros((4, 2))
        v[:n] = x
        xv.append(v)
        xp.append(p)

    # quadrilaterals: jittered unit squares in every vertex order, scaled and rotated
    perms = [(0, 1, 2, 3), (0, 3, 2, 1), (0, 2, 1, 3), (0, 1, 3, 2), (1, 2, 3, 0), (0, 2, 3, 1)]
    base = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    for i in range(1500):
        q = base + rng.normal(0, 0.12, (4, 2))
        q = q[list(perms[i % len(perms)])]
        ang = rng.uniform(0, 2 * np.pi) if i % 3 else (np.pi / 2) * (i % 4)
        R = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
        scale = 10.0 ** rng.choice([-9, -6, -3, 0, 0, 0, 1, 3])
        off = rng.normal(0, 5, 2)
        q = (q @ R.T) * scale + off
        kind = i % 5
        if kind == 0:
            p = q.mean(0)
        elif kind == 1:
            t = rng.uniform()
            a, b = q[i % 4], q[(i + 1) % 4]
            p = a + t * (b - a)
        elif kind == 2:
            p = q[i % 4].copy()
        else:
            p = q.mean(0) + rng.normal(0, 0.7, 2) * scale
        add(4, q, p)
    # axis-aligned squares: zero off-diagonals take the exchange branch of solvec
    for i in range(60):
        s = 10.0 ** rng.integers(-3, 3)
        q = np.array([[0, 0], [0, 1], [1, 1], [1, 0]], float) * s + rng.integers(-4, 4, 2)
        add(4, q, q[0] + rng.uniform(-0.2, 1.2, 2) * s)
    # triangles
    for i in range(1200):
        t = rng.normal(0, 1, (3, 2))
        scale = 10.0 ** rng.choice([-10, -7, 0, 0, 2])
        t = t * scale + rng.normal(0, 3, 2)
        if i % 7 == 0:
            t[0, 0] = t[2, 0]  # zero pivot: row exchange
        w = rng.dirichlet([1, 1, 1]) if i % 2 else rng.uniform(-0.5, 1.5, 3)
        add(3, t, w @ t if i % 2 else t.mean(0) + (w[:2] - 0.5) * scale)
    # cells of the golden meshes with points around them
    for m in meshes:
        cv = m.cell_verts.reshape(-1, 4)
        for c in rng.choice(m.ncell, 300, replace=False):
            n = int(m.cell_nvert[c])
            x = m.xy.reshape(-1, 2)[cv[c, :n]]
            lo, hi = x.min(0), x.max(0)
            add(n, x, lo + rng.uniform(-0.2, 1.2, 2) * (hi - lo))
    return np.array(nv, np.int32), np.array(xv), np.array(xp)


def write_weights(path, nv, xv, xp):
    with open(path, "wb") as f:
        np.array([nv.size], np.int32).tofile(f)
        for i in range(nv.size):
            np.array([nv[i]], np.int32).tofile(f)
            xv[i].astype(np.float64).tofile(f)
            xp[i].astype(np.float64).tofile(f)


def write_mesh(path, m):
    with open(path, "wb") as f:
        np.array([m.nnode, m.ncell], np.int32).tofile(f)
        m.xy.astype(np.float64).tofile(f)
        m.cell_nvert.astype(np.int32).tofile(f)
        m.cell_verts.astype(np.int32).tofile(f)


def cell_centres(m):
    cv = m.cell_verts.reshape(-1, 4)
    xy = m.xy.reshape(-1, 2)
    out = np.zeros((m.ncell, 2))
    for c in range(m.ncell):
        n = m.cell_nvert[c]
        out[c] = xy[cv[c, :n]].mean(0)
    return out


def edge_midpoints(m):
    cv = m.cell_verts.reshape(-1, 4)
    xy = m.xy.reshape(-1, 2)
    e = set()
    for c in range(m.ncell):
        n = m.cell_nvert[c]
        for k in range(n):
            a, b = int(cv[c, k]), int(cv[c, (k + 1) % n])
            e.add((min(a, b), max(a, b)))
    e = np.array(sorted(e))
    return (xy[e[:, 0]] + xy[e[:, 1]]) * 0.5


def ties_cases(rng: np.random.Generator):
    from tmp_gb300 import meshgen

    om = grd.read_grd(HERE / "omesh.grd", -1, -2)
    mx = grd.read_grd(HERE / "mixed.grd", -1, -2)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        g = meshgen.cart_mesh(24, 20, (-1.0, -1.0), (1.0, 1.0))
        meshgen.write_grd(td / "ct.grd", g)
        cart = grd.read_grd(td / "ct.grd", g.wall_tag, g.far_tag)
        for name, m in (("mx", mx), ("om", om), ("ct", cart)):
            xy = m.xy.reshape(-1, 2)
            lo, hi = xy.min(0), xy.max(0)
            base = [xy, edge_midpoints(m), cell_centres(m), lo + rng.uniform(-0.05, 1.05, (400, 2)) * (hi - lo)]
            if name == "ct":  # the nodes of a Cartesian mesh shifted by half a cell lie on this one's edges
                h = (hi - lo) / np.array([24, 20])
                base.append(meshgen.cart_mesh(24, 20, tuple(lo + h / 2), tuple(hi + h / 2)).xy.reshape(-1, 2))
            pts = np.concatenate(base)
            # coincident copies: within the tolerance (L1 below 1e-10) or exact, same tag or another
            pick = rng.choice(len(pts), 300, replace=False)
            dup = pts[pick] + rng.choice([0.0, 2e-11, -3e-11], (300, 2))
            pts = np.concatenate([pts, dup])
            perm = rng.permutation(len(pts))
            pts = pts[perm]
            tags = np.where(rng.random(len(pts)) < 0.2, 2, 1).astype(np.int32)
            res = rng.uniform(0.5, 2.0, len(pts))
            unacc = (rng.random(m.ncell) < 0.3).astype(np.int32)
            write_mesh(td / "m.bin", m)
            with open(td / "p.bin", "wb") as f:
                np.array([len(pts)], np.int32).tofile(f)
                pts.astype(np.float64).tofile(f)
                tags.tofile(f)
                res.astype(np.float64).tofile(f)
                unacc.tofile(f)
            _run("search2", td / "m.bin", td / "p.bin", td / "s.out", cwd=td)
            raw = (td / "s.out").read_bytes()
            n = len(pts)
            out[f"{name}_pts"] = pts
            out[f"{name}_tags"] = tags
            out[f"{name}_res"] = res
            out[f"{name}_unaccept"] = unacc
            out[f"{name}_donor"] = np.frombuffer(raw[:4 * n], np.int32)
            out[f"{name}_xtag"] = np.frombuffer(raw[4 * n:8 * n], np.int32)
            out[f"{name}_res_out"] = np.frombuffer(raw[8 * n:], np.float64)
            if name == "ct":
                out["ct_mesh_xy"] = m.xy
                out["ct_mesh_verts"] = m.cell_verts
                out["ct_mesh_nvert"] = m.cell_nvert
            # tiny query sets: one point and two points take findOBB's special cases (an axis box of
            # half-width 1e-3, or the reference's max(1e-3, d) * 0.5 that halves only the second operand)
            for k, sel in enumerate(([0], [1, 2], [3, 4, 5])):
                tp = np.asarray(xy[rng.choice(len(xy), len(sel), replace=False)], np.float64)
                tg = np.ones(len(tp), np.int32)
                tr = np.ones(len(tp))
                tu = np.zeros(m.ncell, np.int32)
                with open(td / "p.bin", "wb") as f:
                    np.array([len(tp)], np.int32).tofile(f)
                    tp.tofile(f)
                    tg.tofile(f)
                    tr.tofile(f)
                    tu.tofile(f)
                _run("search2", td / "m.bin", td / "p.bin", td / "s.out", cwd=td)
                raw = (td / "s.out").read_bytes()
                out[f"{name}_tiny{k}_pts"] = tp
                out[f"{name}_tiny{k}_donor"] = np.frombuffer(raw[:4 * len(tp)], np.int32)
    np.savez_compressed(HERE / "overset_ties.npz", **out)
    print(f"wrote {HERE / 'overset_ties.npz'}: " + ", ".join(f"{k}: {len(out[k + '_pts'])} points"
                                                           for k in ("mx", "om", "ct")))


def main():
    if not DRV.exists():
        raise SystemExit(f"{DRV} missing: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20240611)
    om = grd.read_grd(HERE / "omesh.grd", -1, -2)
    mx = grd.read_grd(HERE / "mixed.grd", -1, -2)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        nv, xv, xp = weights_cases(rng, [om, mx])
        write_weights(td / "w.in", nv, xv, xp)
        _run("weights", td / "w.in", td / "w.out", cwd=td)
        out.update(w_nvert=nv, w_xv=xv, w_xp=xp, w_frac=np.fromfile(td / "w.out", np.float64).reshape(-1, 4))

        for name, donor, other, shift in (("mx", mx, om, (0.31, -0.17)), ("om", om, mx, (-0.23, 0.41))):
            xy = donor.xy.reshape(-1, 2)
            lo, hi = xy.min(0), xy.max(0)
            pts = np.concatenate([
                lo + rng.uniform(-0.05, 1.05, (1500, 2)) * (hi - lo),
                other.xy.reshape(-1, 2) * 0.9 + np.array(shift),
                cell_centres(donor),
                xy[rng.choice(donor.nnode, 100, replace=False)],
            ])
            write_mesh(td / "m.bin", donor)
            with open(td / "p.bin", "wb") as f:
                np.array([len(pts)], np.int32).tofile(f)
                pts.astype(np.float64).tofile(f)
            _run("search", td / "m.bin", td / "p.bin", td / "s.out", cwd=td)
            out[f"s_{name}_pts"] = pts
            out[f"s_{name}_donor"] = np.fromfile(td / "s.out", np.int32)

        for nvar in (4, 6):
            nnodes, nrecv, n = 300, 200, 150
            q = rng.normal(0, 1, (nnodes, nvar))
            recv = rng.integers(0, nrecv, n).astype(np.int32)
            nw = rng.choice([3, 4], n).astype(np.int32)
            inode = rng.integers(0, nnodes, (n, 4)).astype(np.int32)
            w = np.zeros((n, 4))
            for i in range(n):
                w[i, :nw[i]] = rng.dirichlet(np.ones(nw[i]))
            inode[nw == 3, 3] = 0
            with open(td / "i.bin", "wb") as f:
                np.array([nnodes, nvar, n, nrecv], np.int32).tofile(f)
                q.astype(np.float64).tofile(f)
                for i in range(n):
                    np.array([recv[i], nw[i]], np.int32).tofile(f)
                    inode[i].tofile(f)
                    w[i].astype(np.float64).tofile(f)
            _run("interp", td / "i.bin", td / "i.out", cwd=td)
            res = np.fromfile(td / "i.out", np.float64).reshape(2, -1)
            out.update({f"i{nvar}_q": q, f"i{nvar}_recv": recv, f"i{nvar}_nw": nw, f"i{nvar}_inode": inode,
                        f"i{nvar}_w": w, f"i{nvar}_row": res[0], f"i{nvar}_col": res[1],
                        f"i{nvar}_dims": np.array([nnodes, nrecv])})
        for name, m, other in (("mx", mx, om), ("om", om, mx)):
            wall = oracle.wall_nodes(m)
            xy = m.xy.reshape(-1, 2)
            wxy = xy[wall]
            lo, hi = wxy.min(0), wxy.max(0)
            span = hi - lo
            pts = np.concatenate([lo - 0.1 * span + rng.uniform(0, 1.2, (4000, 2)) * span,
                                  other.xy.reshape(-1, 2) * 0.5 + lo + 0.5 * span - 0.25])
            write_mesh(td / "m.bin", m)
            with open(td / "p.bin", "wb") as f:
                np.array([len(pts)], np.int32).tofile(f)
                pts.astype(np.float64).tofile(f)
            for isym in (3, 1, 2):
                with open(td / "wl.bin", "wb") as f:
                    np.array([isym, wall.size], np.int32).tofile(f)
                    wall.astype(np.int32).tofile(f)
                _run("holemap", td / "m.bin", td / "wl.bin", td / "p.bin", td / "h.out", cwd=td)
                raw = (td / "h.out").read_bytes()
                nxy = np.frombuffer(raw[:8], np.int32)
                geo = np.frombuffer(raw[8:40], np.float64)
                nsam = int(nxy[0]) * int(nxy[1])
                sam = np.frombuffer(raw[40:40 + 4 * nsam], np.int32).reshape(nxy[1], nxy[0])
                inside = np.frombuffer(raw[40 + 4 * nsam:], np.int32)
                out.update({f"h_{name}_{isym}_nx": nxy, f"h_{name}_{isym}_ext": geo,
                            f"h_{name}_{isym}_sam": sam, f"h_{name}_{isym}_in": inside})
            out[f"h_{name}_pts"] = pts
        for name, m in (("mx", mx), ("om", om)):
            xy = m.xy.reshape(-1, 2)
            # clustered blanking: holes near one point, receptors in a ring around it
            c0 = xy[rng.integers(m.nnode)]
            dist = np.hypot(*(xy - c0).T)
            r0 = np.quantile(dist, 0.1)
            ibl = np.ones(m.nnode, np.int32)
            ibl[dist < r0] = 0
            ring = (dist >= r0) & (dist < 1.6 * r0)
            ibl[ring] = -1
            flip = rng.random(m.nnode) < 0.03
            ibl[flip] = rng.choice([-1, 0, 1], flip.sum())
            write_mesh(td / "m.bin", m)
            ibl.tofile(td / "ibl.bin")
            _run("celliblank", td / "m.bin", td / "ibl.bin", td / "c.out", cwd=td)
            out[f"c_{name}_node"] = ibl
            out[f"c_{name}_cell"] = np.fromfile(td / "c.out", np.int32)
    np.savez_compressed(HERE / "overset.npz", **out)
    print(f"wrote {HERE / 'overset.npz'}: {nv.size} weight cases, "
          f"{sum(v.size for k, v in out.items() if k.endswith('_donor'))} search points")
    ties_cases(np.random.default_rng(20261204))


if __name__ == "__main__":
    main()
