"""Generate tests/golden/overset_connect.npz from the reference's own overset
assembly code.

Runs `oracle/_ref/ref_overset connect` (the reference's MeshBlock::preprocess,
getHoleMap, search, processDonors, findInterpData, cancellations and
reduce_fringes, compiled from its sources by oracle/build_ref.sh, in the order
one rank of tioga::performConnectivity runs them) on seeded overset systems:

  cyl     a Cartesian background and a cylinder O-grid (wall inside, overset
          boundary on its outer ring), nfringe 1, mexclude 3 (tioga's defaults)
  cyl2    the same pair with nfringe 2, mexclude 1
  naca    a background and a mixed quad/triangle mesh around a NACA 0012
          section
  three   a background and two overlapping cylinder O-grids (donor lists with
          several candidates)

  tcyl    the cylinder pair unrotated and centred on a background node: nodes
          of each mesh lie on edges and radial lines of the other, so many
          points lie in two or more cells (the donor is the first containing
          cell of the reference's tree walk)
  tthree  the three-mesh system with its O-grids unrotated and centred on
          background nodes

The other component grids are rotated and shifted by irrational amounts, so
that every node lies inside one cell only.  Each case stores every block's .grd arrays, wall
and overset-boundary nodes, and the reference's node iblank, cell iblank and
surviving interpolations per donor block.

usage: python tests/golden/make_golden_connect.py [REFERENCE_ROOT]
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

from oracle import grd  # noqa: E402
from tmp_gb300 import meshgen  # noqa: E402

DRV = ROOT / "oracle" / "_ref" / "ref_overset"


def transform(g: meshgen.GrdMesh, ang: float, shift) -> meshgen.GrdMesh:
    R = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
    return meshgen.GrdMesh(g.xy @ R.T + np.asarray(shift), g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag)


def topo(g):
    return grd.topo_from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag)


def bnodes(t, code):
    lr = t.lr.reshape(-1, 2)
    en = t.edge_nodes.reshape(-1, 2)
    return np.unique(en[lr[:, 1] == code].reshape(-1)).astype(np.int32)


def run_connect(topos, walls, obcs, nfringe, mexclude, isym=3):
    with tempfile.TemporaryDirectory() as td:
        with open(Path(td) / "c.bin", "wb") as f:
            np.array([len(topos), nfringe, mexclude, isym], np.int32).tofile(f)
            for t, w, o in zip(topos, walls, obcs):
                xy = t.xy.reshape(-1)
                np.array([len(xy) // 2, len(t.cell_nvert)], np.int32).tofile(f)
                xy.astype(np.float64).tofile(f)
                np.asarray(t.cell_nvert, np.int32).tofile(f)
                np.asarray(t.cell_verts, np.int32).reshape(-1).tofile(f)
                np.array([len(w)], np.int32).tofile(f)
                np.asarray(w, np.int32).tofile(f)
                np.array([len(o)], np.int32).tofile(f)
                np.asarray(o, np.int32).tofile(f)
        subprocess.run([str(DRV), "connect", "c.bin", "o.bin"], check=True, cwd=td, stdout=subprocess.DEVNULL)
        b = (Path(td) / "o.bin").read_bytes()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(b, dt, n, off).copy()
        off += a.nbytes
        return a

    ibl, iblc = [], []
    for t in topos:
        ibl.append(take(np.int32, len(t.xy.reshape(-1)) // 2))
        iblc.append(take(np.int32, len(t.cell_nvert)))
    interps = []
    for _ in topos:
        n = int(take(np.int32, 1)[0])
        recs = np.zeros((n, 12), np.int32)
        w = np.zeros((n, 4))
        for i in range(n):
            recs[i, :4] = take(np.int32, 4)
            recs[i, 4:8] = take(np.int32, 4)
            w[i] = take(np.float64, 4)
        interps.append((recs[:, :8], w))
    assert off == len(b)
    return ibl, iblc, interps


def cases():
    bg = meshgen.cart_mesh(64, 64, lo=(-3.0, -3.0), hi=(3.0, 3.0))
    cyl = transform(meshgen.o_mesh(48, 16, r0=0.5, dr1=0.01, rout=1.5), 0.1234567, (0.0317, -0.0213))
    yield "cyl", [bg, cyl], 1, 3
    yield "cyl2", [bg, cyl], 2, 1
    body = meshgen.naca_body(64)
    naca = transform(meshgen.mixed_mesh(body, nlayer=6, dr1=0.004, growth=1.3, rfar=0.9, seed=21, density=1.0,
                                        grade=1.0), 0.05123, (-0.4711, 0.0123))
    bg2 = meshgen.cart_mesh(72, 48, lo=(-1.8, -1.2), hi=(1.8, 1.2))
    yield "naca", [bg2, naca], 1, 3
    c2 = transform(meshgen.o_mesh(40, 12, r0=0.3, dr1=0.01, rout=1.0), 0.3141, (1.0371, 0.4129))
    c3 = transform(meshgen.o_mesh(40, 12, r0=0.3, dr1=0.01, rout=1.0), 1.2345, (-0.5213, -0.3377))
    yield "three", [bg, c2, c3], 1, 3
    # background nodes lie on multiples of 6/64 = 0.09375, all exact binary fractions
    yield "tcyl", [bg, meshgen.o_mesh(48, 16, r0=0.5, dr1=0.01, rout=1.5)], 1, 3
    t2 = transform(meshgen.o_mesh(40, 12, r0=0.3, dr1=0.01, rout=1.0), 0.0, (0.9375, 0.375))
    t3 = transform(meshgen.o_mesh(40, 12, r0=0.3, dr1=0.01, rout=1.0), 0.0, (-0.75, -0.5625))
    yield "tthree", [bg, t2, t3], 1, 3


def main():
    out = {}
    names = []
    for name, meshes, nfringe, mexclude in cases():
        topos = [topo(g) for g in meshes]
        walls = [bnodes(t, -2) for t in topos]
        obcs = [np.zeros(0, np.int32)] + [bnodes(t, -3) for t in topos[1:]]
        ibl, iblc, interps = run_connect(topos, walls, obcs, nfringe, mexclude)
        names.append(name)
        out[f"{name}/nblocks"] = np.int32(len(meshes))
        out[f"{name}/nfringe"] = np.int32(nfringe)
        out[f"{name}/mexclude"] = np.int32(mexclude)
        for k, (g, t) in enumerate(zip(meshes, topos)):
            p = f"{name}/{k}/"
            out[p + "xy"] = g.xy
            out[p + "edge_nodes"] = g.edge_nodes
            out[p + "edge_cells"] = g.edge_cells
            out[p + "ncell"] = np.int32(g.ncell)
            out[p + "tags"] = np.array([g.wall_tag, g.far_tag], np.int32)
            out[p + "cell_verts"] = np.asarray(t.cell_verts, np.int32).reshape(-1, 4)
            out[p + "cell_nvert"] = np.asarray(t.cell_nvert, np.int32)
            out[p + "wall"] = walls[k]
            out[p + "obc"] = obcs[k]
            out[p + "iblank"] = ibl[k]
            out[p + "cell_iblank"] = iblc[k]
            out[p + "interp_int"] = interps[k][0]
            out[p + "interp_w"] = interps[k][1]
        print(name, [{v: int((i == v).sum()) for v in (-1, 0, 1)} for i in ibl], [len(x[0]) for x in interps])
    out["cases"] = np.array(names)
    np.savez_compressed(HERE / "overset_connect.npz", **out)


if __name__ == "__main__":
    main()
