"""Synthetic 2D meshes in the reference's .grd topology, and a .grd writer.

Edges are emitted so that the unit normal (dy, -dx)/|d| of the directed edge
p0->p1 points out of the left cell (edge3d::find_normal, toolBox/edge3d_int.h:
200-210), interior edges have left < right cell id, and boundary edges carry
the file's wall / far-field tags.  Cells are numbered in the order the
generator makes them; that order is the LU-SGS sweep order.

Generators:
  o_mesh       structured O-grid around a circular cylinder (quads)
  mixed_mesh   quad layers around a body + seeded Delaunay triangle fill
  naca_body    NACA 4-digit symmetric thickness (public closed form) as a body
  cart_mesh    Cartesian block of quads
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

WALL_TAG = -1   # tags written into generated files
FAR_TAG = -2


@dataclass
class GrdMesh:
    xy: np.ndarray          # (nnode, 2) float64
    edge_nodes: np.ndarray  # (nedge, 2) int32, 1-based
    edge_cells: np.ndarray  # (nedge, 2) int32, 1-based cells or tags
    ncell: int
    wall_tag: int = WALL_TAG
    far_tag: int = FAR_TAG

    @property
    def nnode(self) -> int:
        return len(self.xy)

    @property
    def nedge(self) -> int:
        return len(self.edge_nodes)


def _signed_area(xy: np.ndarray, cells: np.ndarray, nv: np.ndarray) -> np.ndarray:
    a = np.zeros(len(cells))
    for k in range(cells.shape[1]):
        i0 = cells[:, k]
        i1 = np.where(k + 1 < nv, cells[:, (k + 1) % cells.shape[1]], cells[:, 0])
        valid = k < nv
        x0, y0 = xy[i0, 0], xy[i0, 1]
        x1, y1 = xy[i1, 0], xy[i1, 1]
        a += np.where(valid, x0 * y1 - x1 * y0, 0.0)
    return 0.5 * a


def cells_to_grd(xy: np.ndarray, cells: np.ndarray, nv: np.ndarray, boundary_tag) -> GrdMesh:
    """Build the edge list of a polygonal mesh.

    cells: (ncell, 4) 0-based vertex ids (-1 padded), nv: vertices per cell.
    boundary_tag(mid_xy) -> file tag for each boundary edge (array in, array out).
    """
    xy = np.asarray(xy, np.float64)
    cells = np.asarray(cells, np.int64).copy()
    nv = np.asarray(nv, np.int64)
    # orient every cell counter-clockwise
    flip = _signed_area(xy, cells, nv) < 0
    for c in np.nonzero(flip)[0]:
        k = nv[c]
        cells[c, :k] = cells[c, :k][::-1]
    ncell = len(cells)
    # half edges (cell, local index, a, b) with the cell on the left of a->b
    hc, hk, ha, hb = [], [], [], []
    for k in range(4):
        m = k < nv
        cid = np.nonzero(m)[0]
        a = cells[cid, k]
        nxt = np.where(k + 1 < nv[cid], (k + 1) % 4, 0)
        b = cells[cid, nxt]
        hc.append(cid); hk.append(np.full(len(cid), k)); ha.append(a); hb.append(b)
    hc = np.concatenate(hc); hk = np.concatenate(hk); ha = np.concatenate(ha); hb = np.concatenate(hb)
    nn = len(xy)
    key = np.minimum(ha, hb) * nn + np.maximum(ha, hb)
    order = np.lexsort((hc, key))
    key_s = key[order]
    first = np.ones(len(key_s), bool)
    first[1:] = key_s[1:] != key_s[:-1]
    starts = np.nonzero(first)[0]
    counts = np.diff(np.append(starts, len(key_s)))
    if counts.max() > 2:
        raise ValueError("an edge is shared by more than two cells")
    h0 = order[starts]                      # half edge of the lower cell id (sorted by hc within key)
    pair = counts == 2
    h1 = np.full(len(starts), -1)
    h1[pair] = order[starts[pair] + 1]
    l = hc[h0]
    r = np.where(pair, hc[np.maximum(h1, 0)], -1)
    a = ha[h0]
    b = hb[h0]
    tags = np.zeros(len(starts), np.int64)
    bnd = ~pair
    if bnd.any():
        mid = 0.5 * (xy[a[bnd]] + xy[b[bnd]])
        tags[bnd] = boundary_tag(mid)
    # order edges by (left cell, local index) for locality
    eorder = np.lexsort((hk[h0], l))
    l, r, a, b, tags, pair = l[eorder], r[eorder], a[eorder], b[eorder], tags[eorder], pair[eorder]
    edge_nodes = np.stack([a + 1, b + 1], 1).astype(np.int32)
    edge_cells = np.stack([l + 1, np.where(pair, r + 1, tags)], 1).astype(np.int32)
    return GrdMesh(xy, edge_nodes, edge_cells, ncell)


def write_grd(path, m: GrdMesh) -> None:
    """Write the .grd text layout read by UnstructReader::readForUnstruct."""
    with open(path, "w") as f:
        f.write("2   1  2\n")
        f.write(f"{m.nnode} {m.nedge} {m.ncell} 2 4\n")
        np.savetxt(f, m.xy, fmt="%24.16e")
        out = np.column_stack([np.full(m.nedge, 2), m.edge_nodes, m.edge_cells])
        np.savetxt(f, out, fmt="%d")


def geometric_radii(r0: float, dr1: float, n: int, rout: float | None = None, ratio: float | None = None):
    """n+1 radii from r0: first spacing dr1, geometric growth.  When rout is
    given the growth ratio is solved so the last radius is rout."""
    if rout is not None:
        lo, hi = 1.0 + 1e-12, 4.0
        for _ in range(200):
            q = 0.5 * (lo + hi)
            s = dr1 * (q ** n - 1) / (q - 1)
            if r0 + s > rout:
                hi = q
            else:
                lo = q
        ratio = 0.5 * (lo + hi)
    r = [r0]
    h = dr1
    for _ in range(n):
        r.append(r[-1] + h)
        h *= ratio
    r = np.array(r)
    if rout is not None:
        r[-1] = rout
    return r, ratio


def o_mesh(ntheta: int, nr: int, r0: float = 0.5, dr1: float = 1e-3, rout: float = 20.0,
           ratio: float | None = None) -> GrdMesh:
    """Structured O-grid around a cylinder of radius r0: ntheta x nr quads,
    cell id = j*ntheta + i (circumferential index fastest).  Wall on r0, far field
    on the outer ring."""
    r, _ = geometric_radii(r0, dr1, nr, rout if ratio is None else None, ratio)
    th = 2 * np.pi * np.arange(ntheta) / ntheta
    xy = np.stack([np.outer(r, np.cos(th)).ravel(), np.outer(r, np.sin(th)).ravel()], 1)
    j, i = np.meshgrid(np.arange(nr), np.arange(ntheta), indexing="ij")
    i, j = i.ravel(), j.ravel()
    ip = (i + 1) % ntheta
    cells = np.stack([j * ntheta + i, j * ntheta + ip, (j + 1) * ntheta + ip, (j + 1) * ntheta + i], 1)
    rmid = 0.5 * (r0 + r[-1])
    tag = lambda mid: np.where(np.hypot(mid[:, 0], mid[:, 1]) < rmid, WALL_TAG, FAR_TAG)
    return cells_to_grd(xy, cells, np.full(len(cells), 4), tag)


def naca_body(n: int, t: float = 0.12, chord: float = 1.0) -> np.ndarray:
    """Closed NACA 00xx contour (sharp trailing edge variant of the public
    thickness formula), n points counter-clockwise starting at the trailing edge."""
    beta = np.linspace(0, 2 * np.pi, n, endpoint=False)
    x = 0.5 * (1 + np.cos(beta))  # 1 -> 0 -> 1
    yt = 5 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)
    y = np.where(beta <= np.pi, yt, -yt)
    return np.stack([x * chord, y * chord], 1)


def layered_quads(body: np.ndarray, nlayer: int, dr1: float, growth: float, hmax: float | None = None):
    """Quad layers grown along smoothed outward normals of a closed CCW body
    contour; layer thickness starts at dr1 and grows by `growth` up to hmax.
    Returns node coordinates (layer-major) and the outer ring."""
    n = len(body)
    pts = [body]
    cur = body.copy()
    h = dr1
    for k in range(nlayer):
        prv = np.roll(cur, 1, 0)
        nxt = np.roll(cur, -1, 0)
        t = nxt - prv
        nrm = np.stack([t[:, 1], -t[:, 0]], 1)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        # smooth the marching direction (a few Laplacian passes) to avoid crossings at sharp corners
        for _ in range(4 + k // 4):
            nrm = 0.25 * np.roll(nrm, 1, 0) + 0.5 * nrm + 0.25 * np.roll(nrm, -1, 0)
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        cur = cur + h * nrm
        pts.append(cur)
        h *= growth
        if hmax is not None:
            h = min(h, hmax)
    xy = np.concatenate(pts, 0)
    return xy, n


def mixed_mesh(body: np.ndarray, nlayer: int, dr1: float, growth: float, rfar: float, seed: int = 0,
               density: float = 1.0, grade: float = 1.0, hmax: float | None = None) -> GrdMesh:
    """Quad layers around `body` (structured sweep numbering: along the body
    fastest, then outward), then a seeded Delaunay triangle fill out to a circle
    of radius rfar centred on the body's centroid; triangles keep the order in
    which the triangulation returns them."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    qxy, n = layered_quads(body, nlayer, dr1, growth, hmax)
    j, i = np.meshgrid(np.arange(nlayer), np.arange(n), indexing="ij")
    i, j = i.ravel(), j.ravel()
    ip = (i + 1) % n
    qcells = np.stack([j * n + i, j * n + ip, (j + 1) * n + ip, (j + 1) * n + i], 1)
    ring = qxy[nlayer * n:]
    ring_ids = np.arange(nlayer * n, (nlayer + 1) * n)
    ctr = body.mean(0)
    rr = np.hypot(*(ring - ctr).T)
    r_in = rr.max()
    seg = np.linalg.norm(np.roll(ring, -1, 0) - ring, axis=1)
    h0 = seg.mean() / density
    # seeded points on jittered concentric rings; spacing grows ~ r^grade
    pts = []
    r = r_in + h0
    while True:
        h = h0 * (r / r_in) ** grade
        if r > rfar - 0.5 * h:
            break
        m = max(8, int(round(2 * np.pi * r / h)))
        ang = 2 * np.pi * (np.arange(m) + rng.uniform(-0.3, 0.3, m)) / m + rng.uniform(0, 2 * np.pi)
        rad = r + rng.uniform(-0.15, 0.15, m) * h
        pts.append(np.stack([ctr[0] + rad * np.cos(ang), ctr[1] + rad * np.sin(ang)], 1))
        r += h
    hfar = h0 * (rfar / r_in) ** grade
    mfar = max(16, int(round(2 * np.pi * rfar / hfar)))
    af = 2 * np.pi * np.arange(mfar) / mfar
    pts.append(np.stack([ctr[0] + rfar * np.cos(af), ctr[1] + rfar * np.sin(af)], 1))
    outer = np.concatenate(pts, 0)
    # keep exterior points clear of the quad block's outer ring
    d_ring = np.min(np.hypot(*(outer[:, None, :] - ring[None, ::max(1, n // 256), :]).transpose(2, 0, 1)), 1) \
        if len(outer) * (n // max(1, n // 256)) < 5e7 else np.full(len(outer), np.inf)
    outer = outer[(np.hypot(*(outer - ctr).T) > r_in + 0.6 * h0) & (d_ring > 0.6 * h0)]
    allp = np.concatenate([ring, outer], 0)
    tri = Delaunay(allp).simplices
    nring = len(ring)
    inside = (tri < nring).all(1)
    tri = tri[~inside]
    # map local ids: ring -> quad outer ring nodes, others appended after the quad nodes
    gid = np.concatenate([ring_ids, len(qxy) + np.arange(len(outer))])
    tri_g = gid[tri]
    xy = np.concatenate([qxy, outer], 0)
    cells = np.concatenate([qcells, np.column_stack([tri_g, np.full(len(tri_g), -1)])], 0)
    nv = np.concatenate([np.full(len(qcells), 4), np.full(len(tri_g), 3)])
    body_r = np.hypot(*(body - ctr).T).max()
    tag = lambda mid: np.where(np.hypot(*(mid - ctr).T) < 0.5 * (body_r + rfar), WALL_TAG, FAR_TAG)
    m = cells_to_grd(xy, cells, nv, tag)
    # every ring edge must be shared by one quad and one triangle
    if (m.edge_cells[:, 1] < 0).sum() != n + mfar:
        raise RuntimeError("triangle fill does not conform to the quad block; change seed or density")
    return m


def cart_mesh(nx: int, ny: int, lo=(-10.0, -10.0), hi=(10.0, 10.0)) -> GrdMesh:
    """Cartesian quads, cell id = j*nx + i; every outer edge is far field."""
    x = np.linspace(lo[0], hi[0], nx + 1)
    y = np.linspace(lo[1], hi[1], ny + 1)
    X, Y = np.meshgrid(x, y)
    xy = np.stack([X.ravel(), Y.ravel()], 1)
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i, j = i.ravel(), j.ravel()
    w = nx + 1
    cells = np.stack([j * w + i, j * w + i + 1, (j + 1) * w + i + 1, (j + 1) * w + i], 1)
    return cells_to_grd(xy, cells, np.full(len(cells), 4), lambda mid: np.full(len(mid), FAR_TAG))


def perturbed_state(ncell: int, centers: np.ndarray, fs_prim: np.ndarray, amp: float = 0.05, seed: int = 0):
    """Smooth seeded perturbation of a freestream primitive state [rho, p, u, v]
    (keeps rho, p > 0) to exercise every branch of the residual."""
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.5, 3.0, (4, 2))
    ph = rng.uniform(0, 2 * np.pi, 4)
    U = np.tile(fs_prim, (ncell, 1)).astype(np.float64)
    for q in range(4):
        wave = np.sin(k[q, 0] * centers[:, 0] + k[q, 1] * centers[:, 1] + ph[q])
        scale = 1.0 if q < 2 else max(abs(fs_prim[2]), abs(fs_prim[3]), 0.3)
        U[:, q] += amp * scale * wave
    U[:, 0] = np.maximum(U[:, 0], 0.2)
    U[:, 1] = np.maximum(U[:, 1], 0.2)
    return U
