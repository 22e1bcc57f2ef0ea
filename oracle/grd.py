"""Pure-Python restatement of the reference's .grd reader (test oracle).

Follows UnstructReader::readForUnstruct (reader/UnstructReader.h:124-272):
cells are assembled edge by edge in file order with Brick4Cobalt2D::insert
(UniTioga/CellBrick.cpp:13-136), each cell's edge list is filled in edge order,
negative right-cell codes map to WALL (-2) / FARFIELD (-3).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

WALL, FARFIELD = -2, -3


@dataclass
class Topo:
    nnode: int
    nedge: int
    ncell: int
    xy: np.ndarray           # (nnode*2,) float64
    edge_nodes: np.ndarray   # (nedge*2,) int32, 0-based
    lr: np.ndarray           # (nedge*2,) int32
    cell_verts: np.ndarray   # (ncell*4,) int32
    cell_nvert: np.ndarray   # (ncell,) int32
    cell_edges: np.ndarray   # (ncell*4,) int32
    cell_nedge: np.ndarray   # (ncell,) int32


def _insert(nodes: list, state: list, e0: int, e1: int) -> None:
    """Brick4Cobalt2D::insert; state = [size, closed]."""
    size, closed = state
    if closed:
        return
    if size == 0:
        nodes[0], nodes[1] = e0, e1
        state[0] = 2
        return
    e = (e0, e1)
    idx = []
    for i in range(4):
        for j in range(2):
            if nodes[i] == e[j]:
                idx += [i, j]
    if not idx:
        return
    if len(idx) == 2:
        if idx[0] < 2:
            nodes[3 - idx[0]] = e[1 - idx[1]]
        else:
            nodes[5 - idx[0]] = e[1 - idx[1]]
        state[0] = size + 1
        if state[0] == 4:
            state[1] = True
        return
    if size == 3 and nodes[2] == -1 and nodes[3] != -1:
        nodes[2], nodes[3] = nodes[3], -1
    state[1] = True


def topo_from_arrays(xy, edge_nodes_1b, edge_cells_1b, ncell: int, wall_tag: int, far_tag: int) -> Topo:
    xy = np.asarray(xy, np.float64).reshape(-1)
    en = np.asarray(edge_nodes_1b, np.int64).reshape(-1, 2)
    ec = np.asarray(edge_cells_1b, np.int64).reshape(-1, 2)
    nedge = len(en)
    nodes = [[-1, -1, -1, -1] for _ in range(ncell)]
    state = [[0, False] for _ in range(ncell)]
    cedges = np.full((ncell, 4), -1, np.int32)
    cne = np.zeros(ncell, np.int32)
    lr = np.zeros((nedge, 2), np.int32)
    for i in range(nedge):
        n0, n1 = int(en[i, 0]), int(en[i, 1])
        l, r = int(ec[i, 0]), int(ec[i, 1])
        if l <= 0:
            raise ValueError("Left cell can't be negative")
        _insert(nodes[l - 1], state[l - 1], n0, n1)
        if r > 0:
            _insert(nodes[r - 1], state[r - 1], n0, n1)
        lr[i, 0] = l - 1
        cedges[l - 1, cne[l - 1]] = i
        cne[l - 1] += 1
        if r > 0:
            lr[i, 1] = r - 1
            cedges[r - 1, cne[r - 1]] = i
            cne[r - 1] += 1
        elif r == wall_tag:
            lr[i, 1] = WALL
        elif r == far_tag:
            lr[i, 1] = FARFIELD
        else:
            raise ValueError("Not a valid boundary type")
    cv = np.full((ncell, 4), -1, np.int32)
    cnv = np.zeros(ncell, np.int32)
    for c in range(ncell):
        cnv[c] = state[c][0]
        for j in range(state[c][0]):
            cv[c, j] = nodes[c][j] - 1
    return Topo(len(xy) // 2, nedge, ncell, xy, (en - 1).astype(np.int32).reshape(-1), lr.reshape(-1),
                cv.reshape(-1), cnv, cedges.reshape(-1), cne)


def read_grd(path, wall_tag: int, far_tag: int) -> Topo:
    with open(path) as f:
        tok = f.read().split()
    p = 3
    nnode, nedge, ncell = int(tok[p]), int(tok[p + 1]), int(tok[p + 2])
    p += 5
    xy = np.array(tok[p:p + 2 * nnode], dtype=np.float64)
    p += 2 * nnode
    rec = np.array(tok[p:p + 5 * nedge], dtype=np.int64).reshape(nedge, 5)
    if (rec[:, 0] != 2).any():
        raise ValueError("2D edges need 2 nodes")
    return topo_from_arrays(xy, rec[:, 1:3], rec[:, 3:5], ncell, wall_tag, far_tag)
