"""Host-side chain schedule of the binary32 LU-SGS sweep (sweep modes 5 and 6),
checked without a GPU: the invariants that the sweep's results and its freedom
from deadlock rest on.

* every cell appears once; each list is in non-decreasing level order;
* each slot records the neighbour the reference's SolveDF waits for (the lower-
  indexed face neighbour forward, the higher-indexed one backward) and the
  cell's signed face code;
* every dependency lies on a strictly lower level (so the lowest unfinished
  cell can always proceed when all warps are co-resident);
* a slot marked "registers" waits for the list's previous cell or the one
  before, and a slot encoded as a shared-memory table entry waits for a cell
  of the same block at exactly that entry (and every such same-block
  dependency whose producer sits below the table's cap is encoded so when the
  table is on); the entries fit the table.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, manifest


def _meshes():
    from tmp_gb300 import abi, learn

    out = []
    seen = set()
    for name, c in manifest().items():
        if c["mesh"] in seen:
            continue
        seen.add(c["mesh"])
        out.append((c["mesh"], abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])))
    spec = learn.CaseSpec(nbody=96, nlayer=24, seed=12, dr1=5e-3, growth=1.05, rfar=30.0)
    out.append(("cylinder", spec.mesh()))
    return out


MESHES = None


def meshes():
    global MESHES
    if MESHES is None:
        MESHES = _meshes()
    return MESHES


def _face_codes_and_deps(mesh, fwd):
    t = mesh.topology()
    lr, ce, sizes = t["lr"], t["cell_edges"], t["cell_sizes"]
    nc = mesh.ncell
    code = np.zeros((nc, 4), np.int64)
    dep = np.full((nc, 4), -1, np.int64)
    for c in range(nc):
        for s in range(sizes[c][1]):
            e = ce[c][s]
            left = lr[e][0] == c
            code[c, s] = e + 1 if left else -(e + 1)
            nbr = lr[e][1] if left else lr[e][0]
            if (fwd and 0 <= nbr < c) or (not fwd and nbr > c):
                dep[c, s] = nbr
    lev = np.zeros(nc, np.int64)
    for c in (range(nc) if fwd else range(nc - 1, -1, -1)):
        d = dep[c][dep[c] >= 0]
        lev[c] = (lev[d].max() + 1) if len(d) else 0
    return code, dep, lev


@pytest.mark.parametrize("fwd", [True, False])
@pytest.mark.parametrize("nlists,local,table", [(8, False, False), (64, False, False), (64, True, False),
                                               (64, True, True), (456 * 8, True, True), (64, True, 97),
                                               (16, True, 300)])
def test_chain_schedule_invariants(built_lib, fwd, nlists, local, table):
    for name, mesh in meshes():
        nc = mesh.ncell
        code, dep, lev = _face_codes_and_deps(mesh, fwd)
        sch = mesh.chain_schedule(fwd, nlists, local, table)
        hptr, cells, rec, jenc = sch["hptr"], sch["cells"], sch["rec"], sch["jenc"]
        assert hptr[0] == 0 and hptr[-1] == nc and np.all(np.diff(hptr) >= 0), name
        cell = cells[:, 0].astype(np.int64)
        assert np.array_equal(np.sort(cell), np.arange(nc)), name
        pos = np.empty(nc, np.int64)
        pos[cell] = np.arange(nc)
        lst = np.repeat(np.arange(nlists), np.diff(hptr))
        # lists in non-decreasing level order
        same = lst[1:] == lst[:-1]
        assert np.all(lev[cell][1:][same] >= lev[cell][:-1][same]), name
        # slots: the reference's dependency and face code
        assert np.array_equal(rec[:, :, 0], dep[cell]), name
        assert np.array_equal(rec[:, :, 1], code[cell]), name
        j = rec[:, :, 0].astype(np.int64)
        has = j >= 0
        # every dependency on a strictly lower level
        assert np.all(lev[j[has]] < np.repeat(lev[cell], 4).reshape(-1, 4)[has]), name
        bits = (cells[:, 1][:, None] >> (2 * np.arange(4))[None, :]) & 3
        tbl = sch["table_entries"]
        for q, s in zip(*np.nonzero(has)):
            b, e, jj = bits[q, s], jenc[q, s], j[q, s]
            h = lst[q]
            if b == 1:
                assert q >= 1 and lst[q - 1] == h and cell[q - 1] == jj and e == -2, (name, q, s)
            elif b == 2:
                assert q >= 2 and lst[q - 2] == h and cell[q - 2] == jj and e == -3, (name, q, s)
            else:
                pj = pos[jj]
                same_block = lst[pj] // 8 == h // 8
                rel = pj - hptr[8 * (h // 8)]
                if table is not False and local and same_block and rel < tbl:
                    t = -4 - e
                    assert e <= -4 and t == rel and 0 <= t < tbl, (name, q, s)
                else:
                    assert e == jj, (name, q, s)
        assert np.all(jenc[~has] == -1), name
        if local and table is not False:
            blocks = hptr[8::8] - hptr[:-1:8]
            cap = blocks.max() if table is True else min(blocks.max(), table)
            assert tbl == cap, name
        else:
            assert tbl == 0, name


def test_chain_schedule_rejects_bad_list_counts(built_lib):
    from tmp_gb300 import abi

    _, mesh = meshes()[0]
    for n in (0, 12):
        with pytest.raises(abi.CfdError):
            mesh.chain_schedule(True, n)
