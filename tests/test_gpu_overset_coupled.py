"""Coupled overset solve of one case (cfd_connectivity + the per-step fringe
exchange) against a restatement on the host.

System: a Cartesian background on [-3, 3]^2 and an O-grid around the unit
cylinder out to r = 1.5 (its outer ring is the overset boundary), Euler, M 0.3,
LU-SGS.  The host restatement takes the same connectivity from the standalone
assembly (abi.overset_connect, itself pinned bit for bit to the reference's
assembly by test_gpu_overset_connect.py), steps each mesh with the C oracle
(oracle/cfd_oracle.c) keeping the state of every non-field cell, and runs the
exchange in numpy: cell means at the donor nodes, interpolation of the
receptor nodes, node means into the receptor cells.  Tolerance 1e-11 relative
(the sums are formed in another order on the host).  Graph-replayed coupled
steps give the bits of direct ones.
"""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build_system():
    from tmp_gb300 import meshgen

    bg = meshgen.cart_mesh(40, 40, (-3.0, -3.0), (3.0, 3.0))
    og = meshgen.o_mesh(48, 12, r0=0.5, dr1=0.02, rout=1.5)
    # rotate and shift the O-grid by irrational amounts: no background node on a component edge
    a = np.sqrt(2.0) * 0.01
    R = np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])
    og.xy = og.xy @ R.T + np.array([np.sqrt(3) * 1e-3, np.sqrt(5) * 1e-3])
    obc = np.arange(12 * 48, 13 * 48, dtype=np.int32)  # the outer ring's nodes
    return bg, og, obc


def rel(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_coupled_overset_steps_match_host_restatement(built_lib, built_oracle):
    import oracle
    from oracle import grd
    from tmp_gb300 import abi, meshgen

    bg, og, obc = build_system()
    gms = [bg, og]
    meshes = [abi.Mesh.from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag) for g in gms]
    fs = dict(mach=0.3, aoa_deg=3.0, reynolds=1e6)
    cfl = 5.0
    case = abi.Case(meshes, [fs, fs], abi.FLOW_EULER, abi.ADV_LUSGS, abi.PREC_FP64, cfl=cfl)
    case.init_freestream()
    case.connect(meshes, [None, obc], nfringe=2, mexclude=3)
    ib_dev = [case.iblank(0), case.iblank(1)]
    # the same assembly through the standalone blocks
    blocks = [abi.Block(m) for m in meshes]
    hm = abi.HoleMap(blocks[1])
    asm = abi.overset_connect(blocks, [None, hm], [np.zeros(0, np.int32), obc], nfringe=2, mexclude=3)
    for k in range(2):
        np.testing.assert_array_equal(ib_dev[k], asm["cell_iblank"][k])
    assert (ib_dev[0] == 0).sum() > 0 and (ib_dev[0] == -1).sum() > 0 and (ib_dev[1] == -1).sum() > 0
    # host restatement of the coupled step
    orc, topo = [], []
    with tempfile.TemporaryDirectory() as td:
        for k, g in enumerate(gms):
            p = Path(td) / f"m{k}.grd"
            meshgen.write_grd(p, g)
            t = grd.read_grd(p, g.wall_tag, g.far_tag)
            topo.append(t)
            orc.append(oracle.Oracle(t, 0.3, 3.0, 1e6, False))
    cv = [t.cell_verts.reshape(-1, 4) for t in topo]
    nv = [t.cell_nvert for t in topo]
    nn = [t.nnode for t in topo]
    # node -> cells (ascending) for the donor nodes
    entries = []  # (recv mesh, recv node, donor mesh, nweights, inode, weights)
    for d in range(2):
        it = asm["interp"][d]
        for i in range(len(it["recv_node"])):
            entries.append((int(it["recv_block"][i]), int(it["recv_node"][i]), d, int(it["nweights"][i]),
                            it["inode"][i], it["weights"][i]))
    cells_of = [dict(), dict()]
    for m in range(2):
        for c in range(len(nv[m])):
            for v in cv[m][c, :nv[m][c]]:
                cells_of[m].setdefault(int(v), []).append(c)

    def exchange():
        U = [o.field("U") for o in orc]
        W = [o.field("W") for o in orc]
        qn = [np.zeros((nn[m], 4)) for m in range(2)]
        for (_, _, d, nw, inode, _) in entries:
            for v in inode[:nw]:
                cs = cells_of[d][int(v)]
                s = np.zeros(4)
                for c in cs:
                    s = s + U[d][c]
                qn[d][int(v)] = s / len(cs)
        vals = []
        for (r, node, d, nw, inode, w) in entries:
            q = np.zeros(4)
            for m in range(nw):
                q = q + qn[d][int(inode[m])] * w[m]
            vals.append(q)
        for (r, node, _, _, _, _), q in zip(entries, vals):
            qn[r][node] = q
        for m in range(2):
            for c in np.flatnonzero(ib_dev[m] == -1):
                s = np.zeros(4)
                for v in cv[m][c, :nv[m][c]]:
                    s = s + qn[m][int(v)]
                u = s / nv[m][c]
                U[m][c] = u
                vm = u[2] * u[2] + u[3] * u[3]
                W[m][c] = [u[0], u[1] / (1.4 - 1) + 0.5 * u[0] * vm, u[0] * u[2], u[0] * u[3]]

    nsteps = 12
    for _ in range(nsteps):
        for m, o in enumerate(orc):
            keep = ib_dev[m] != 1
            u0, w0 = o.field("U")[keep].copy(), o.field("W")[keep].copy()
            assert o.lusgs_step(cfl) == 0
            o.field("U")[keep] = u0
            o.field("W")[keep] = w0
        exchange()
    case.step(nsteps)
    case.sync()
    for m in range(2):
        assert rel(case.get("U", m), orc[m].field("U")) <= 1e-11, m
    # holes kept the freestream
    u_bg = case.get("U", 0)
    assert np.all(u_bg[ib_dev[0] == 0] == u_bg[ib_dev[0] == 0][0])
    case.close()


def test_coupled_overset_graph_equals_direct_steps(built_lib):
    from tmp_gb300 import abi

    bg, og, obc = build_system()
    meshes = [abi.Mesh.from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag) for g in (bg, og)]
    fs = dict(mach=0.3, aoa_deg=3.0, reynolds=1e6)
    cases = []
    for _ in range(2):
        c = abi.Case(meshes, [fs, fs], abi.FLOW_EULER, abi.ADV_LUSGS, abi.PREC_MIXFF, cfl=5.0)
        c.init_freestream()
        c.connect(meshes, [None, obc], nfringe=2, mexclude=3)
        cases.append(c)
    cases[0].step_graph(15)
    for _ in range(15):
        cases[1].step(1)
    for c in cases:
        c.sync()
    for m in range(2):
        np.testing.assert_array_equal(cases[0].get("U", m), cases[1].get("U", m))
    # an explicit exchange after the steps leaves the field cells as they are
    ib = cases[0].iblank(0)
    before = cases[0].get("U", 0)
    cases[0].fringe_update()
    cases[0].sync()
    np.testing.assert_array_equal(cases[0].get("U", 0)[ib == 1], before[ib == 1])
    for c in cases:
        c.close()
