"""Overset assembly on the GPU (cfd_overset_connect) against the reference's
own assembly code: node iblank, cell iblank and the surviving interpolation
lists, bit for bit, on the systems of tests/golden/overset_connect.npz
(background + cylinder O-grid with two fringe settings, background + mixed
mesh around an airfoil, background + two overlapping O-grids, and the
cylinder and three-mesh systems unrotated on background nodes, where many
nodes lie in two or more donor cells).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gc():
    return np.load(GOLDEN / "overset_connect.npz")


@pytest.mark.parametrize("case", ["cyl", "cyl2", "naca", "three", "tcyl", "tthree"])
def test_connect_matches_reference(built_lib, gc, case):
    from tmp_gb300 import abi

    nb = int(gc[f"{case}/nblocks"])
    meshes, blocks, maps, obcs = [], [], [], []
    for k in range(nb):
        p = f"{case}/{k}/"
        t = gc[p + "tags"]
        m = abi.Mesh.from_arrays(gc[p + "xy"], gc[p + "edge_nodes"], gc[p + "edge_cells"], int(gc[p + "ncell"]),
                                 int(t[0]), int(t[1]))
        topo = m.topology()
        assert np.array_equal(topo["cell_verts"], gc[p + "cell_verts"])  # the vertex orders the reference saw
        b = abi.Block(m)
        meshes.append(m)
        blocks.append(b)
        maps.append(abi.HoleMap(b) if len(gc[p + "wall"]) else None)
        obcs.append(gc[p + "obc"])
    out = abi.overset_connect(blocks, maps, obcs, nfringe=int(gc[f"{case}/nfringe"]),
                              mexclude=int(gc[f"{case}/mexclude"]))
    for k in range(nb):
        p = f"{case}/{k}/"
        np.testing.assert_array_equal(out["iblank"][k], gc[p + "iblank"], err_msg=f"block {k} node iblank")
        np.testing.assert_array_equal(out["cell_iblank"][k], gc[p + "cell_iblank"], err_msg=f"block {k} cell iblank")
        ref_i, ref_w = gc[p + "interp_int"], gc[p + "interp_w"]
        it = out["interp"][k]
        got = np.column_stack([it["recv_block"], it["recv_node"], it["donor_cell"], it["nweights"], it["inode"]])
        np.testing.assert_array_equal(got, ref_i, err_msg=f"donor block {k} interpolation list")
        assert np.array_equal(it["weights"].view(np.int64), ref_w.view(np.int64)), f"donor block {k} weights"
    # the receptor counts agree with the lists the donors serve
    for k in range(nb):
        served = sum(int((out["interp"][d]["recv_block"] == k).sum()) for d in range(nb))
        assert served == int((out["iblank"][k] == -1).sum())
