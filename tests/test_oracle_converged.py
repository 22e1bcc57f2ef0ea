"""The C restatement (oracle/cfd_oracle.c) against the reference's converged
runs (tests/golden/c1_conv.npz, c2s_conv.npz, written by
make_golden_converged.py from the reference's own serial path): the same
iterations from the freestream give the reference's final field bit for bit
(C1: 2,000 first-order RK iterations on the 8,192-cell O-grid; the small
C2-recipe mesh: LU-SGS at CFL 50 to a 1e-10 fall of the L2 density residual).
"""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import golden


@pytest.mark.parametrize("name", ["c1_conv", "c2s_conv"])
def test_oracle_reproduces_converged_reference(name, built_oracle):
    import oracle
    from oracle import grd
    from tmp_gb300 import meshgen

    g = golden(name)
    m = meshgen.GrdMesh(g["xy"], g["edge_nodes"], g["edge_cells"], int(g["ncell"]), int(g["wall_tag"]),
                        int(g["far_tag"]))
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "m.grd"
        meshgen.write_grd(p, m)
        topo = grd.read_grd(p, m.wall_tag, m.far_tag)
    viscous = name == "c2s_conv"
    o = oracle.Oracle(topo, float(g["mach"]), float(g["aoa"]), float(g["re"]), viscous)
    fo = bool(g["first_order"])
    n = int(g["nsteps"])
    l2 = np.empty(n)
    for k in range(n):
        rc = o.lusgs_step(float(g["cfl"]), fo) if viscous else o.rk_step(fo)
        assert rc == 0
        r = o.field("R")[:, 0]
        l2[k] = np.sqrt(np.sum(r * r) / m.ncell)
    np.testing.assert_array_equal(o.field("U").view(np.int64), g["end_U"].view(np.int64))
    np.testing.assert_array_equal(l2, g["l2_hist"])
    if viscous:
        assert l2[-1] <= 1e-10 * l2[0]
