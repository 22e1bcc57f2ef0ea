"""Host-side mesh handling through the C ABI (no GPU needed): .grd parsing,
topology identical to the reference's, LU-SGS level schedule, error paths."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, golden, manifest


@pytest.mark.parametrize("mesh_case", ["omesh_euler_rk5", "mixed_lam_lusgs"])
def test_topology_matches_reference(built_lib, mesh_case):
    from tmp_gb300 import abi

    c = manifest()[mesh_case]
    g = golden(mesh_case)
    m = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    t = m.topology()
    np.testing.assert_array_equal(t["lr"].ravel(), g["topo_lr"])
    np.testing.assert_array_equal(t["cell_edges"].ravel(), g["topo_cedges"])
    np.testing.assert_array_equal(t["cell_verts"].ravel(), g["topo_cverts"])
    np.testing.assert_array_equal(t["cell_sizes"].ravel(), g["topo_csize"])


def test_from_arrays_equals_file(built_lib):
    from tmp_gb300 import abi, meshgen

    gm = meshgen.o_mesh(16, 6, r0=0.5, dr1=0.05, rout=3.0)
    m = abi.Mesh.from_arrays(gm.xy, gm.edge_nodes, gm.edge_cells, gm.ncell, gm.wall_tag, gm.far_tag)
    assert (m.nnode, m.nedge, m.ncell) == (gm.nnode, gm.nedge, gm.ncell)


def _levels_py(topo):
    lr = topo["lr"]
    ce = topo["cell_edges"]
    n = len(ce)
    lf = np.zeros(n, int)
    for c in range(n):
        for e in ce[c]:
            if e < 0:
                continue
            j = lr[e, 1] if lr[e, 0] == c else lr[e, 0]
            if 0 <= j < c:
                lf[c] = max(lf[c], lf[j] + 1)
    lb = np.zeros(n, int)
    for c in range(n - 1, -1, -1):
        for e in ce[c]:
            if e < 0:
                continue
            j = lr[e, 1] if lr[e, 0] == c else lr[e, 0]
            if j > c:
                lb[c] = max(lb[c], lb[j] + 1)
    return lf.max() + 1, lb.max() + 1


def test_level_schedule(built_lib):
    """Level counts equal a direct longest-chain count over lower/upper neighbours;
    a structured O-grid numbered circumferentially has ntheta + nr - 1 levels."""
    from tmp_gb300 import abi, meshgen

    c = manifest()["mixed_lam_lusgs"]
    m = abi.Mesh.load_grd(GOLDEN / c["mesh"], c["wall_tag"], c["far_tag"])
    assert m.levels() == _levels_py(m.topology())
    gm = meshgen.o_mesh(12, 5, r0=0.5, dr1=0.05, rout=3.0)
    mo = abi.Mesh.from_arrays(gm.xy, gm.edge_nodes, gm.edge_cells, gm.ncell, gm.wall_tag, gm.far_tag)
    assert mo.levels() == _levels_py(mo.topology())


def test_missing_file_is_io_error(built_lib, tmp_path):
    from tmp_gb300 import abi

    with pytest.raises(abi.CfdError) as ei:
        abi.Mesh.load_grd(tmp_path / "nope.grd", -1, -2)
    assert ei.value.code == -2


def test_bad_boundary_tag_is_mesh_error(built_lib):
    from tmp_gb300 import abi

    c = manifest()["omesh_euler_rk5"]
    with pytest.raises(abi.CfdError) as ei:
        abi.Mesh.load_grd(GOLDEN / c["mesh"], -7, -8)  # file uses -1/-2
    assert ei.value.code == -3
    assert "boundary" in str(ei.value)


def test_truncated_file_is_mesh_error(built_lib, tmp_path):
    from tmp_gb300 import abi

    src = (GOLDEN / "omesh.grd").read_text().splitlines()
    p = tmp_path / "cut.grd"
    p.write_text("\n".join(src[: len(src) // 2]) + "\n")
    with pytest.raises(abi.CfdError) as ei:
        abi.Mesh.load_grd(p, -1, -2)
    assert ei.value.code == -3


def test_reference_shipped_mesh_if_present(built_lib):
    from oracle.build import reference_root
    from tmp_gb300 import abi

    p = reference_root() / "mix_element_laminar.grd"
    if not p.exists():
        pytest.skip("reference meshes not present")
    m = abi.Mesh.load_grd(p, -1, -2)
    assert (m.nnode, m.nedge, m.ncell) == (40359, 80308, 39949)


def test_uneven_batch_definition():
    """The uneven batch: seeded, sizes log-uniform within the bounds, the
    generated meshes near their target sizes, half Euler and half viscous."""
    from tmp_gb300 import configs

    a, b = configs.c5_cases(), configs.c5_cases()
    assert a == b and len(a) == 256
    t = np.array([c.target_cells for c in a])
    assert t.min() >= 5_000 and t.max() <= 200_000
    # log-uniform: the median of the log sizes sits near the middle of the range
    mid = 0.5 * (np.log(5e3) + np.log(2e5))
    assert abs(np.median(np.log(t)) - mid) < 0.35
    assert [c.flow for c in a].count("euler") == 128
    assert all(0.2 <= c.mach <= 0.8 and -4 <= c.aoa <= 10 and 1e5 <= c.re <= 1e7 for c in a)
    small = configs.c5_cases(6, seed=3, lo=2_000, hi=20_000)
    for c in small:
        g = c.grd()
        assert 0.6 < g.ncell / c.target_cells < 1.6, (c, g.ncell)


@pytest.mark.parametrize("name", ["mixed_lam_lusgs", "omesh_euler_rk5"])
def test_tecplot_node_and_tioga_dumps_match_reference(tmp_path, name):
    """writeNOdeData / writeTiogaFormat layouts, byte for byte against the
    reference's own files (tests/golden/tecplot.npz)."""
    import json

    from tmp_gb300 import abi

    golden = GOLDEN
    c = json.loads((golden / "manifest.json").read_text())[name]
    tec = np.load(golden / "tecplot.npz")
    m = abi.Mesh.load_grd(golden / c["mesh"], c["wall_tag"], c["far_tag"])
    node_q = np.array([[0.001 * i + k for k in range(4)] for i in range(m.nnode)])
    abi.write_node_data(m, str(tmp_path / "nodes"), node_q)
    assert (tmp_path / "nodes_1_1").read_bytes() == bytes(tec[f"{name}/nodes"])
    abi.write_tioga_format(m, str(tmp_path / "tioga"), np.arange(m.ncell) % 3 - 1)
    assert (tmp_path / "tioga00").read_bytes() == bytes(tec[f"{name}/tioga"])
