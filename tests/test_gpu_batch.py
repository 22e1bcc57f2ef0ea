"""The uneven batch: many independent meshes of different sizes packed in one
case give, mesh by mesh, the same bits as the same meshes run as separate
cases, in every precision form, through the graph-captured step, with the
dataflow sweeps at an autotuned width and with the learned relaxation on.

Packing concatenates the meshes (cell, face and node ids offset per mesh) and
merges their sweep levels; nothing in a step couples two meshes, so any
difference would be a bookkeeping error (a wrong offset, a norm or a sampled
mean taken across meshes).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n=8, seed=77, lo=2_000, hi=12_000):
    from tmp_gb300 import abi, configs

    cases = configs.c5_cases(n, seed=seed, lo=lo, hi=hi)
    meshes = []
    for bc in cases:
        g = bc.grd()
        meshes.append(abi.Mesh.from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag))
    fs = [dict(mach=bc.mach, aoa_deg=bc.aoa, reynolds=bc.re) for bc in cases]
    return cases, meshes, fs


@pytest.mark.parametrize("precision,sweep_mode", [("fp64", 0), ("fp32", 0), ("mixed", 0), ("fp32", 5), ("mixed", 5),
                                                   ("mixff", 5), ("fp32", 6), ("mixff", 6)])
@pytest.mark.parametrize("flow", ["euler", "laminar"])
def test_uneven_batch_packed_matches_separate(precision, sweep_mode, flow):
    from tmp_gb300 import abi

    prec = dict(fp64=abi.PREC_FP64, fp32=abi.PREC_FP32, mixed=abi.PREC_MIXED, mixff=abi.PREC_MIXFF)[precision]
    fl = abi.FLOW_EULER if flow == "euler" else abi.FLOW_LAMINAR
    _, meshes, fs = _batch()
    packed = abi.Case(meshes, fs, fl, abi.ADV_LUSGS, prec, cfl=10.0, sweep_mode=sweep_mode)
    packed.autotune(1)
    packed.init_freestream()
    packed.step_graph(4)
    packed.sync()
    for k, (m, f) in enumerate(zip(meshes, fs)):
        single = abi.Case([m], [f], fl, abi.ADV_LUSGS, prec, cfl=10.0, sweep_mode=sweep_mode)
        single.init_freestream()
        single.step_graph(4)
        single.sync()
        np.testing.assert_array_equal(packed.get("U", mesh=k), single.get("U"), err_msg=f"mesh {k}")
        assert packed.norm("DW_RHO2", mesh=k) == single.norm("DW_RHO2"), f"mesh {k}"
        single.close()
    packed.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixff"])
def test_uneven_batch_sst_packed_matches_separate(precision):
    """The batch's SST half: packed SST meshes (the model's per-mesh freestream turbulence, wall distance per mesh,
    the turbulence sweeps over the merged levels, overlapped with the flow's) give each mesh's separate bits."""
    from tmp_gb300 import abi

    prec = dict(fp64=abi.PREC_FP64, mixed=abi.PREC_MIXED, mixff=abi.PREC_MIXFF)[precision]
    _, meshes, fs = _batch(n=6, seed=91)
    packed = abi.Case(meshes, fs, abi.FLOW_SST, abi.ADV_LUSGS, prec, cfl=10.0)
    packed.init_freestream()
    packed.step_graph(4)
    packed.sync()
    for k, (m, f) in enumerate(zip(meshes, fs)):
        single = abi.Case([m], [f], abi.FLOW_SST, abi.ADV_LUSGS, prec, cfl=10.0)
        single.init_freestream()
        single.step_graph(4)
        single.sync()
        for name in ("U", "SST_T", "SST_MUT"):
            np.testing.assert_array_equal(packed.get(name, mesh=k), single.get(name), err_msg=f"mesh {k} {name}")
        single.close()
    packed.close()


def test_uneven_batch_learned_packed_matches_separate():
    """With the learned relaxation attached, each mesh's pooled factor comes
    from its own sampled cells only.  The relaxation is attached after 30 plain
    steps: over-relaxing the impulsive start diverges on the high-Mach
    cylinders of the batch (the oracle's plain steps with W += 1.6 dW fail
    there at step 2 from the freestream, and pass after the 30 steps)."""
    from tmp_gb300 import abi, learn

    net = learn.load()
    if net is None:
        pytest.skip("no committed relaxation weights")
    _, meshes, fs = _batch()
    packed = abi.Case(meshes, fs, abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_MIXED, cfl=10.0)
    packed.init_freestream()
    packed.step_graph(30)
    abi.case_track(packed, True)
    abi.case_set_mlp(packed, net, False)
    packed.step_graph(5)
    packed.sync()
    for k, (m, f) in enumerate(zip(meshes, fs)):
        single = abi.Case([m], [f], abi.FLOW_LAMINAR, abi.ADV_LUSGS, abi.PREC_MIXED, cfl=10.0)
        single.init_freestream()
        single.step_graph(30)
        abi.case_track(single, True)
        abi.case_set_mlp(single, net, False)
        single.step_graph(5)
        single.sync()
        np.testing.assert_array_equal(packed.get("U", mesh=k), single.get("U"), err_msg=f"mesh {k}")
        single.close()
    packed.close()
