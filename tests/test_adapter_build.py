"""The reference-side adapter (include/cfdgb_adapter.hpp, the TimeIntegrator a
maintainer of the reference would add) compiles against the reference's own
headers, links with the reference's objects and libcfdgb.so, and hands the
library meshes with the reference's topology (tests/adapter_check.cpp).  Runs
on the CPU where the reference sources are present (no GPU call is made)."""
from __future__ import annotations

import json
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT


def test_adapter_compiles_and_hands_over_reference_topology(built_lib, tmp_path):
    from oracle.build import build_ref, reference_root

    ref = reference_root()
    if not (ref / "src" / "UnstructSolver").is_dir() or shutil.which("g++") is None:
        pytest.skip("reference sources or g++ not present")
    build_ref()
    obj = ROOT / "oracle" / "_ref" / "obj"
    units = ["UnstructSolver_UnstructIntegrator", "UnstructSolver_TopologyHolderStrategy",
             "UnstructSolver_TopologyHolderStrategyOutput", "UnstructSolver_Euler2D", "UnstructSolver_ViscousFlow2D",
             "UnstructSolver_FluxStrategy", "UnstructSolver_LimiterStrategy", "UnstructSolver_TimeIntegrator",
             "UnstructSolver_LUSGS_Integrator", "UnstructSolver_HLLCFluxStrategy", "UnstructSolver_UnstructFeeder",
             "UnstructSolver_commCell", "reader_Reader", "UniTioga_CellBrick", "mathTools_cellVolume",
             "mathTools_vector3d"]
    src = ref / "src"
    shims = ROOT / "oracle" / "shims"
    exe = tmp_path / "adapter_check"
    cmd = ["g++", "-O1", "-std=c++17", "-w", "-include", str(shims / "compat.h"), f"-I{shims}", f"-I{src}",
           f"-I{src / 'UnstructSolver'}", f"-I{src / 'toolBox'}", f"-I{src / 'mathTools'}", f"-I{src / 'UniTioga'}",
           f"-I{src / 'reader'}", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "adapter_check.cpp"),
           *[str(obj / f"{u}.o") for u in units], f"-L{built_lib.parent}", "-lcfdgb",
           f"-Wl,-rpath,{built_lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    for mesh, wall, far in (("mixed.grd", -1, -2), ("omesh.grd", -1, -2)):
        r = subprocess.run([str(exe), str(GOLDEN / mesh), str(wall), str(far)], capture_output=True, text=True)
        assert r.returncode == 0, (r.stdout, r.stderr[-2000:])
        info = json.loads(r.stdout.strip().splitlines()[-1])
        assert info["mismatches"] == 0 and info["cells"] > 0
