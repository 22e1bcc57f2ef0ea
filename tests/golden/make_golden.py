"""Generate the golden fixtures in this directory from the reference solver itself.

Runs the reference's own serial path (built from its sources by
oracle/build_ref.sh into oracle/_ref/ref_driver) on small generated meshes and
stores every dumped array in one .npz per case, next to the .grd mesh it used.
The fixtures pin both the C restatement in oracle/ and the CUDA kernels.

usage: python tests/golden/make_golden.py [REFERENCE_ROOT [sst]]   ("sst": only the SST fixtures)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from tmp_gb300 import meshgen  # noqa: E402

# name -> (mesh, flow, advance, mach, aoa, re, cfl, nsteps, perturb seed, first_order)
CASES = {
    "omesh_euler_rk5": ("omesh", "euler", "rk5", 0.3, 0.0, 1e6, 0.8, 3, 1, 0),
    "omesh_euler_rk5_sup": ("omesh", "euler", "rk5", 1.5, 5.0, 1e6, 0.8, 2, 2, 0),
    "omesh_euler_lusgs": ("omesh", "euler", "lusgs", 0.5, 2.0, 1e6, 5.0, 3, 3, 0),
    "omesh_euler_rk5_o1": ("omesh", "euler", "rk5", 0.3, 0.0, 1e6, 0.8, 2, 4, 1),
    "mixed_lam_lusgs": ("mixed", "viscous", "lusgs", 0.2, 0.0, 40.0, 50.0, 3, 5, 0),
    "mixed_lam_rk5": ("mixed", "viscous", "rk5", 0.2, 3.0, 40.0, 0.8, 2, 6, 0),
    "mixed_euler_lusgs_sup": ("mixed", "euler", "lusgs", 1.2, -4.0, 1e6, 2.0, 2, 7, 0),
    "mixed_lam_lusgs_o1": ("mixed", "viscous", "lusgs", 0.4, 10.0, 1000.0, 20.0, 2, 8, 1),
}

FILES = ["dims", "freestream", "geo_vol", "geo_cen", "geo_nrm", "geo_area", "geo_ecen", "geo_wall", "topo_lr",
         "topo_cedges", "topo_cverts", "topo_csize", "res0_U", "res0_R", "res0_Uedge", "res0_grad", "res0_specc",
         "res0_UL", "res0_UR", "res0_phi", "res0_gradT", "res0_specv", "res0_mu", "res0_muedge", "res0_dt",
         "end_U", "hist", "end_D", "end_dW1", "end_dW", "end_W", "end_R", "end_dt", "end_W0"]
INT_FILES = {"dims", "topo_lr", "topo_cedges", "topo_cverts", "topo_csize"}


def meshes():
    om = meshgen.o_mesh(32, 12, r0=0.5, dr1=0.02, rout=6.0)
    mx = meshgen.mixed_mesh(meshgen.naca_body(32), nlayer=4, dr1=0.01, growth=1.3, rfar=2.5, seed=11,
                            density=0.8, grade=1.0)
    return {"omesh": om, "mixed": mx}


def centroids(m: meshgen.GrdMesh) -> np.ndarray:
    """Vertex mean of each cell (only used to seed the perturbation)."""
    ncell = m.ncell
    acc = np.zeros((ncell, 2))
    cnt = np.zeros(ncell)
    for side in (0, 1):
        c = m.edge_cells[:, side]
        ok = c > 0
        for k in (0, 1):
            np.add.at(acc, c[ok] - 1, m.xy[m.edge_nodes[ok, k] - 1])
            np.add.at(cnt, c[ok] - 1, 1)
    return acc / cnt[:, None]


# SST k-omega phase: name -> (mesh, mach, aoa, re, seed).  The driver runs one
# laminar residual from a perturbed state and then the reference's SST
# functions on it, from per-cell multipliers of the freestream k, omega and mu_t.
SST_CASES = {
    "mixed_lam_sst": ("mixed", 0.4, 5.0, 1000.0, 9),
    "omesh_lam_sst": ("omesh", 0.2, 0.0, 40.0, 10),
}
SST_FILES = ["sst_inf", "sst_T_in", "sst_mut_in", "sst_tface", "sst_tgrad", "sst_f1", "sst_f2", "sst_mutf",
             "sst_fconv", "sst_fvisc", "sst_R", "sst_diag", "sst_T2", "sst_mut", "res0_U", "res0_Uedge",
             "res0_grad", "res0_mu", "res0_muedge", "res0_specc", "res0_specv", "res0_dt", "geo_wall"]


def sst_main(ms, drv):
    for case, (mname, ma, aoa, re, seed) in SST_CASES.items():
        m = ms[mname]
        g = 1.4
        a = 3.141593 * aoa / 180
        fs = np.array([1.0, 1.0, ma * np.sqrt(g) * np.cos(a), ma * np.sqrt(g) * np.sin(a)])
        U0 = meshgen.perturbed_state(m.ncell, centroids(m), fs, amp=0.05, seed=seed)
        rng = np.random.default_rng(seed)
        tm = np.exp(rng.uniform(-1.0, 1.0, 2 * m.ncell))
        mm = np.exp(rng.uniform(-1.0, 2.0, m.ncell))
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            U0.astype(np.float64).tofile(td / "u0.bin")
            tm.tofile(td / "t.bin")
            mm.tofile(td / "m.bin")
            env = dict(os.environ, SST_T=str(td / "t.bin"), SST_MUT=str(td / "m.bin"))
            r = subprocess.run([str(drv), str(HERE / f"{mname}.grd"), str(m.wall_tag), str(m.far_tag), "viscous",
                                "lusgs", repr(ma), repr(aoa), repr(re), "50.0", "0", str(td / "out"),
                                str(td / "u0.bin"), "0"], capture_output=True, text=True, env=env)
            if r.returncode != 0:
                raise RuntimeError(f"{case}: reference driver failed\n{r.stdout}\n{r.stderr}")
            arrs = {"init_U": U0}
            for f in SST_FILES:
                arrs[f] = np.fromfile(td / "out" / f"{f}.bin", np.float64)
        np.savez_compressed(HERE / f"{case}.npz", **arrs)
        print(case, m.ncell, "cells")


def main(ref_root: str = "", only: str = ""):
    from oracle.build import reference_root

    ref_root = ref_root or str(reference_root())
    drv = ROOT / "oracle" / "_ref" / "ref_driver"
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), ref_root], check=True)
    ms = meshes()
    if only == "sst":
        sst_main(ms, drv)
        return
    for name, m in ms.items():
        meshgen.write_grd(HERE / f"{name}.grd", m)
    manifest = {}
    for case, (mname, flow, adv, ma, aoa, re, cfl, nsteps, seed, fo) in CASES.items():
        m = ms[mname]
        g = 1.4
        a = 3.141593 * aoa / 180
        fs = np.array([1.0, 1.0, ma * np.sqrt(g) * np.cos(a), ma * np.sqrt(g) * np.sin(a)])
        U0 = meshgen.perturbed_state(m.ncell, centroids(m), fs, amp=0.05, seed=seed)
        with tempfile.TemporaryDirectory() as td:
            init = Path(td) / "u0.bin"
            U0.astype(np.float64).tofile(init)
            out = Path(td) / "out"
            r = subprocess.run([str(drv), str(HERE / f"{mname}.grd"), str(m.wall_tag), str(m.far_tag), flow, adv,
                                repr(ma), repr(aoa), repr(re), repr(cfl), str(nsteps), str(out), str(init), str(fo)],
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{case}: reference driver failed\n{r.stdout}\n{r.stderr}")
            arrs = {"init_U": U0}
            for f in FILES:
                p = out / f"{f}.bin"
                if p.exists():
                    arrs[f] = np.fromfile(p, np.int32 if f in INT_FILES else np.float64)
        np.savez_compressed(HERE / f"{case}.npz", **arrs)
        manifest[case] = dict(mesh=f"{mname}.grd", flow=flow, advance=adv, mach=ma, aoa=aoa, re=re, cfl=cfl,
                              nsteps=nsteps, seed=seed, first_order=fo, wall_tag=m.wall_tag, far_tag=m.far_tag,
                              ncell=int(m.ncell), nedge=int(m.nedge))
        print(case, m.ncell, "cells", json.loads(r.stdout.strip().splitlines()[-1]))
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    sst_main(ms, drv)


if __name__ == "__main__":
    main(*sys.argv[1:])
