"""Converged-state fixtures from the reference solver itself.

Two runs of the reference's own serial path (oracle/_ref/ref_driver, built from
its sources by oracle/build_ref.sh) from the uniform freestream to a converged
state:

  c1_conv   the C1 configuration: O-grid 128 x 64 around the unit-diameter
            cylinder (first spacing 1e-3 D, outer radius 20 D), Euler, M 0.3,
            AoA 0, first-order reconstruction (limiter 0), the reference's
            5-stage Runge-Kutta at CFL 0.8, 2000 iterations;
  c2s_conv  the C2 mesh recipe at 3,268 cells (32 body points, 8 quad layers
            from 5e-3 D with growth 1.08, seeded Delaunay fill to 30 D),
            laminar Re 40, M 0.2, second order, LU-SGS at CFL 50, run until
            the L2 density residual has fallen by 1e-10 from iteration 1.

The iteration count of c2s_conv is found with the C restatement
(oracle/cfd_oracle.c), which must reproduce the reference's final state bit
for bit; the script checks that before writing.  Each .npz holds the mesh
arrays (so the fixture does not depend on regenerating the mesh), the
reference's final primitive field, residual and per-step history, the
restatement's L2 density residual history and the wall force of the final
state (Fx, Fy: the restatement's wall-face flux sum of one residual
evaluation at that state).

usage: python tests/golden/make_golden_converged.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from tmp_gb300 import configs, meshgen  # noqa: E402

C2S_FALL = 1e-10


def c2s_mesh() -> meshgen.GrdMesh:
    return meshgen.mixed_mesh(configs.cylinder(32), nlayer=8, dr1=5e-3, growth=1.08, rfar=30.0, seed=77, density=1.0,
                              grade=0.82)


# name -> (mesh, flow, advance, mach, aoa, re, cfl, first_order)
CASES = {
    "c1_conv": (lambda: configs.c1().mesh, "euler", "rk5", 0.3, 0.0, 1e6, 0.8, 1),
    "c2s_conv": (c2s_mesh, "viscous", "lusgs", 0.2, 0.0, 40.0, 50.0, 0),
}


def oracle_run(p: Path, m: meshgen.GrdMesh, flow, adv, ma, aoa, re, cfl, fo, nsteps=None, fall=None):
    """Run the C restatement from the freestream; returns (steps, final U, L2 density residual history)."""
    import oracle
    from oracle import grd

    topo = grd.read_grd(p, m.wall_tag, m.far_tag)
    o = oracle.Oracle(topo, ma, aoa, re, flow == "viscous")
    l2 = []
    k = 0
    while True:
        rc = o.lusgs_step(cfl, bool(fo)) if adv == "lusgs" else o.rk_step(bool(fo))
        if rc != 0:
            raise RuntimeError(f"oracle step failed ({rc})")
        k += 1
        r = o.field("R").reshape(-1, 4)[:, 0]
        l2.append(float(np.sqrt(np.sum(r * r) / m.ncell)))
        if nsteps is not None and k >= nsteps:
            break
        if fall is not None and l2[-1] <= fall * l2[0]:
            break
        if k > 200000:
            raise RuntimeError("no convergence")
    u = o.field("U").copy()
    o.residual(bool(fo))  # the wall force of the final state
    return k, u, np.array(l2), o.wall_force().copy()


def main(ref_root: str = ""):
    from oracle.build import build as build_oracle, reference_root

    ref_root = ref_root or str(reference_root())
    build_oracle()
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), ref_root], check=True)
    drv = ROOT / "oracle" / "_ref" / "ref_driver"
    for name, (mk, flow, adv, ma, aoa, re, cfl, fo) in CASES.items():
        m = mk()
        with tempfile.TemporaryDirectory() as td:
            p = Path(td) / f"{name}.grd"
            meshgen.write_grd(p, m)
            n, u_o, l2, force = oracle_run(p, m, flow, adv, ma, aoa, re, cfl, fo,
                                           nsteps=2000 if name == "c1_conv" else None,
                                           fall=C2S_FALL if name == "c2s_conv" else None)
            out = Path(td) / "out"
            r = subprocess.run([str(drv), str(p), str(m.wall_tag), str(m.far_tag), flow, adv, repr(ma), repr(aoa),
                                repr(re), repr(cfl), str(n), str(out), "-", str(fo)], capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{name}: reference driver failed\n{r.stdout}\n{r.stderr}")
            end_u = np.fromfile(out / "end_U.bin", np.float64).reshape(-1, 4)
            hist = np.fromfile(out / "hist.bin", np.float64)
            end_r = np.fromfile(out / "end_R.bin", np.float64) if (out / "end_R.bin").exists() else None
            if not np.array_equal(end_u.view(np.int64), u_o.reshape(-1, 4).view(np.int64)):
                d = np.max(np.abs(end_u - u_o.reshape(-1, 4)))
                raise RuntimeError(f"{name}: the C restatement's final state differs from the reference's ({d:.3e})")
        arrs = dict(xy=m.xy, edge_nodes=m.edge_nodes, edge_cells=m.edge_cells, ncell=np.int64(m.ncell),
                    wall_tag=np.int64(m.wall_tag), far_tag=np.int64(m.far_tag), nsteps=np.int64(n),
                    mach=np.float64(ma), aoa=np.float64(aoa), re=np.float64(re), cfl=np.float64(cfl),
                    first_order=np.int64(fo), end_U=end_u, hist=hist, l2_hist=l2, wall_force=force)
        if end_r is not None:
            arrs["end_R"] = end_r
        np.savez_compressed(HERE / f"{name}.npz", **arrs)
        print(f"{name}: {m.ncell} cells, {n} steps, L2 fall {l2[-1] / l2[0]:.3e}, wall force {force}")


if __name__ == "__main__":
    main(*sys.argv[1:])
