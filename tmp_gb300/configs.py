"""Workload definitions: the synthetic meshes and flow settings of the five
benchmark configurations, generated from fixed seeds (no dataset involved).

C1  Euler, O-grid 128 x 64 around a unit-diameter cylinder, first spacing 1e-3 D
    to an outer radius of 20 D, M 0.3, 5-stage RK at CFL 0.8.
C2  laminar NS, 48 quad layers (first spacing 5e-3 D) around the cylinder plus
    a seeded Delaunay triangle fill to 30 D, ~130k cells, Re 40, M 0.2,
    LU-SGS at CFL 50.
C3  SST k-omega RANS around a NACA 0012 (chord 1): 256 quad layers from a
    first spacing of 2e-6 growing by 1.1 up to 4e-3, then a seeded Delaunay
    triangle fill to 100 chords, 1,071,543 cells; Re 6e6, M 0.15, AoA 4 deg
    (0 and 10 as variants), freestream turbulence intensity 0.1% and
    mu_t / mu = 10, LU-SGS.
C5  256 independent cases of uneven size (5k-200k cells, log-uniform from a
    seed), cylinder or NACA 0012 bodies with quad layers and a triangle fill,
    M ~ U[0.2, 0.8], AoA ~ U[-4, 10] deg, half Euler and half viscous with
    Re log-uniform in [1e5, 1e7], all advanced by LU-SGS.
"""
from __future__ import annotations

import hashlib
import os
import tempfile
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import meshgen


@dataclass
class Workload:
    name: str
    mesh: meshgen.GrdMesh
    flow: str          # "euler" | "laminar" | "sst"
    advance: str       # "rk5" | "lusgs"
    mach: float
    aoa: float
    re: float
    cfl: float
    extra: dict = field(default_factory=dict)


def cylinder(n: int = 256, r: float = 0.5) -> np.ndarray:
    th = 2 * np.pi * np.arange(n) / n
    return np.stack([r * np.cos(th), r * np.sin(th)], 1)


def c1() -> Workload:
    m = meshgen.o_mesh(128, 64, r0=0.5, dr1=1e-3, rout=20.0)
    return Workload("C1 cylinder O-grid 128x64 Euler RK5", m, "euler", "rk5", 0.3, 0.0, 1e6, 0.8)


def c2() -> Workload:
    m = meshgen.mixed_mesh(cylinder(256), nlayer=48, dr1=5e-3, growth=1.05, rfar=30.0, seed=2024, density=1.0,
                           grade=0.82)
    return Workload("C2 cylinder mixed quad/tri ~130k laminar LU-SGS", m, "laminar", "lusgs", 0.2, 0.0, 40.0, 50.0)


def c2big() -> Workload:
    """The C2 recipe at ~1M cells (larger than L2, used for DRAM-level profiles)."""
    m = meshgen.mixed_mesh(cylinder(720), nlayer=96, dr1=2.5e-3, growth=1.03, rfar=30.0, seed=2025, density=1.0,
                           grade=0.79)
    return Workload("C2big cylinder mixed quad/tri ~1M laminar LU-SGS", m, "laminar", "lusgs", 0.2, 0.0, 40.0, 50.0)


def c3_mesh() -> meshgen.GrdMesh:
    return meshgen.mixed_mesh(meshgen.naca_body(1024), nlayer=256, dr1=2e-6, growth=1.1, rfar=100.0, seed=3003,
                              density=1.0, grade=1.25, hmax=4e-3)


def c3(aoa: float = 4.0, cfl: float = 400.0) -> Workload:
    """The SST airfoil case; extra: freestream turbulence (intensity, mu_t / mu).  CFL 400 is the reference's
    LU-SGS default (LUSGS_Integrator.h:18); the case names none."""
    return Workload(f"C3 NACA 0012 ~1.07M SST k-omega AoA {aoa:g}", c3_mesh(), "sst", "lusgs", 0.15, aoa, 6e6, cfl,
                    extra=dict(tu=0.001, mut_ratio=10.0))


WORKLOADS = {"c1": c1, "c2": c2, "c2big": c2big, "c3": c3}


@dataclass
class BatchCase:
    """One case of the uneven batch: body kind, target size and flow."""

    index: int
    body: str          # "cylinder" | "naca0012"
    target_cells: int
    nbody: int
    seed: int
    flow: str          # "euler" | "laminar"
    mach: float
    aoa: float
    re: float

    def grd(self) -> meshgen.GrdMesh:
        body = cylinder(self.nbody) if self.body == "cylinder" else meshgen.naca_body(self.nbody)
        dr1 = 5e-3 if self.body == "cylinder" else 2e-3
        return meshgen.mixed_mesh(body, nlayer=16, dr1=dr1, growth=1.08, rfar=30.0, seed=self.seed, density=1.0,
                                  grade=0.82)


def c5_cases(n: int = 256, seed: int = 5005, lo: int = 5_000, hi: int = 200_000) -> list[BatchCase]:
    """The uneven batch.  Sizes are drawn log-uniform in [lo, hi]; the body
    resolution that gives a size follows the generator's own scaling (cells
    ~ 2.8 nbody^2 for the cylinder recipe, ~ 6.1 nbody^2 for the airfoil, with
    16 quad layers and the triangle fill to 30 body lengths).  The first half
    of the cases (in index order) is Euler, the second half viscous (the
    batch leg runs it with the SST k-omega model)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        target = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        body = "cylinder" if rng.uniform() < 0.5 else "naca0012"
        nbody = max(16, int(round(np.sqrt(target / (2.8 if body == "cylinder" else 6.1)))))
        out.append(BatchCase(index=i, body=body, target_cells=target, nbody=nbody,
                             seed=int(rng.integers(1, 1 << 30)), flow="euler" if i < n // 2 else "laminar",
                             mach=float(rng.uniform(0.2, 0.8)), aoa=float(rng.uniform(-4.0, 10.0)),
                             re=float(np.exp(rng.uniform(np.log(1e5), np.log(1e7))))))
    return out


def _batch_grd(case: BatchCase) -> meshgen.GrdMesh:
    return case.grd()


def c5_meshes(cases: list[BatchCase], workers: int = 0) -> list[meshgen.GrdMesh]:
    """Generate the batch's meshes, in parallel over host cores (a spawned
    process pool, safe after CUDA has been initialised in the caller)."""
    workers = workers or min(len(cases), os.cpu_count() or 1, 16)
    if workers <= 1:
        return [c.grd() for c in cases]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_batch_grd, cases, chunksize=1))


def grd_path(w: Workload, cache_dir: str | os.PathLike | None = None) -> Path:
    """Write the workload's mesh once per content hash and return the path."""
    d = Path(cache_dir or tempfile.gettempdir()) / "tmp_gb300_meshes"
    d.mkdir(parents=True, exist_ok=True)
    h = hashlib.sha1(w.mesh.xy.tobytes() + w.mesh.edge_cells.tobytes()).hexdigest()[:16]
    p = d / f"{w.name.split()[0]}_{h}.grd"
    if not p.exists():
        tmp = p.with_suffix(".tmp")
        meshgen.write_grd(tmp, w.mesh)
        os.replace(tmp, p)
    return p
