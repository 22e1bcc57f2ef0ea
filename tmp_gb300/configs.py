"""Workload definitions: the synthetic meshes and flow settings of the five
benchmark configurations, generated from fixed seeds (no dataset involved).

C1  Euler, O-grid 128 x 64 around a unit-diameter cylinder, first spacing 1e-3 D
    to an outer radius of 20 D, M 0.3, 5-stage RK at CFL 0.8.
C2  laminar NS, 48 quad layers (first spacing 5e-3 D) around the cylinder plus
    a seeded Delaunay triangle fill to 30 D, ~130k cells, Re 40, M 0.2,
    LU-SGS at CFL 50.
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
    flow: str          # "euler" | "laminar"
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


WORKLOADS = {"c1": c1, "c2": c2, "c2big": c2big}


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
