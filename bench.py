#!/usr/bin/env python
"""Benchmark of the GB300 unstructured finite-volume hot path.

Workload (default, config C2): laminar Navier-Stokes around a cylinder on a
~130k-cell mixed quad/triangle mesh (48 quad layers + seeded Delaunay fill to
30 D), Re 40, Mach 0.2, Venkatakrishnan-limited second-order HLLC, implicit
LU-SGS at CFL 50.  One step = one LU-SGS iteration (residual, local dt,
diagonal, forward + backward level-scheduled sweeps, update) over the mesh.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--precision fp64|fp32|mixed|mixff]

Precision forms: fp64 = the plain path (every kernel in binary64, results
equal to the reference's); fp32 = fluxes, gradients, limiter and the LU-SGS
sweep in binary32 with the update, norms and diagonal in binary64; mixed =
binary64 residual with the binary32 sweep (defect correction; converges to
the binary64 solution in the same number of iterations as fp64); mixff = the
mixed form with fluxes, gradients and limiter in float-float pairs of binary32
numbers (48-bit significands on the binary32 pipe, residual summed into
binary64; the same iterations as mixed to a 1e-3 fall; the default).
`value` is the --precision form; "forms" adds the
others measured the same way in the same run, and "time_to_drop" the wall
time each form takes from the freestream start to a --drop fall of the L2
density residual (normalised by iteration 1), capped at --drop-seconds.

Prints ONE JSON line on rank 0.  value = cell-iterations per second of the
whole job with the state resident in HBM (CUDA events on the solver's stream,
L2 flushed between timed steps); e2e = the same metric through the C ABI with
the step's input field copied from pinned host memory and its residual norm
read back inside the timed region.  Multi-GPU runs are independent replicas
(the reference's spatial decomposition is not needed on one GB300), so the
scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-iters/s and time-to-1e-8 residual drop: FP32+learned vs FP64 plain"
UNIT = "cell-iters/s"
# arithmetic of each form: residual (fluxes, gradients, limiter) + sweep + update/norms/diagonal
DTYPE = {"fp64": "f64", "fp32": "f32+f64", "mixed": "f64 residual+f32 sweep+f64",
         "mixff": "f32-pair residual+f32 sweep+f64"}
FLUSH_BYTES = 256 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3", help="workload: c3 (SST airfoil, 1.07M cells), c2, c2big, c1")
    ap.add_argument("--aoa", type=float, default=None,
                    help="c3 only: angle of attack in degrees (the case is named at 0, 4 and 10; default 4)")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "fp32", "mixed", "mixff"],
                    help="headline form (auto: mixff, the float-float residual with the binary32 sweeps)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="bounded CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--sweep-mode", type=int, default=-1,
                    help="LU-SGS schedule (-1 auto: 5 for the binary32-sweep forms, 0 for fp64; 0 dataflow, "
                         "1/2 per level, 5 chain-scheduled binary32 dataflow)")
    ap.add_argument("--sweep-bpsm", type=int, default=0, help="dataflow sweep blocks per SM (0 = autotune)")
    ap.add_argument("--sweep-poll-ns", type=int, default=0, help="dataflow sweep back-off between polls (ns)")
    ap.add_argument("--forms", default="fp64,fp32,mixed", help="precision forms timed besides --precision ('' = none)")
    ap.add_argument("--drop", type=float, default=1e-8, help="residual fall for time_to_drop (0 = skip)")
    ap.add_argument("--drop-seconds", type=float, default=200.0, help="cap per form for time_to_drop")
    ap.add_argument("--drop-forms", default="fp64,mixff,fp32+learned>mixff",
                    help="forms for time_to_drop: PREC[>PREC2][+learned]; '>' switches at --switch-at "
                         "(others: fp32, mixed, mixed+learned, fp32+learned>mixed)")
    ap.add_argument("--sst-drop-forms", default="fp64,mixff,mixed",
                    help="forms of the SST case's equal-fall run (the first sets the fall)")
    ap.add_argument("--sst-drop-seconds", type=float, default=120.0,
                    help="time the first form of the SST case runs; the others run to the fall it reached")
    ap.add_argument("--switch-at", type=float, default=3e-4,
                    help="residual fall at which 'A>B' switches form (or earlier, once A's residual stalls)")
    ap.add_argument("--no-overset", action="store_true", help="skip the overset connectivity / exchange leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the uneven-batch leg (256 packed cases)")
    ap.add_argument("--batch-meshes", type=int, default=256, help="meshes in the uneven-batch leg")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peak_gbs() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def alg_bytes(pass_name: str, nc: int, nf: int, viscous: bool, precision: str) -> int:
    """Compulsory bytes of one launch: each array the kernel touches, once.

    The residual passes run in binary32 only in the fp32 form (float-float
    pairs in the mixff form take binary64's 8 bytes); the LU-SGS sweeps in
    binary32 in the fp32, mixed and mixff forms."""
    sweep = pass_name in ("sweep_fwd", "sweep_bwd", "lusgs_update")
    fp32 = precision == "fp32" or (precision in ("mixed", "mixff") and sweep)
    s = 4 if fp32 else 8
    v = 1 if viscous else 0
    if pass_name == "face_state":
        return nf * (8 + 4 * s + 4 * s + 2 * s + v * s) + nc * 4 * s
    if pass_name == "cell_grad":
        return nc * (16 + 4 * s + 4 * s + 8 * s + 4 * s + s + v * 4 * s) + nf * (8 + 4 * s + 4 * s + 4 * s + 2 * s)
    if pass_name == "face_flux":
        return nf * (8 + 4 * s + 4 * s + 4 * s + 4 * s + v * (4 * s + s + 4 * s)) + nc * (4 * s + 8 * s + 4 * s + v * 2 * s)
    if pass_name == "cell_update":
        return nc * (16 + 32 + s + v * s + 32 + 8 + 8) + nf * (4 * s + v * 4 * s)
    if pass_name in ("sweep_fwd", "sweep_bwd"):
        return nc * (4 + 16 + 32 + 8 + v * s + 32 + 32 + 32 + 32) + nf * (8 + 32 + v * 32)
    if pass_name == "lusgs_update":
        return nc * (32 + 64 + 32 + (16 if fp32 else 0))
    # the coupled SST model (binary64 arrays): its four residual passes (face values and mu_t; k, omega
    # gradients and F1 / F2; face fluxes; sources, residual and diagonal), the turbulence sweeps (per-slot
    # constants, then forward and backward), the k, omega, mu_t update
    if pass_name == "sst_residual":
        face = nf * (8 + 32 + 4 + 32 + 8 + 16 + 8) + nc * (16 + 8 + 8)
        cell = nc * (16 + 32 + 16 + 8 + 8 + 32 + 8 + 8 + 32) + nf * (32 + 16)
        flux = nf * (8 + 32 + 32 + 16 + 16 + 8 + 8 + 16) + nc * (16 + 32 + 32 + 8 + 32)
        total = nc * (8 + 32 + 32 + 16 + 8 + 32 + 32 + 16 + 16 + 16 + 8 + 8 + 8) + nf * 32
        return face + cell + flux + total
    if pass_name == "sst_sweeps":
        prep = nc * (16 + 32 + 32 + 32 + 16 + 32 + 8 + 8 + 16 + 64 + 32 + 32 + 32 + 16) + nf * (8 + 32 + 32)
        sweep = nc * (4 + 16 + 16 + 64 + 32 + 32 + 16 + 16 + 16) + nf * 8
        return prep + 2 * sweep
    if pass_name == "sweeps_overlapped":  # both directions of the flow's and the turbulence sweeps, with their constants
        return (alg_bytes("sweep_fwd", nc, nf, viscous, precision) + alg_bytes("sweep_bwd", nc, nf, viscous, precision)
                + alg_bytes("sst_sweeps", nc, nf, viscous, precision))
    if pass_name == "sst_update":
        return nc * (4 + 16 + 16 + 32 + 16 + 16 + 8 + 32 + 8)
    raise KeyError(pass_name)


def sweep_dict(case) -> dict:
    """The LU-SGS schedule a case runs (after autotune), with, for SST, whether the turbulence sweeps share the
    flow's sweep launches."""
    from tmp_gb300 import abi

    d = dict(zip(("mode", "blocks_per_sm", "threads", "lookahead"), case.sweep_config()))
    if case.flow == abi.FLOW_SST:
        d["turbulence_overlapped"] = case.sst_overlapped()
    return d


def traffic_table() -> dict:
    p = ROOT / "profiles" / "traffic.json"
    try:
        return json.loads(p.read_text())
    except Exception:
        return {}


def traffic_bytes(pass_name: str, precision: str, nc: int, sweep_mode: int = 0):
    """DRAM bytes of one launch (one pass for the chain-scheduled sweep) from the committed ncu capture (per cell,
    scaled by the cell count)."""
    sweep = pass_name in ("sweep_fwd", "sweep_bwd")
    form = "fp32" if precision == "fp32" or (precision in ("mixed", "mixff") and sweep) else "fp64"
    if sweep and form == "fp32" and sweep_mode in (5, 6):
        row = traffic_table().get(f"fp32_chain_{pass_name}")
    elif precision == "mixed" and not sweep and f"fp64c_{pass_name}" in traffic_table():
        # the mixed form's residual passes are the contracted binary64 build
        row = traffic_table().get(f"fp64c_{pass_name}")
    elif precision == "mixff" and not sweep:
        row = traffic_table().get(f"ffq_{pass_name}")  # the float-float residual
    else:
        row = traffic_table().get(f"{form}_{'sweep_fwd' if sweep else pass_name}")
    if not row:
        return None
    out = {"bytes": round(row["bytes_per_cell"] * nc), "from": row["source"],
           "note": "DRAM read+write of one launch on C2big (947,090 cells), scaled by the cell count"}
    if "fp64_pipe_pct" in row:
        out["fp64_pipe_pct"] = row["fp64_pipe_pct"]
    return out


# ---------------------------------------------------------------------------
def overset_leg(stream) -> dict:
    """Overset connectivity and fringe exchange at the two-component size: a
    1024 x 1024 Cartesian background on [-10, 10]^2 and a 512 x 128 O-grid
    around a unit cylinder out to r = 1.5 (synthetic, no dataset).  Times the
    device connectivity (bins, hole map, blanking of the background's nodes,
    donor search of both receptor sets) and one fringe exchange each way, and
    checks size-independent properties: weights in [-TOL, 1+TOL] summing to 1,
    and exact interpolation of a linear field."""
    import numpy as np
    import torch

    from tmp_gb300 import abi, meshgen

    bg_m = meshgen.cart_mesh(1024, 1024, (-10.0, -10.0), (10.0, 10.0))
    og_m = meshgen.o_mesh(512, 128, r0=0.5, dr1=1e-3, rout=1.5)
    paths = []
    meshes = []
    for m, name in ((bg_m, "bg"), (og_m, "og")):
        p = Path(tempfile.gettempdir()) / f"tmp_gb300_overset_{name}.grd"
        meshgen.write_grd(p, m)
        paths.append(p)
        meshes.append(abi.Mesh.load_grd(p, m.wall_tag, m.far_tag))
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    out = {"workload": "Cartesian 1024x1024 + O-grid 512x128 (r 0.5 to 1.5)",
           "cells": [meshes[0].ncell, meshes[1].ncell], "nodes": [meshes[0].nnode, meshes[1].nnode]}
    t0, t1 = ev(), ev()
    t0.record(stream)
    bg, og = abi.Block(meshes[0], stream.cuda_stream), abi.Block(meshes[1], stream.cuda_stream)
    hm = abi.HoleMap(og)
    iblank, mand = abi.overset_blank(bg, [og], [hm], nfringe=2)
    t1.record(stream)
    torch.cuda.synchronize()
    out["connectivity_ms"] = round(t0.elapsed_time(t1), 3)
    out["holes"] = int((iblank == 0).sum())
    out["mandatory"] = int(mand.sum())
    bxy = bg_m.xy
    oxy = og_m.xy
    rec_b = np.flatnonzero(mand == 1).astype(np.int32)
    r = np.hypot(oxy[:, 0], oxy[:, 1])
    rec_o = np.flatnonzero(r > 1.5 - 1e-9).astype(np.int32)
    t0.record(stream)
    it_b = abi.Interp.search(og, bxy[rec_b], rec_b)   # background fringe <- O-grid
    it_o = abi.Interp.search(bg, oxy[rec_o], rec_o)   # O-grid outer ring <- background
    t1.record(stream)
    torch.cuda.synchronize()
    out["search_ms"] = round(t0.elapsed_time(t1), 3)
    out["receptors"] = [int(it_b.info()[0]), int(it_o.info()[0])]
    out["receptors_requested"] = [int(rec_b.size), int(rec_o.size)]
    # properties: convex weights summing to 1, linear fields reproduced
    ok = True
    for itp, src_xy, rec_xy in ((it_b, oxy, bxy), (it_o, bxy, oxy)):
        recv, _, inode, w = itp.get()
        nw = np.where(inode[:, 3] < 0, 3, 4)
        wsum = w.sum(1)
        ok &= bool(np.all(w >= -1e-10) and np.all(w <= 1 + 1e-10) and np.max(np.abs(wsum - 1)) < 1e-12)
        lin = lambda xy: 1.0 + 0.3 * xy[:, 0] - 0.7 * xy[:, 1]  # noqa: E731
        q = lin(src_xy)
        est = np.array([np.dot(w[i, :nw[i]], q[inode[i, :nw[i]]]) for i in range(0, len(recv), max(1, len(recv) // 2000))])
        ref = lin(rec_xy[recv[:: max(1, len(recv) // 2000)]])
        ok &= bool(np.max(np.abs(est - ref)) < 1e-11 * max(1.0, np.abs(ref).max()))
    out["properties_ok"] = ok
    # one fringe exchange each way, ROW layout, 4 variables per node
    qb = torch.rand(4 * meshes[0].nnode, dtype=torch.float64, device="cuda")
    qo = torch.rand(4 * meshes[1].nnode, dtype=torch.float64, device="cuda")
    for _ in range(3):
        it_b.update(qo.data_ptr(), meshes[1].nnode, qb.data_ptr(), meshes[0].nnode, 4, stream=stream.cuda_stream)
        it_o.update(qb.data_ptr(), meshes[0].nnode, qo.data_ptr(), meshes[1].nnode, 4, stream=stream.cuda_stream)
    reps = 100
    t0.record(stream)
    for _ in range(reps):
        it_b.update(qo.data_ptr(), meshes[1].nnode, qb.data_ptr(), meshes[0].nnode, 4, stream=stream.cuda_stream)
        it_o.update(qb.data_ptr(), meshes[0].nnode, qo.data_ptr(), meshes[1].nnode, 4, stream=stream.cuda_stream)
    t1.record(stream)
    torch.cuda.synchronize()
    out["exchange_us"] = round(1e3 * t0.elapsed_time(t1) / reps, 2)
    # the full assembly (holes, resolution-based fringes, cancellations, fringe
    # reduction, double fringe) and an exchange through the lists it returns
    obc = [np.zeros(0, np.int32), rec_o]
    tw = time.perf_counter()
    asm = abi.overset_connect([bg, og], [None, hm], obc, nfringe=2, mexclude=3)
    out_a = {"ms": round(1e3 * (time.perf_counter() - tw), 1), "nfringe": 2, "mexclude": 3}
    out_a["holes"] = [int((i == 0).sum()) for i in asm["iblank"]]
    out_a["receptors"] = [int((i == -1).sum()) for i in asm["iblank"]]
    served = [sum(int((asm["interp"][d]["recv_block"] == k).sum()) for d in range(2)) for k in range(2)]
    ok_a = served == out_a["receptors"]
    lists = []
    for d, (src_xy, rec_xy, r_k) in enumerate(((bxy, oxy, 1), (oxy, bxy, 0))):
        it = asm["interp"][d]
        sel = it["recv_block"] == r_k
        w, inode, nw, recv = it["weights"][sel], it["inode"][sel], it["nweights"][sel], it["recv_node"][sel]
        ok_a &= bool(np.all(w >= -1e-10) and np.all(w <= 1 + 1e-10) and np.max(np.abs(w.sum(1) - 1), initial=0) < 1e-12)
        lin = lambda xy: 1.0 + 0.3 * xy[:, 0] - 0.7 * xy[:, 1]  # noqa: E731
        q = lin(src_xy)
        est = np.array([np.dot(w[i, :nw[i]], q[inode[i, :nw[i]]]) for i in range(len(recv))])
        ok_a &= bool(len(recv) == 0 or np.max(np.abs(est - lin(rec_xy[recv]))) < 1e-11 * max(1.0, np.abs(q).max()))
        lists.append(abi.Interp.from_list(recv, nw, inode, w, stream=stream.cuda_stream))
    out_a["properties_ok"] = ok_a
    t0.record(stream)
    for _ in range(reps):
        lists[0].update(qb.data_ptr(), meshes[0].nnode, qo.data_ptr(), meshes[1].nnode, 4, stream=stream.cuda_stream)
        lists[1].update(qo.data_ptr(), meshes[1].nnode, qb.data_ptr(), meshes[0].nnode, 4, stream=stream.cuda_stream)
    t1.record(stream)
    torch.cuda.synchronize()
    out_a["exchange_us"] = round(1e3 * t0.elapsed_time(t1) / reps, 2)
    out["assembly"] = out_a
    # the coupled solve: both components in one case (Euler, M 0.3, LU-SGS in the MIXFF form), field cells
    # updated, the fringe exchange (cell means at the donor nodes, interpolation, node means into the
    # receptor cells) at the end of every graph-captured step
    fs = dict(mach=0.3, aoa_deg=0.0, reynolds=1e6)
    case = abi.Case(meshes, [fs, fs], abi.FLOW_EULER, abi.ADV_LUSGS, abi.PREC_MIXFF, cfl=5.0,
                    stream=stream.cuda_stream, sweep_mode=5)
    case.init_freestream()
    tc = time.perf_counter()
    case.connect(meshes, [None, rec_o], nfringe=2, mexclude=3)
    connect_ms = 1e3 * (time.perf_counter() - tc)
    case.autotune(2)
    case.step_graph(5)
    case.sync()
    step_ms = case.bench_pass("step", 10, FLUSH_BYTES)
    fringe_ms = case.bench_pass("fringe", 10, FLUSH_BYTES)
    case.step_graph(200)
    case.sync()
    ib = [case.iblank(0), case.iblank(1)]
    ncell = meshes[0].ncell + meshes[1].ncell
    out["coupled"] = {"workload": "the two components in one case, Euler M 0.3, LU-SGS CFL 5, MIXFF form",
                      "cells": ncell, "connect_ms": round(connect_ms, 1), "ms_per_step": round(step_ms, 4),
                      "cell_iters_per_s": ncell / (step_ms * 1e-3), "fringe_ms": round(fringe_ms, 4),
                      "hole_cells": [int((i == 0).sum()) for i in ib],
                      "receptor_cells": [int((i == -1).sum()) for i in ib],
                      "sweep": sweep_dict(case),
                      "finite_after_200_steps": bool(np.isfinite(case.get("U", 0)).all() and
                                                     np.isfinite(case.get("U", 1)).all())}
    case.close()
    for p in paths:
        p.unlink()
    return out


def batch_leg(stream, precision: int, nmesh: int = 256, steps: int = 5, mode: int = 0) -> dict:
    """The uneven batch: `nmesh` independent meshes of 5k-200k cells (sizes
    log-uniform from a seed, cylinder or NACA 0012 bodies, quads + triangles),
    half Euler and half SST k-omega, advanced by LU-SGS.  Each flow family is one
    packed case (all its meshes concatenated: one launch per pass, the sweep
    levels of all meshes merged, blocks per SM autotuned, steps replayed from a
    CUDA graph); the same meshes are then advanced as separate cases one after
    another, and once more packed with the learned relaxation attached."""
    import torch

    from tmp_gb300 import abi, configs, learn

    cases = configs.c5_cases(nmesh)
    grds = configs.c5_meshes(cases)
    meshes = [abi.Mesh.from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag) for g in grds]
    del grds
    groups = {}
    for bc, m in zip(cases, meshes):
        # the viscous half runs the SST k-omega model (the reference's freestream turbulence, 1% and 0.035)
        fl = "sst" if bc.flow == "laminar" else bc.flow
        groups.setdefault(fl, []).append((m, dict(mach=bc.mach, aoa_deg=bc.aoa, reynolds=bc.re)))
    flow_code = dict(euler=abi.FLOW_EULER, laminar=abi.FLOW_LAMINAR, sst=abi.FLOW_SST)
    cfl = 10.0
    ncell = sum(m.ncell for m in meshes)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def run(case_list, init=True):
        for c in case_list:
            if init:
                c.init_freestream()
            c.step_graph(2)
        torch.cuda.synchronize()
        t0, t1 = ev(), ev()
        t0.record(stream)
        for c in case_list:
            c.step_graph(steps)
        t1.record(stream)
        torch.cuda.synchronize()
        for c in case_list:
            try:
                c.sync()
            except abi.CfdError as ex:
                errors.append(str(ex))
        return t0.elapsed_time(t1) / steps

    errors: list[str] = []
    packed = [abi.Case([m for m, _ in g], [f for _, f in g], flow_code[fl], abi.ADV_LUSGS, precision, cfl=cfl,
                       stream=stream.cuda_stream, sweep_mode=mode) for fl, g in groups.items()]
    tuned = []
    for c in packed:
        c.autotune(2)
        tuned.append(sweep_dict(c))
    ms_packed = run(packed)
    net = learn.load()
    ms_learned = None
    if net is not None:
        # attached after 30 plain steps: over-relaxing the impulsive start
        # diverges on the high-Mach cylinders of the batch
        for c in packed:
            c.init_freestream()
            c.step_graph(30)
            abi.case_track(c, True)
            abi.case_set_mlp(c, net, False)
        ms_learned = run(packed, init=False)
    for c in packed:
        c.close()
    separate = [abi.Case([m], [f], flow_code[fl], abi.ADV_LUSGS, precision, cfl=cfl, stream=stream.cuda_stream,
                         sweep_mode=mode) for fl, g in groups.items() for m, f in g]
    ms_sep = run(separate)
    for c in separate:
        c.close()
    levels = [m.levels()[0] for m in meshes]
    sizes = sorted(m.ncell for m in meshes)
    return {"workload": f"{nmesh} meshes, 5k-200k cells log-uniform (seed 5005), half Euler / half SST k-omega, LU-SGS CFL {cfl:g}",
            "meshes": nmesh, "cells": ncell, "cells_min_median_max": [sizes[0], sizes[len(sizes) // 2], sizes[-1]],
            "packed_cases": {fl: len(g) for fl, g in groups.items()}, "packed_sweep": tuned,
            "forward_levels_max_sum": [max(levels), sum(levels)], "steps": steps,
            "packed_ms_per_step": round(ms_packed, 3), "packed_cell_iters_per_s": ncell / (ms_packed * 1e-3),
            "packed_learned_ms_per_step": round(ms_learned, 3) if ms_learned else None,
            "packed_learned_cell_iters_per_s": ncell / (ms_learned * 1e-3) if ms_learned else None,
            "separate_sweep_mode": mode, "separate_ms_per_step": round(ms_sep, 3), "separate_cell_iters_per_s": ncell / (ms_sep * 1e-3),
            "solver_errors": sorted(set(errors))}


def oracle_for(w, topo=None):
    """The C restatement (the reference's serial path; with the SST model coupled as the GPU runs it) on the
    workload's mesh (its reader's topology `topo`, built here when not given), from the freestream."""
    import oracle
    from oracle import grd

    if topo is None:
        g = w.mesh
        topo = grd.topo_from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag)
    t = topo
    o = oracle.Oracle(t, w.mach, w.aoa, w.re, w.flow in ("laminar", "sst"))
    if w.flow == "sst":
        o.sst_enable(True, w.extra.get("tu", 0.01), w.extra.get("mut_ratio", 0.035))
    return t, o


def cpu_baseline(w, seconds: float) -> dict:
    """C restatement of the reference's serial LU-SGS path on one host core."""
    t, o = oracle_for(w)
    o.lusgs_step(w.cfl) if w.advance == "lusgs" else o.rk_step()  # warm-up step
    n = 0
    t0 = time.perf_counter()
    while True:
        o.lusgs_step(w.cfl) if w.advance == "lusgs" else o.rk_step()
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 2000:
            break
    return {"value": t.ncell * n / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} {w.advance} steps of the same {t.ncell}-cell workload, oracle/cfd_oracle.c -O2, "
                      f"{el:.1f} s on 1 host core"}


def _ref_worker(args):
    wd, topo_path, steps, warmup, barrier = args
    sys.path.insert(0, str(ROOT))
    import types

    import numpy as np

    from oracle import grd

    w = types.SimpleNamespace(**wd)  # the workload's flow settings (its mesh comes as the topology file)
    z = np.load(topo_path)
    t = grd.Topo(int(z["nnode"]), int(z["nedge"]), int(z["ncell"]), z["xy"], z["edge_nodes"], z["lr"],
                 z["cell_verts"], z["cell_nvert"], z["cell_edges"], z["cell_nedge"])
    t, o = oracle_for(w, t)
    step = (lambda: o.lusgs_step(w.cfl)) if w.advance == "lusgs" else (lambda: o.rk_step())
    for _ in range(warmup):
        step()
    barrier.wait()  # every copy times the same contended window of the host's memory system
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    return t.ncell * steps, time.perf_counter() - t0


def workload(args):
    """The named workload; --aoa sets C3's angle of attack."""
    from tmp_gb300 import configs

    if args.aoa is None:
        return configs.WORKLOADS[args.config]()
    if args.config != "c3":
        raise SystemExit("--aoa applies to the c3 workload only")
    return configs.c3(aoa=args.aoa)


def run_reference(args):
    """Reference arm: the reference's CPU algorithm (C restatement, bit-exact to
    the reference's compiled serial path) on all host cores as independent
    copies of the workload (the reference has no threading)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp

    import oracle
    from tmp_gb300 import configs

    import numpy as np
    from oracle import grd

    oracle.build()
    w = workload(args)
    ncores = os.cpu_count() or 1
    # the reader's topology once, shared by the copies through a file
    g = w.mesh
    t = grd.topo_from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag)
    fd, topo_path = tempfile.mkstemp(suffix=".npz")
    os.close(fd)
    np.savez(topo_path, nnode=t.nnode, nedge=t.nedge, ncell=t.ncell, xy=t.xy, edge_nodes=t.edge_nodes, lr=t.lr,
             cell_verts=t.cell_verts, cell_nvert=t.cell_nvert, cell_edges=t.cell_edges, cell_nedge=t.cell_nedge)
    steps = max(1, args.steps)  # the same timed steps as the GPU arm
    warm = max(3, args.warmup)  # at least three untimed steps per copy
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Manager() as mgr, ctx.Pool(ncores) as pool:
        barrier = mgr.Barrier(ncores)
        wd = dict(mach=w.mach, aoa=w.aoa, re=w.re, cfl=w.cfl, flow=w.flow, advance=w.advance, extra=w.extra)
        res = pool.map(_ref_worker, [(wd, topo_path, steps, warm, barrier)] * ncores, chunksize=1)
    wall = time.perf_counter() - t0
    os.unlink(topo_path)
    cells = sum(r[0] for r in res)
    slowest = max(r[1] for r in res)
    value = cells / slowest
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * slowest / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "ncell": w.mesh.ncell, "nedge": w.mesh.nedge, "mach": w.mach,
                       "aoa": w.aoa, "re": w.re, "cfl": w.cfl, "flow": w.flow, "copies": ncores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": f"{ncores} independent copies x {steps} {w.advance} steps of the "
                                       f"{w.mesh.ncell}-cell workload (oracle/cfd_oracle.c, bit-exact restatement "
                                       f"of the reference's serial path), {wall:.1f} s wall"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch

    from tmp_gb300 import abi, configs, replicas
    from tmp_gb300.build import build_library

    t_start = time.perf_counter()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_library()
    w = workload(args)
    g = w.mesh
    mesh = abi.Mesh.from_arrays(g.xy, g.edge_nodes, g.edge_cells, g.ncell, g.wall_tag, g.far_tag)
    viscous = w.flow in ("laminar", "sst")
    if args.precision == "auto":
        args.precision = "mixff"
    stream = torch.cuda.Stream()  # a real stream: graph capture is not allowed on the legacy default stream
    torch.cuda.set_stream(stream)
    prec_code = dict(fp64=abi.PREC_FP64, fp32=abi.PREC_FP32, mixed=abi.PREC_MIXED, mixff=abi.PREC_MIXFF)
    flow_code = dict(euler=abi.FLOW_EULER, laminar=abi.FLOW_LAMINAR, sst=abi.FLOW_SST)

    def sweep_mode_for(precision):
        if args.sweep_mode >= 0:
            return args.sweep_mode
        return 5 if precision in ("fp32", "mixed", "mixff") else 0

    def make_case(precision, wl=None, msh=None):
        wl, msh = wl or w, msh or mesh
        mode = sweep_mode_for(precision)
        c = abi.Case([msh], [dict(mach=wl.mach, aoa_deg=wl.aoa, reynolds=wl.re)], flow_code[wl.flow],
                     abi.ADV_LUSGS if wl.advance == "lusgs" else abi.ADV_RK5,
                     prec_code[precision], cfl=wl.cfl, stream=stream.cuda_stream,
                     sweep_mode=mode, sweep_blocks_per_sm=args.sweep_bpsm,
                     sweep_poll_ns=args.sweep_poll_ns)
        if wl.flow == "sst":
            abi.sst_set_inflow(c, wl.extra.get("tu", 0.01), wl.extra.get("mut_ratio", 0.035))
        c.init_freestream()
        c.tuned = None
        if args.sweep_bpsm == 0 and wl.advance == "lusgs" and mode in (0, 3, 4, 5):
            c.autotune(3)  # the sweeps' launch shape (and mode 0, 5 or 6), by timing whole steps
            c.tuned = c.sweep_config()
        return c

    def form_ok(f, wl=None):
        wl = wl or w
        if wl.advance != "lusgs" and "mix" in f:  # the mixed forms are LU-SGS forms
            return False
        if wl.flow == "sst" and "fp32" in f:  # the coupled SST model runs with the binary64 or float-float residual
            return False
        return True

    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def timed_steps(c, nsteps, before_timing=None):
        """(per-step device ms, kernel launches) of graph-replayed steps, L2 flushed between them."""
        c.step_graph(max(args.warmup, 3))  # warm-up; also captures the step's CUDA graph
        torch.cuda.synchronize()
        if before_timing:
            before_timing()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        l0 = c.launches()
        for k in range(nsteps):
            flush.zero_()  # evict L2 (129 MB) between timed steps, outside the events
            evs[k][0].record(stream)
            c.step_graph(1)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs], c.launches() - l0

    case = make_case(args.precision)
    nc, nf = case.ncell, case.nedge
    U0 = case.get("U").copy()

    sampler = ClockSampler(local)

    def start_timing():
        sampler.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    ms, launches = timed_steps(case, args.steps, start_timing)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    t_local = sum(ms) / 1e3
    t_max, value = replicas.job_rate(nc * args.steps, t_local, world, dist, device="cuda")
    case.sync()

    # end to end through the C ABI: the step's field in from pinned host memory, one step, its residual norm
    # and the updated field back to pinned host memory (one call, one synchronisation)
    def e2e_of(c):
        host = torch.from_numpy(U0.reshape(-1)).pin_memory()
        hv = host.numpy()
        back = torch.zeros(4 * nc, dtype=torch.float64).pin_memory().numpy()
        nrm = torch.zeros(c.nmesh, dtype=torch.float64).pin_memory().numpy()
        c.step_io(hv, 1, "DW_RHO2", nrm, u_out=back)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            c.step_io(hv, 1, "DW_RHO2", nrm, u_out=back)
        el = time.perf_counter() - t0
        return {"value": replicas.job_rate(nc * args.steps, el, world, dist, device="cuda")[1], "unit": UNIT,
                "h2d_bytes_per_step": hv.nbytes, "d2h_bytes_per_step": back.nbytes + nrm.nbytes}

    e2e = None if args.no_e2e else e2e_of(case)
    legs = {"setup_and_timed": round(time.perf_counter() - t_start, 1)}
    t_leg = time.perf_counter()

    # the other precision forms, timed the same way
    forms = {}
    for f in [x for x in args.forms.split(",") if x and x != args.precision and form_ok(x)]:
        c2 = make_case(f)
        fm, _ = timed_steps(c2, args.steps)
        forms[f] = {"ms_per_step": sum(fm) / args.steps, "value": nc * args.steps / (sum(fm) / 1e3),
                    "sweep": sweep_dict(c2)}
        if f == "fp64" and not args.no_e2e:
            forms[f]["e2e"] = e2e_of(c2)
        c2.close()
    forms[args.precision] = {"ms_per_step": 1e3 * t_local / args.steps, "value": nc * args.steps / t_local,
                             "sweep": sweep_dict(case), "e2e": e2e}
    # the plain binary64 form (results equal to the reference's) next to the headline form
    plain = forms.get("fp64")

    # wall time from the freestream start to a residual fall of args.drop, per
    # form, and with the committed learned relaxation
    def time_to_drop(wl, msh, forms, target, cap, equal_fall=False):
        """equal_fall: the first form runs for `cap` seconds (or to `target`), the others to the fall it
        reached (at most 3 cap), so that every form is timed to the same residual fall."""
        from tmp_gb300 import learn

        net = learn.load()
        out = {"workload": wl.name, "target": target, "norm": "L2 density residual / iteration 1", "cap_s": cap,
               "learned_weights": str(learn.WEIGHTS.relative_to(ROOT)) if net else None}
        first_done = False
        for f in [x for x in forms.split(",") if x]:
            # "A>B" switches form A to B; "+learned" at the end keeps the learned
            # relaxation on throughout, "A+learned>B" only until the switch
            learned = "+learned" in f
            if learned and (net is None or wl.advance != "lusgs"):
                continue
            if not form_ok(f, wl):
                continue
            first, _, then = f.partition(">")
            until_switch = first.endswith("+learned")
            first = first.replace("+learned", "")
            then = then.replace("+learned", "")
            c2 = make_case(first, wl, msh)
            torch.cuda.synchronize()
            r = learn.run_to_drop(c2, target, 10 ** 9, net if learned else None, chunk=50,
                                  max_seconds=cap if not (equal_fall and first_done) else 3 * cap,
                                  switch_at=args.switch_at if then else None,
                                  switch_to=prec_code[then] if then else None, detach_at_switch=until_switch)
            reached = r.reached
            if equal_fall and not first_done:
                target = max(target, r.history[-1][1])  # the fall the first form reached in its time
                out["equal_fall_target"] = target
                reached = True
            first_done = True
            out[f] = {"reached": reached, "seconds": round(r.seconds, 3), "iterations": r.iterations,
                      "fall": r.history[-1][1], "fell_back": r.fell_back}
            try:  # lift and drag of the state reached (wall force in the form's own arithmetic)
                wf = c2.wall_force()
                out[f]["cl"], out[f]["cd"] = wf["cl"], wf["cd"]
            except abi.CfdError:
                pass
            c2.close()
        ref = out.get("fp64")
        if isinstance(ref, dict) and "cd" in ref:
            # each form's lift and drag at its final state against the plain binary64 run's (CL is
            # compared absolutely: it is near zero on a symmetric body at zero incidence)
            out["vs_fp64"] = {f: {"cl_abs_diff": abs(v["cl"] - ref["cl"]),
                                  "cd_rel_diff": abs(v["cd"] - ref["cd"]) / max(abs(ref["cd"]), 1e-300),
                                  "fall_ratio": v["fall"] / ref["fall"]}
                              for f, v in out.items() if isinstance(v, dict) and "cd" in v and f != "fp64"}
            done = {f: v for f, v in out.items() if isinstance(v, dict) and v.get("reached")}
            if "fp64" in done:
                out["speedup_vs_fp64"] = {f: done["fp64"]["seconds"] / v["seconds"] for f, v in done.items()
                                          if f != "fp64"}
        return out

    drop = None
    drop_c2 = None
    if args.drop > 0 and rank == 0:
        if w.flow == "sst":
            # the SST airfoil: both forms for a bounded time (the fall each reaches in it)
            drop = time_to_drop(w, mesh, args.sst_drop_forms, args.drop, args.sst_drop_seconds, equal_fall=True)
            # and the metric's 1e-8 fall, measured, on the laminar cylinder (C2)
            w2 = configs.c2()
            g2 = w2.mesh
            m2 = abi.Mesh.from_arrays(g2.xy, g2.edge_nodes, g2.edge_cells, g2.ncell, g2.wall_tag, g2.far_tag)
            drop_c2 = time_to_drop(w2, m2, args.drop_forms, args.drop, args.drop_seconds)
        else:
            drop = time_to_drop(w, mesh, args.drop_forms, args.drop, args.drop_seconds)

    legs["forms_and_time_to_drop"] = round(time.perf_counter() - t_leg, 1)
    t_leg = time.perf_counter()
    # per-pass device times for the roofline (L2 flushed before each rep)
    passes = ["face_state", "cell_grad", "face_flux", "cell_update"]
    if w.advance == "lusgs":
        passes += ["sweep_fwd", "sweep_bwd", "lusgs_update"]
    if w.flow == "sst":
        passes += ["sst_residual", "sst_sweeps", "sst_update"]
        if case.sst_overlapped():  # the step runs the flow's and the turbulence sweeps in one launch each
            passes += ["sweeps_overlapped"]
    mode = sweep_mode_for(args.precision)
    per, launches_of = {}, {}
    for p in passes:
        l0 = case.launches()
        per[p] = case.bench_pass(p, 5, FLUSH_BYTES)
        n_l = round((case.launches() - l0) / 5)
        if p == "sweep_bwd" and mode not in (1, 2):
            n_l -= 1  # the untimed reset that a lone backward sweep needs
        launches_of[p] = n_l
    per_step = dict(per)
    if w.advance == "rk5":
        per_step = {p: 5 * v for p, v in per.items()}
    # the dominant single kernel (the SST rows hold several launches each)
    dominant = max((p for p in per_step if p not in ("sst_residual", "sst_sweeps", "sweeps_overlapped")),
                   key=per_step.get)
    nlev = mesh.levels()
    peak, peak_kind = measured_peak_gbs()
    rows = {}
    for p, v in per.items():
        b = alg_bytes(p, nc, nf, viscous, args.precision)
        rows[p] = {"ms": round(v, 5), "alg_bytes": b, "gbs": round(b / (v * 1e-3) / 1e9, 1),
                   "frac": round(b / (v * 1e-3) / 1e9 / peak, 4), "launches": launches_of.get(p, 1)}
        t = traffic_bytes(p, args.precision, nc, case.sweep_config()[0])
        if t:
            rows[p]["traffic"] = t["bytes"]
    # the sweeps are latency bound: time per dependency level against the measured
    # floor of one hand-off through global memory (wait, compute, publish)
    try:
        floor = abi.hop_latency_us(300, 0, stream.cuda_stream)
    except abi.CfdError:
        floor = None
    for p, lev in (("sweep_fwd", nlev[0]), ("sweep_bwd", nlev[1])):
        if p in rows:
            rows[p]["levels"] = lev
            rows[p]["us_per_level"] = round(1e3 * per[p] / lev, 3)
            rows[p]["floor_us_per_hop"] = round(floor, 3) if floor else None
    db = alg_bytes(dominant, nc, nf, viscous, args.precision)
    achieved = db / (per[dominant] * 1e-3) / 1e9
    tr = traffic_bytes(dominant, args.precision, nc, case.sweep_config()[0])
    latency = None
    if dominant in ("sweep_fwd", "sweep_bwd"):
        latency = {"levels": rows[dominant]["levels"], "us_per_level": rows[dominant]["us_per_level"],
                   "floor_us_per_hop": rows[dominant]["floor_us_per_hop"],
                   "note": "dependency-level latency bound: one level's cells wait for lower levels' increments"}
    compute = None
    if tr and "fp64_pipe_pct" in tr:
        compute = {"pipe": "fp64", "active_pct_of_peak": tr["fp64_pipe_pct"], "from": tr["from"],
                   "note": "binary64 residual pass: FP64-issue bound on GB300 (DFMA 1.0 TFLOP/s measured, a warp-wide "
                           "FP64 instruction holds its sub-partition for 64 cycles); DRAM traffic equals its "
                           "algorithmic bytes"}
    roofline = {"bound": "hbm", "kernel": dominant, "latency": latency, "compute": compute,
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": tr["bytes"] if tr else None, "traffic_source": tr, "alg_bytes_per_launch": db,
                "per_pass": rows}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.precision], "data": "synthetic",
            "config": {"workload": w.name, "ncell": nc, "nedge": nf, "levels": list(nlev), "mach": w.mach,
                       "aoa": w.aoa, "re": w.re, "cfl": w.cfl, "flow": w.flow, **w.extra, "precision": args.precision,
                       "sweep": sweep_dict(case),
                       "l2": "flushed (256 MiB write) between timed steps", "parallelism": f"replicas x{world}"},
            "clocks": clocks, "gpu_launches": launches, "e2e": e2e, "roofline": roofline,
            "plain_fp64": {"value": plain["value"], "ms_per_step": plain["ms_per_step"], "e2e": plain.get("e2e"),
                           "note": "every kernel in binary64, results equal to the reference's"} if plain else None,
            "forms": forms, "time_to_drop": drop}
    if drop_c2 is not None:
        line["time_to_drop_c2"] = drop_c2
    legs["per_pass"] = round(time.perf_counter() - t_leg, 1)
    t_leg = time.perf_counter()
    if rank == 0 and not args.no_overset:
        line["overset"] = overset_leg(stream)
        legs["overset"] = round(time.perf_counter() - t_leg, 1)
        t_leg = time.perf_counter()
    if rank == 0 and not args.no_batch and w.advance == "lusgs":
        try:
            line["batch"] = batch_leg(stream, prec_code[args.precision], args.batch_meshes, mode=mode)
        except Exception as ex:  # the leg is reported beside the headline, never instead of it
            line["batch"] = {"error": f"{type(ex).__name__}: {ex}"}
    legs["batch"] = round(time.perf_counter() - t_leg, 1)
    t_leg = time.perf_counter()
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds)
    legs["cpu_baseline"] = round(time.perf_counter() - t_leg, 1)
    line["leg_seconds"] = legs
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
