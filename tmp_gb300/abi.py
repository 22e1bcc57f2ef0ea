"""ctypes binding of the C ABI in include/cfdgb.h (libcfdgb.so).

Loading fails loudly: there is no fallback path.  Every call checks the
returned status and raises :class:`CfdError` with the library's message.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Sequence

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libcfdgb.so"

# status / enums (mirrors include/cfdgb.h)
OK = 0
ERR = {-1: "ARG", -2: "IO", -3: "MESH", -4: "CUDA", -5: "PSTAR", -6: "NONPHYSICAL", -7: "TIMEOUT",
       -8: "STATE", -9: "WALLTAN"}
BC_WALL, BC_FARFIELD = -2, -3
FLOW_EULER, FLOW_LAMINAR, FLOW_SST = 0, 1, 2
ADV_RK5, ADV_LUSGS = 0, 1
PREC_FP64, PREC_FP32, PREC_MIXED, PREC_MIXFF = 0, 1, 2, 3
FIELD = dict(U=0, W=1, R=2, GRAD=3, PHI=4, SPEC_C=5, SPEC_V=6, DT=7, DIAG=8, DW1=9, DW=10, GRADT=11, MU=12,
             UEDGE=13, MUEDGE=14, VOL=15, CENTER=16, NORMAL=17, AREA=18, ECENTER=19, WALLDIST=20, SST_T=21,
             SST_TFACE=22, SST_TGRAD=23, SST_F1=24, SST_F2=25, SST_MUT=26, SST_MUTF=27, SST_FCONV=28,
             SST_FVISC=29, SST_R=30, SST_DIAG=31, UL=32, UR=33)
# values per element and whether the field lives on faces
FIELD_SHAPE = dict(U=(4, 0), W=(4, 0), R=(4, 0), GRAD=(8, 0), PHI=(4, 0), SPEC_C=(1, 0), SPEC_V=(1, 0),
                   DT=(1, 0), DIAG=(1, 0), DW1=(4, 0), DW=(4, 0), GRADT=(2, 0), MU=(1, 0), UEDGE=(4, 1),
                   MUEDGE=(1, 1), VOL=(1, 0), CENTER=(2, 0), NORMAL=(2, 1), AREA=(1, 1), ECENTER=(2, 1),
                   WALLDIST=(1, 0), SST_T=(2, 0), SST_TFACE=(2, 1), SST_TGRAD=(4, 0), SST_F1=(1, 0), SST_F2=(1, 0),
                   SST_MUT=(1, 0), SST_MUTF=(1, 1), SST_FCONV=(2, 1), SST_FVISC=(2, 1), SST_R=(2, 0),
                   SST_DIAG=(2, 0), UL=(4, 1), UR=(4, 1))
NORM = dict(DW_RHO2=0, RK_DRHO=1, L2_R_RHO=2)
LAYOUT_ROW, LAYOUT_COLUMN = 0, 1
MLP_INPUTS, MLP_OUTPUTS, MLP_PARAMS = 12, 2, 5122


class CfdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR.get(code, code)}: {msg}")
        self.code = code


class Freestream(C.Structure):
    _fields_ = [("mach", C.c_double), ("aoa_deg", C.c_double), ("reynolds", C.c_double),
                ("density", C.c_double), ("pressure", C.c_double)]


class Params(C.Structure):
    _fields_ = [("flow", C.c_int), ("advance", C.c_int), ("precision", C.c_int), ("first_order", C.c_int),
                ("cfl", C.c_double), ("sweep_mode", C.c_int), ("sweep_blocks_per_sm", C.c_int),
                ("sweep_poll_ns", C.c_int), ("sweep_threads", C.c_int), ("sst_sequential", C.c_int),
                ("sst_sweep_share", C.c_int), ("chain_table_cap", C.c_int), ("reserved", C.c_int * 1)]


_lib = None


def lib() -> C.CDLL:
    """Load libcfdgb.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with tmp_gb300.build.build_library() "
                           "(there is no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    vp, ip, dp, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_float)
    sig = {
        "cfd_last_error": (C.c_char_p, []),
        "cfd_version": (C.c_int, []),
        "cfd_mesh_load_grd": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(vp)]),
        "cfd_mesh_from_arrays": (C.c_int, [C.c_int, dp, C.c_int, ip, ip, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
        "cfd_mesh_info": (C.c_int, [vp, ip, ip, ip]),
        "cfd_mesh_topology": (C.c_int, [vp, ip, ip, ip, ip]),
        "cfd_mesh_levels": (C.c_int, [vp, ip, ip]),
        "cfd_mesh_free": (None, [vp]),
        "cfd_case_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(Freestream), C.POINTER(Params), vp,
                                      C.POINTER(vp)]),
        "cfd_case_free": (None, [vp]),
        "cfd_case_info": (C.c_int, [vp, ip, ip, ip]),
        "cfd_case_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "cfd_set_cfl": (C.c_int, [vp, C.c_double]),
        "cfd_init_freestream": (C.c_int, [vp]),
        "cfd_residual": (C.c_int, [vp, C.c_int]),
        "cfd_local_dt": (C.c_int, [vp, C.c_double]),
        "cfd_step": (C.c_int, [vp, C.c_int]),
        "cfd_rk_step": (C.c_int, [vp]),
        "cfd_lusgs_step": (C.c_int, [vp]),
        "cfd_step_graph": (C.c_int, [vp, C.c_int]),
        "cfd_residual_norm": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "cfd_step_io": (C.c_int, [vp, dp, C.c_int, C.c_int, dp, dp]),
        "cfd_get_field": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "cfd_put_field": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "cfd_sync": (C.c_int, [vp]),
        "cfd_launch_count": (C.c_longlong, [vp]),
        "cfd_bench_pass": (C.c_int, [vp, C.c_int, C.c_int, C.c_longlong, dp]),
        "cfd_selftest_bounded_wait": (C.c_int, [vp, C.c_longlong]),
        "cfd_set_cell_cfl": (C.c_int, [vp, C.c_int, dp]),
        "cfd_wall_force": (C.c_int, [vp, C.c_int, C.c_double, dp]),
        "cfd_nodal_weights": (C.c_int, [C.c_longlong, ip, dp, dp, dp]),
        "cfd_block_create": (C.c_int, [vp, vp, C.POINTER(vp)]),
        "cfd_block_free": (None, [vp]),
        "cfd_block_search": (C.c_int, [vp, C.c_longlong, dp, ip, ip, dp]),
        "cfd_block_search_ex": (C.c_int, [vp, C.c_longlong, dp, ip, dp, C.c_char_p, ip, ip, dp, ip]),
        "cfd_block_node_to_cell": (C.c_int, [vp, vp, C.c_int, vp, vp]),
        "cfd_interp_create": (C.c_int, [vp, C.c_longlong, dp, ip, C.POINTER(vp)]),
        "cfd_interp_create_list": (C.c_int, [C.c_longlong, ip, ip, ip, dp, vp, C.POINTER(vp)]),
        "cfd_interp_info": (C.c_int, [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "cfd_interp_get": (C.c_int, [vp, ip, ip, ip, dp]),
        "cfd_interp_update": (C.c_int, [vp, vp, C.c_longlong, vp, C.c_longlong, C.c_int, C.c_int, vp]),
        "cfd_interp_free": (None, [vp]),
        "cfd_holemap_create": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
        "cfd_holemap_info": (C.c_int, [vp, ip, dp]),
        "cfd_holemap_get": (C.c_int, [vp, ip]),
        "cfd_holemap_check": (C.c_int, [vp, C.c_longlong, dp, ip]),
        "cfd_holemap_free": (None, [vp]),
        "cfd_overset_blank": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.POINTER(vp), C.c_int, ip, ip]),
        "cfd_cell_iblank": (C.c_int, [vp, ip, ip]),
        "cfd_overset_connect": (C.c_int, [C.c_int, C.POINTER(vp), C.POINTER(vp), C.POINTER(ip), ip, C.c_int, C.c_int,
                                          C.POINTER(vp)]),
        "cfd_connect_iblank": (C.c_int, [vp, C.c_int, ip, ip]),
        "cfd_connect_interp_count": (C.c_int, [vp, C.c_int, C.POINTER(C.c_longlong)]),
        "cfd_connect_interp_get": (C.c_int, [vp, C.c_int, ip, ip, ip, ip, ip, dp]),
        "cfd_connect_free": (None, [vp]),
        "cfd_connectivity": (C.c_int, [vp, C.POINTER(vp), C.POINTER(ip), ip, C.c_int, C.c_int]),
        "cfd_fringe_update": (C.c_int, [vp, C.c_int]),
        "cfd_case_iblank": (C.c_int, [vp, C.c_int, ip]),
        "cfd_write_cell_data": (C.c_int, [vp, C.c_int, vp, C.c_char_p, C.c_int]),
        "cfd_write_node_data": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int, dp]),
        "cfd_write_tioga_format": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int, ip]),
        "cfd_mlp_create": (C.c_int, [C.c_ulonglong, C.POINTER(vp)]),
        "cfd_mlp_free": (None, [vp]),
        "cfd_mlp_get_params": (C.c_int, [vp, fp, fp]),
        "cfd_mlp_set_params": (C.c_int, [vp, fp, fp]),
        "cfd_mlp_forward": (C.c_int, [vp, vp, C.c_longlong, vp, vp]),
        "cfd_mlp_loss_grad": (C.c_int, [vp, vp, vp, vp, C.c_longlong, dp, fp]),
        "cfd_mlp_train": (C.c_int, [vp, vp, vp, vp, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_ulonglong, fp]),
        "cfd_case_track": (C.c_int, [vp, C.c_int]),
        "cfd_case_features": (C.c_int, [vp, vp]),
        "cfd_case_set_mlp": (C.c_int, [vp, vp, C.c_int, C.c_double]),
        "cfd_measure_hop_latency": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "cfd_set_precision": (C.c_int, [vp, C.c_int]),
        "cfd_autotune": (C.c_int, [vp, C.c_int, ip, dp]),
        "cfd_case_sweep": (C.c_int, [vp, ip, ip, ip, ip]),
        "cfd_case_sst_overlap": (C.c_int, [vp, ip]),
        "cfd_chain_schedule": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, ip, ip, ip, ip, ip]),
        "cfd_sst_enable": (C.c_int, [vp]),
        "cfd_sst_freestream": (C.c_int, [vp, C.c_int, dp]),
        "cfd_sst_residual": (C.c_int, [vp]),
        "cfd_sst_update_mut": (C.c_int, [vp]),
        "cfd_sst_set_inflow": (C.c_int, [vp, C.c_double, C.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        raise CfdError(rc, lib().cfd_last_error().decode(errors="replace"))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Mesh:
    """A 2D mesh in the reference's .grd topology (UnstructReader semantics)."""

    def __init__(self, handle: int):
        self.h = C.c_void_p(handle)
        n = [C.c_int(), C.c_int(), C.c_int()]
        check(lib().cfd_mesh_info(self.h, *[C.byref(x) for x in n]))
        self.nnode, self.nedge, self.ncell = (x.value for x in n)

    @classmethod
    def load_grd(cls, path: str | os.PathLike, wall_tag: int, far_tag: int) -> "Mesh":
        h = C.c_void_p()
        check(lib().cfd_mesh_load_grd(str(path).encode(), int(wall_tag), int(far_tag), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_arrays(cls, xy: np.ndarray, edge_nodes: np.ndarray, edge_cells: np.ndarray, ncell: int,
                    wall_tag: int, far_tag: int) -> "Mesh":
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        en = np.ascontiguousarray(edge_nodes, dtype=np.int32).reshape(-1)
        ec = np.ascontiguousarray(edge_cells, dtype=np.int32).reshape(-1)
        h = C.c_void_p()
        check(lib().cfd_mesh_from_arrays(len(xy) // 2, _dptr(xy), len(en) // 2, _iptr(en), _iptr(ec), int(ncell),
                                         int(wall_tag), int(far_tag), C.byref(h)))
        return cls(h.value)

    def topology(self):
        lr = np.empty(2 * self.nedge, np.int32)
        ce = np.empty(4 * self.ncell, np.int32)
        cv = np.empty(4 * self.ncell, np.int32)
        cs = np.empty(2 * self.ncell, np.int32)
        check(lib().cfd_mesh_topology(self.h, _iptr(lr), _iptr(ce), _iptr(cv), _iptr(cs)))
        return dict(lr=lr.reshape(-1, 2), cell_edges=ce.reshape(-1, 4), cell_verts=cv.reshape(-1, 4),
                    cell_sizes=cs.reshape(-1, 2))

    def levels(self):
        a, b = C.c_int(), C.c_int()
        check(lib().cfd_mesh_levels(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def chain_schedule(self, forward: bool, nlists: int, local: bool = False, table: bool | int = False) -> dict:
        """The binary32 sweep's chain schedule of this mesh (host only): per-list
        position ranges, (cell, register bits) per position, (neighbour, face
        code) per slot, each slot's dependency encoding and the table size.
        table: False none, True a table over each block's whole range, an int
        a table capped at that many entries per block."""
        cap = 0 if table is False else (2**31 - 1 if table is True else int(table))
        nc = self.ncell
        hptr = np.empty(nlists + 1, np.int32)
        cells = np.empty(2 * nc, np.int32)
        rec = np.empty(8 * nc, np.int32)
        jenc = np.empty(4 * nc, np.int32)
        tbl = C.c_int()
        check(lib().cfd_chain_schedule(self.h, int(bool(forward)), int(nlists), int(bool(local)), cap,
                                       _iptr(hptr), _iptr(cells), _iptr(rec), _iptr(jenc), C.byref(tbl)))
        return dict(hptr=hptr, cells=cells.reshape(-1, 2), rec=rec.reshape(-1, 4, 2), jenc=jenc.reshape(-1, 4),
                    table_entries=tbl.value)

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_mesh_free(self.h)
            self.h = None


class Case:
    """Device-resident solver state for one or more packed meshes."""

    def __init__(self, meshes: Sequence[Mesh], freestreams: Sequence[dict], flow: int, advance: int,
                 precision: int = PREC_FP64, cfl: float = 1.0, first_order: bool = False, stream: int | None = None,
                 sweep_mode: int = 0, sweep_blocks_per_sm: int = 0, sweep_poll_ns: int = 0, sweep_threads: int = 0,
                 sst_sequential: bool = False, sst_sweep_share: int = 0, chain_table_cap: int = 0):
        self.meshes = list(meshes)
        arr = (C.c_void_p * len(meshes))(*[m.h.value for m in meshes])
        fs = (Freestream * len(meshes))(*[Freestream(f["mach"], f.get("aoa_deg", 0.0), f.get("reynolds", 1.0),
                                                     f.get("density", 1.225), f.get("pressure", 101325.0))
                                          for f in freestreams])
        p = Params(flow, advance, precision, int(first_order), float(cfl), int(sweep_mode), int(sweep_blocks_per_sm),
                   int(sweep_poll_ns), int(sweep_threads), int(bool(sst_sequential)), int(sst_sweep_share),
                   int(chain_table_cap))
        h = C.c_void_p()
        check(lib().cfd_case_create(arr, len(meshes), fs, C.byref(p), C.c_void_p(stream) if stream else None,
                                    C.byref(h)))
        self.h = h
        self.flow, self.advance, self.precision = flow, advance, precision
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().cfd_case_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        self.nmesh, self.ncell, self.nedge = a.value, b.value, c.value

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().cfd_case_stream(self.h, C.byref(s)))
        return s.value or 0

    def write_cell_data(self, filename: str, mesh: int = 0, proc: int = 0):
        """Tecplot cell dump of one mesh (TopologyHolderStrategy::writeCellData)."""
        check(lib().cfd_write_cell_data(self.h, int(mesh), self.meshes[mesh].h, str(filename).encode(), int(proc)))

    def wall_force(self, mesh: int = 0, ref_length: float = 1.0) -> dict:
        """Wall force of the current state: Fx, Fy, CL, CD."""
        out = np.zeros(4)
        check(lib().cfd_wall_force(self.h, int(mesh), float(ref_length), _dptr(out)))
        return dict(fx=out[0], fy=out[1], cl=out[2], cd=out[3])

    def set_cell_cfl(self, mult, mesh: int = 0):
        """Per-cell CFL multipliers (None removes them)."""
        if mult is None:
            check(lib().cfd_set_cell_cfl(self.h, int(mesh), None))
            return
        a = np.ascontiguousarray(mult, dtype=np.float64).reshape(-1)
        check(lib().cfd_set_cell_cfl(self.h, int(mesh), _dptr(a)))

    def init_freestream(self):
        check(lib().cfd_init_freestream(self.h))

    def autotune(self, reps: int = 5):
        """Pick the sweeps' blocks per SM by timing whole steps; returns (blocks_per_sm, ms)."""
        b, t = C.c_int(), C.c_double()
        check(lib().cfd_autotune(self.h, int(reps), C.byref(b), C.byref(t)))
        return b.value, t.value

    def sweep_config(self):
        """(sweep_mode, blocks_per_sm, threads per block, look-ahead) in use, e.g. after autotune()."""
        a, b, t, la = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib().cfd_case_sweep(self.h, C.byref(a), C.byref(b), C.byref(t), C.byref(la)))
        return a.value, b.value, t.value, la.value

    def sst_overlapped(self) -> bool:
        """Whether the LU-SGS step runs the turbulence sweeps in the flow's sweep launches."""
        v = C.c_int()
        check(lib().cfd_case_sst_overlap(self.h, C.byref(v)))
        return bool(v.value)

    def connect(self, meshes, obc_nodes=None, nfringe: int = 1, mexclude: int = 3):
        """Overset connectivity of the case's meshes (the handles it was created from); afterwards every LU-SGS
        step updates the field cells and ends with the fringe exchange."""
        n = len(meshes)
        ms = (C.c_void_p * n)(*[m.h.value for m in meshes])
        obc = [np.ascontiguousarray(o if o is not None else np.zeros(0), dtype=np.int32) for o in (obc_nodes or [None] * n)]
        op = (C.POINTER(C.c_int) * n)(*[_iptr(o) for o in obc])
        no = np.array([len(o) for o in obc], np.int32)
        check(lib().cfd_connectivity(self.h, ms, op, _iptr(no), int(nfringe), int(mexclude)))

    def fringe_update(self):
        check(lib().cfd_fringe_update(self.h, 4))

    def iblank(self, mesh: int = 0) -> np.ndarray:
        n = self._count("VOL", mesh)
        out = np.zeros(n, np.int32)
        check(lib().cfd_case_iblank(self.h, int(mesh), _iptr(out)))
        return out

    def set_precision(self, precision: int):
        check(lib().cfd_set_precision(self.h, int(precision)))

    def set_cfl(self, cfl: float):
        check(lib().cfd_set_cfl(self.h, float(cfl)))

    def residual(self, stage: int = 0):
        check(lib().cfd_residual(self.h, int(stage)))

    def local_dt(self, cfl: float):
        check(lib().cfd_local_dt(self.h, float(cfl)))

    def step(self, n: int = 1):
        check(lib().cfd_step(self.h, int(n)))

    def step_graph(self, n: int = 1):
        check(lib().cfd_step_graph(self.h, int(n)))

    def step_io(self, u_host: np.ndarray | None, nsteps: int = 1, which: str | None = "DW_RHO2",
                out: np.ndarray | None = None, u_out: np.ndarray | None = None) -> np.ndarray | None:
        """Upload the primitive field (host, all meshes), step, read every mesh's norm and, when u_out is
        given (float64, 4*ncell_total, contiguous), the updated field back: one call, one sync."""
        up = _dptr(u_host) if u_host is not None else None
        if which is not None and out is None:
            out = np.zeros(self.nmesh)
        if u_out is not None:
            assert u_out.dtype == np.float64 and u_out.flags.c_contiguous and u_out.size == 4 * self.ncell
        check(lib().cfd_step_io(self.h, up, int(nsteps), NORM[which] if which else 0,
                                _dptr(out) if which is not None else None,
                                _dptr(u_out) if u_out is not None else None))
        return out

    def sync(self):
        check(lib().cfd_sync(self.h))

    def norm(self, which: str = "DW_RHO2", mesh: int = 0) -> float:
        v = C.c_double()
        check(lib().cfd_residual_norm(self.h, int(mesh), NORM[which], C.byref(v)))
        return v.value

    def launches(self) -> int:
        return int(lib().cfd_launch_count(self.h))

    PASSES = dict(face_state=0, cell_grad=1, face_flux=2, cell_update=3, sweep_fwd=4, sweep_bwd=5,
                  lusgs_update=6, step=7, sst_residual=8, sst_sweeps=9, sst_update=10, fringe=11,
                  sweeps_overlapped=12)

    def bench_pass(self, name: str, reps: int, flush_bytes: int = 0) -> float:
        """Mean device time (ms) of one pass, CUDA events on the case's stream."""
        v = C.c_double()
        check(lib().cfd_bench_pass(self.h, self.PASSES[name], int(reps), int(flush_bytes), C.byref(v)))
        return v.value

    def _count(self, name: str, mesh: int) -> int:
        width, per_face = FIELD_SHAPE[name]
        m = self.meshes[mesh]
        return width * (m.nedge if per_face else m.ncell)

    def get(self, name: str, mesh: int = 0) -> np.ndarray:
        width, _ = FIELD_SHAPE[name]
        out = np.empty(self._count(name, mesh), np.float64)
        check(lib().cfd_get_field(self.h, int(mesh), FIELD[name], _dptr(out)))
        return out.reshape(-1, width) if width > 1 else out

    def put(self, name: str, values: np.ndarray, mesh: int = 0):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if a.size != self._count(name, mesh):
            raise ValueError(f"{name} needs {self._count(name, mesh)} values, got {a.size}")
        check(lib().cfd_put_field(self.h, int(mesh), FIELD[name], _dptr(a)))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_case_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


# ---- overset (UniTioga MeshBlock) -------------------------------------------

def nodal_weights(nvert: np.ndarray, xv: np.ndarray, xp: np.ndarray) -> np.ndarray:
    """computeNodalWeight2D on the device for n (cell, point) pairs.

    nvert[n] in {3, 4}; xv[n, 4, 2] vertices; xp[n, 2] points -> frac[n, 4]."""
    nv = np.ascontiguousarray(nvert, dtype=np.int32)
    x = np.ascontiguousarray(xv, dtype=np.float64).reshape(-1)
    p = np.ascontiguousarray(xp, dtype=np.float64).reshape(-1)
    n = nv.size
    if x.size != 8 * n or p.size != 2 * n:
        raise ValueError("xv must be [n, 4, 2] and xp [n, 2]")
    out = np.zeros(4 * n)
    check(lib().cfd_nodal_weights(n, _iptr(nv), _dptr(x), _dptr(p), _dptr(out)))
    return out.reshape(n, 4)


class Block:
    """One mesh on the device as an overset donor (MeshBlock)."""

    def __init__(self, mesh: Mesh, stream: int | None = None):
        self.h = C.c_void_p()
        self.ncell = mesh.ncell
        self.nnode = mesh.nnode
        check(lib().cfd_block_create(mesh.h, C.c_void_p(stream) if stream else None, C.byref(self.h)))

    def search(self, xy: np.ndarray):
        """(donor_cell[n], donor_nodes[n, 4], weights[n, 4]) for points xy[n, 2]."""
        p = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        n = p.size // 2
        d = np.zeros(n, np.int32)
        nodes = np.zeros(4 * n, np.int32)
        w = np.zeros(4 * n)
        check(lib().cfd_block_search(self.h, n, _dptr(p), _iptr(d), _iptr(nodes), _dptr(w)))
        return d, nodes.reshape(n, 4), w.reshape(n, 4)

    def search_ex(self, xy: np.ndarray, tags=None, res=None, unaccept=None):
        """MeshBlock::search with per-point mesh tags and resolutions and per-cell refusals:
        (donor_cell[n], donor_nodes[n, 4], weights[n, 4], xtag[n], merged resolutions[n] or None)."""
        p = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        n = p.size // 2
        d = np.empty(n, np.int32)
        nodes = np.empty(4 * n, np.int32)
        w = np.empty(4 * n)
        xt = np.empty(n, np.int32)
        tg = None if tags is None else np.ascontiguousarray(tags, np.int32)
        rs = None if res is None else np.array(res, np.float64)
        ua = None if unaccept is None else np.ascontiguousarray(unaccept, np.uint8)
        check(lib().cfd_block_search_ex(self.h, n, _dptr(p), _iptr(tg) if tg is not None else None,
                                        _dptr(rs) if rs is not None else None,
                                        ua.ctypes.data_as(C.c_char_p) if ua is not None else None, _iptr(d),
                                        _iptr(nodes), _dptr(w), _iptr(xt)))
        return d, nodes.reshape(n, 4), w.reshape(n, 4), xt, rs

    def cell_iblank(self, node_iblank: np.ndarray) -> np.ndarray:
        """getCellIblanks: 0 if any node is a hole, -1 if all nodes are receptors, else 1."""
        n = np.ascontiguousarray(node_iblank, dtype=np.int32)
        if n.size != self.nnode:
            raise ValueError("node_iblank needs one value per node")
        out = np.zeros(self.ncell, np.int32)
        check(lib().cfd_cell_iblank(self.h, _iptr(n), _iptr(out)))
        return out

    def node_to_cell(self, q_node_ptr: int, nvar: int, q_cell_ptr: int, stream: int | None = None):
        """Device arrays (raw pointers) in ROW layout."""
        check(lib().cfd_block_node_to_cell(self.h, C.c_void_p(q_node_ptr), int(nvar), C.c_void_p(q_cell_ptr),
                                           C.c_void_p(stream) if stream else None))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_block_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Interp:
    """An interpolation list (MeshBlock::interpList) resident on the device."""

    def __init__(self, handle: C.c_void_p):
        self.h = handle

    @classmethod
    def search(cls, donor: Block, xy: np.ndarray, recv_node: np.ndarray) -> "Interp":
        p = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        r = np.ascontiguousarray(recv_node, dtype=np.int32)
        h = C.c_void_p()
        check(lib().cfd_interp_create(donor.h, r.size, _dptr(p), _iptr(r), C.byref(h)))
        return cls(h)

    @classmethod
    def from_list(cls, recv_node, nweights, inode, weights, stream: int | None = None) -> "Interp":
        r = np.ascontiguousarray(recv_node, dtype=np.int32)
        nw = np.ascontiguousarray(nweights, dtype=np.int32)
        i4 = np.ascontiguousarray(inode, dtype=np.int32).reshape(-1)
        w4 = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        h = C.c_void_p()
        check(lib().cfd_interp_create_list(r.size, _iptr(r), _iptr(nw), _iptr(i4), _dptr(w4),
                                           C.c_void_p(stream) if stream else None, C.byref(h)))
        return cls(h)

    def info(self):
        a, b = C.c_longlong(), C.c_longlong()
        check(lib().cfd_interp_info(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def get(self):
        n, _ = self.info()
        recv = np.zeros(n, np.int32)
        donor = np.zeros(n, np.int32)
        inode = np.zeros(4 * n, np.int32)
        w = np.zeros(4 * n)
        check(lib().cfd_interp_get(self.h, _iptr(recv), _iptr(donor), _iptr(inode), _dptr(w)))
        return recv, donor, inode.reshape(n, 4), w.reshape(n, 4)

    def update(self, q_donor_ptr: int, nnodes_donor: int, q_recv_ptr: int, nnodes_recv: int, nvar: int,
               layout: int = LAYOUT_ROW, stream: int | None = None):
        """Device arrays (raw pointers)."""
        check(lib().cfd_interp_update(self.h, C.c_void_p(q_donor_ptr), int(nnodes_donor), C.c_void_p(q_recv_ptr),
                                      int(nnodes_recv), int(nvar), int(layout),
                                      C.c_void_p(stream) if stream else None))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_interp_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


class HoleMap:
    """Cartesian hole map of one block's walls (tioga::getHoleMap)."""

    def __init__(self, block: Block, isym: int = 3):
        self.h = C.c_void_p()
        check(lib().cfd_holemap_create(block.h, int(isym), C.byref(self.h)))

    def info(self):
        nx = np.zeros(2, np.int32)
        ext = np.zeros(4)
        check(lib().cfd_holemap_info(self.h, _iptr(nx), _dptr(ext)))
        return nx, ext

    def get(self) -> np.ndarray:
        nx, _ = self.info()
        sam = np.zeros(int(nx[0]) * int(nx[1]), np.int32)
        check(lib().cfd_holemap_get(self.h, _iptr(sam)))
        return sam.reshape(nx[1], nx[0])

    def check(self, xy: np.ndarray) -> np.ndarray:
        p = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        out = np.zeros(p.size // 2, np.int32)
        check(lib().cfd_holemap_check(self.h, out.size, _dptr(p), _iptr(out)))
        return out

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_holemap_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def overset_blank(block: Block, others: Sequence[Block], maps: Sequence[HoleMap | None], nfringe: int = 1):
    """(iblank, mandatory) of the block's nodes against the other blocks (processDonors)."""
    n = len(others)
    ob = (C.c_void_p * max(n, 1))(*[o.h.value for o in others])
    mp = (C.c_void_p * max(n, 1))(*[(m.h.value if m is not None else None) for m in maps])
    ib = np.zeros(block.nnode, np.int32)
    md = np.zeros(block.nnode, np.int32)
    check(lib().cfd_overset_blank(block.h, n, ob, mp, int(nfringe), _iptr(ib), _iptr(md)))
    return ib, md


def write_node_data(mesh: Mesh, filename: str, node_q: np.ndarray, mesh_index: int = 0, proc: int = 0):
    """Tecplot node dump (TopologyHolderStrategy::writeNOdeData), node_q (nnode, 4)."""
    q = np.ascontiguousarray(node_q, dtype=np.float64).reshape(-1)
    check(lib().cfd_write_node_data(mesh.h, int(mesh_index), str(filename).encode(), int(proc), _dptr(q)))


def write_tioga_format(mesh: Mesh, filename: str, cell_data: np.ndarray, mesh_index: int = 0, proc: int = 0):
    """Tecplot cell-integer dump (TopologyHolderStrategy::writeTiogaFormat)."""
    a = np.ascontiguousarray(cell_data, dtype=np.int32)
    check(lib().cfd_write_tioga_format(mesh.h, int(mesh_index), str(filename).encode(), int(proc), _iptr(a)))


def overset_connect(blocks: Sequence[Block], maps: Sequence[HoleMap | None], obc_nodes: Sequence[np.ndarray],
                    nfringe: int = 1, mexclude: int = 3) -> dict:
    """Overset assembly of the blocks (tioga::performConnectivity on one rank).

    Returns {"iblank": [node iblank per block], "cell_iblank": [...],
    "interp": [per donor block dict(recv_block, recv_node, donor_cell,
    nweights, inode (n,4), weights (n,4))]}."""
    n = len(blocks)
    bl = (C.c_void_p * n)(*[b.h.value for b in blocks])
    mp = (C.c_void_p * n)(*[(m.h.value if m is not None else None) for m in maps])
    obc = [np.ascontiguousarray(o, dtype=np.int32) for o in obc_nodes]
    op = (C.POINTER(C.c_int) * n)(*[_iptr(o) for o in obc])
    no = np.array([len(o) for o in obc], np.int32)
    h = C.c_void_p()
    check(lib().cfd_overset_connect(n, bl, mp, op, _iptr(no), int(nfringe), int(mexclude), C.byref(h)))
    try:
        out = {"iblank": [], "cell_iblank": [], "interp": []}
        for k, b in enumerate(blocks):
            ib = np.zeros(b.nnode, np.int32)
            ic = np.zeros(b.ncell, np.int32)
            check(lib().cfd_connect_iblank(h, k, _iptr(ib), _iptr(ic)))
            out["iblank"].append(ib)
            out["cell_iblank"].append(ic)
            cnt = C.c_longlong()
            check(lib().cfd_connect_interp_count(h, k, C.byref(cnt)))
            m = cnt.value
            rb, rn, dc, nw = (np.zeros(m, np.int32) for _ in range(4))
            inode = np.zeros((m, 4), np.int32)
            w = np.zeros((m, 4))
            if m:
                check(lib().cfd_connect_interp_get(h, k, _iptr(rb), _iptr(rn), _iptr(dc), _iptr(nw), _iptr(inode),
                                                   _dptr(w)))
            out["interp"].append(dict(recv_block=rb, recv_node=rn, donor_cell=dc, nweights=nw, inode=inode, weights=w))
        return out
    finally:
        lib().cfd_connect_free(h)


# ---- learned relaxation -------------------------------------------------------

def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """The 12-64-64-2 relaxation network (bf16 weights, fp32 arithmetic) on the device."""

    def __init__(self, seed: int = 0):
        self.h = C.c_void_p()
        check(lib().cfd_mlp_create(int(seed), C.byref(self.h)))

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        n = np.zeros(2 * MLP_INPUTS, np.float32)
        check(lib().cfd_mlp_get_params(self.h, _fptr(p), _fptr(n)))
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, np.float32)
        if p is not None and p.size != MLP_PARAMS or n is not None and n.size != 2 * MLP_INPUTS:
            raise ValueError("wrong parameter count")
        check(lib().cfd_mlp_set_params(self.h, _fptr(p) if p is not None else None,
                                       _fptr(n) if n is not None else None))

    def forward(self, x_ptr: int, n: int, y_ptr: int, stream: int | None = None):
        check(lib().cfd_mlp_forward(self.h, C.c_void_p(x_ptr), int(n), C.c_void_p(y_ptr),
                                    C.c_void_p(stream) if stream else None))

    def loss_grad(self, x_ptr: int, t_ptr: int, m_ptr: int | None, n: int):
        loss = C.c_double()
        g = np.zeros(MLP_PARAMS, np.float32)
        check(lib().cfd_mlp_loss_grad(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr),
                                      C.c_void_p(m_ptr) if m_ptr else None, int(n), C.byref(loss), _fptr(g)))
        return loss.value, g

    def train(self, x_ptr: int, t_ptr: int, m_ptr: int | None, n: int, steps: int, batch: int, lr: float,
              seed: int = 0) -> np.ndarray:
        hist = np.zeros(max(steps, 1), np.float32)
        check(lib().cfd_mlp_train(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), C.c_void_p(m_ptr) if m_ptr else None,
                                  int(n), int(steps), int(batch), float(lr), int(seed), _fptr(hist)))
        return hist[:steps]

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.cfd_mlp_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def case_track(case: "Case", on: bool = True):
    check(lib().cfd_case_track(case.h, int(on)))


def case_features(case: "Case", x_ptr: int):
    check(lib().cfd_case_features(case.h, C.c_void_p(x_ptr)))


def case_set_mlp(case: "Case", mlp: Mlp | None, apply_cfl: bool = False, spread: float = 0.0):
    check(lib().cfd_case_set_mlp(case.h, mlp.h if mlp is not None else None, int(apply_cfl), float(spread)))


# ---- SST k-omega ----------------------------------------------------------------

def sst_enable(case: "Case") -> np.ndarray:
    """Allocate the k-omega arrays; returns the freestream (k, omega, mu_t) of mesh 0."""
    check(lib().cfd_sst_enable(case.h))
    out = np.zeros(3)
    check(lib().cfd_sst_freestream(case.h, 0, _dptr(out)))
    return out


def sst_set_inflow(case: "Case", intensity: float, viscosity_ratio: float):
    """Freestream turbulence intensity and mu_t / mu of the SST model (the reference: 0.01, 0.035)."""
    check(lib().cfd_sst_set_inflow(case.h, float(intensity), float(viscosity_ratio)))


def sst_freestream(case: "Case", mesh: int = 0) -> np.ndarray:
    out = np.zeros(3)
    check(lib().cfd_sst_freestream(case.h, int(mesh), _dptr(out)))
    return out


def sst_residual(case: "Case"):
    check(lib().cfd_sst_residual(case.h))


def sst_update_mut(case: "Case"):
    check(lib().cfd_sst_update_mut(case.h))


def hop_latency_us(hops: int = 300, fp64_ops: int = 0, stream: int | None = None) -> float:
    """Latency floor of one dataflow hand-off (wait, compute, publish), in microseconds."""
    v = C.c_double()
    check(lib().cfd_measure_hop_latency(C.c_void_p(stream) if stream else None, int(hops), int(fp64_ops), C.byref(v)))
    return v.value
