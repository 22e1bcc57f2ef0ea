"""Test oracle: a CPU restatement of the reference solver's per-iteration path.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg may import this package, and only as the checker or as the
reported CPU baseline; the product path (tmp_gb300) never uses it.

Pinning: tests/test_oracle_golden.py checks the oracle against fixtures dumped
by the reference's own compiled code (tests/golden/).

  grd.read_grd      .grd reader + cell assembly restated in numpy/Python
                    (reader/UnstructReader.h:124-272, UniTioga/CellBrick.cpp:13-136)
  Oracle            ctypes wrapper of cfd_oracle.c (geometry, residual, RK5, LU-SGS)
  nodal_weights, donor_search, interp_update
                    overset weights / containment / fringe update restated in C
                    (mathTools/math.cpp, UniTioga/checkContainment.cpp, dataUpdate.cpp)
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import grd  # noqa: F401
from .build import LIB, build

FIELD = dict(U=0, W=1, R=2, GRAD=3, PHI=4, SPEC_C=5, SPEC_V=6, DT=7, DIAG=8, DW1=9, DW=10, GRADT=11, MU=12,
             UEDGE=13, MUEDGE=14, VOL=15, CENTER=16, NORMAL=17, AREA=18, ECENTER=19, WALLDIST=20, UL=21, UR=22,
             WNOW=23)
# values per element, per-face flag
SHAPE = dict(U=(4, 0), W=(4, 0), R=(4, 0), GRAD=(8, 0), PHI=(4, 0), SPEC_C=(1, 0), SPEC_V=(1, 0), DT=(1, 0),
             DIAG=(1, 0), DW1=(4, 0), DW=(4, 0), GRADT=(2, 0), MU=(1, 0), UEDGE=(4, 1), MUEDGE=(1, 1), VOL=(1, 0),
             CENTER=(2, 0), NORMAL=(2, 1), AREA=(1, 1), ECENTER=(2, 1), WALLDIST=(1, 0), UL=(4, 1), UR=(4, 1),
             WNOW=(4, 0))

_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        ip, dp, vp = C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, dp, C.c_int, ip, ip, C.c_int, ip, ip, ip, ip]
        L.orc_free.argtypes = [vp]
        L.orc_geometry.argtypes = [vp]
        L.orc_set_freestream.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_init_freestream.argtypes = [vp]
        L.orc_cons_from_U.argtypes = [vp]
        L.orc_residual.argtypes = [vp, C.c_int]
        L.orc_residual.restype = C.c_int
        L.orc_solve_time.argtypes = [vp, C.c_double]
        L.orc_rk_step.argtypes = [vp, C.c_int]
        L.orc_rk_step.restype = C.c_int
        L.orc_lusgs_step.argtypes = [vp, C.c_double, C.c_int]
        L.orc_lusgs_step.restype = C.c_int
        L.orc_wall_force.argtypes = [vp, dp]
        L.orc_hold_limiter.argtypes = [vp, C.c_int]
        L.orc_hold_turbulence.argtypes = [vp, C.c_int]
        L.orc_sst_production_limit.argtypes = [vp, C.c_double]
        L.orc_field.argtypes = [vp, C.c_int]
        L.orc_field.restype = dp
        L.orc_nodal_weights.argtypes = [C.c_long, ip, dp, dp, dp]
        L.orc_nodal_weights.restype = C.c_long
        L.orc_donor_search.argtypes = [dp, C.c_int, ip, ip, C.c_long, dp, ip, ip, dp]
        L.orc_adt_search.argtypes = [dp, C.c_int, ip, ip, C.c_char_p, C.c_long, dp, ip, dp, ip, ip]
        L.orc_holemap.argtypes = [dp, C.c_int, ip, ip, C.c_int, ip, C.c_int, ip, dp, ip, C.c_long]
        L.orc_holemap.restype = C.c_int
        L.orc_holemap_check.argtypes = [ip, dp, ip, C.c_long, dp, ip]
        L.orc_interp_update.argtypes = [C.c_long, ip, ip, ip, dp, dp, C.c_long, dp, C.c_long, C.c_int, C.c_int]
        L.orc_sst_enable.argtypes = [vp, C.c_int, C.c_double, C.c_double]
        for f in ("orc_sst_cons", "orc_sst_equation", "orc_sst_diag", "orc_sst_update_mut"):
            getattr(L, f).argtypes = [vp]
        L.orc_sst_field.argtypes = [vp, C.c_int]
        L.orc_sst_field.restype = dp
        _lib = L
    return _lib


class Oracle:
    """One mesh, one flow strategy; mirrors the reference's serial driver calls."""

    def __init__(self, mesh: "grd.Topo", mach: float, aoa: float, re: float, viscous: bool,
                 density: float = 1.225, pressure: float = 101325.0):
        L = _load()
        self.m = mesh
        self._keep = [np.ascontiguousarray(a) for a in (mesh.xy, mesh.edge_nodes, mesh.lr, mesh.cell_verts,
                                                         mesh.cell_nvert, mesh.cell_edges, mesh.cell_nedge)]
        xy, en, lr, cv, cnv, ce, cne = self._keep
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        self.h = L.orc_create(mesh.nnode, xy.ctypes.data_as(C.POINTER(C.c_double)), mesh.nedge, ip(en), ip(lr),
                              mesh.ncell, ip(cv), ip(cnv), ip(ce), ip(cne))
        L.orc_geometry(self.h)
        L.orc_set_freestream(self.h, mach, aoa, re, density, pressure, int(viscous))
        L.orc_init_freestream(self.h)
        L.orc_cons_from_U(self.h)
        self.viscous = viscous

    def set_U(self, U: np.ndarray):
        self.field("U")[:] = np.asarray(U, np.float64).reshape(self.field("U").shape)
        _load().orc_cons_from_U(self.h)

    def residual(self, first_order: bool = False) -> int:
        return _load().orc_residual(self.h, int(first_order))

    def solve_time(self, cfl: float):
        _load().orc_solve_time(self.h, cfl)

    def rk_step(self, first_order: bool = False) -> int:
        return _load().orc_rk_step(self.h, int(first_order))

    def lusgs_step(self, cfl: float, first_order: bool = False) -> int:
        return _load().orc_lusgs_step(self.h, cfl, int(first_order))

    # SST k-omega: arrays by name, (values per element, per face)
    SST = dict(SST_T=(21, 2, 0), SST_TFACE=(22, 2, 1), SST_TGRAD=(23, 4, 0), SST_F1=(24, 1, 0), SST_F2=(25, 1, 0),
               SST_MUT=(26, 1, 0), SST_MUTF=(27, 1, 1), SST_FCONV=(28, 2, 1), SST_FVISC=(29, 2, 1), SST_R=(30, 2, 0),
               SST_DIAG=(31, 2, 0), SST_W=(40, 2, 0), SST_DW1=(41, 2, 0), SST_DW=(42, 2, 0))

    def sst_enable(self, coupled: bool, tu: float = 0.01, ratio: float = 0.035):
        """Allocate the SST arrays and set the freestream k, omega, mu_t; coupled: every LU-SGS step then runs the
        turbulence model with the flow (the build's turbulent path), else its functions are called one by one."""
        L = _load()
        L.orc_sst_enable(self.h, int(coupled), float(tu), float(ratio))
        L.orc_sst_cons(self.h)

    def sst_cons(self):
        _load().orc_sst_cons(self.h)

    def sst_equation(self):
        _load().orc_sst_equation(self.h)

    def sst_diag(self):
        _load().orc_sst_diag(self.h)

    def sst_update_mut(self):
        _load().orc_sst_update_mut(self.h)

    def sst_field(self, name: str) -> np.ndarray:
        fid, width, per_face = self.SST[name]
        n = (self.m.nedge if per_face else self.m.ncell) * width
        a = np.ctypeslib.as_array(_load().orc_sst_field(self.h, fid), shape=(n,))
        return a.reshape(-1, width) if width > 1 else a

    def hold_limiter(self, on: bool = True):
        """Freeze the limiter factors at their current values (analysis only)."""
        _load().orc_hold_limiter(self.h, int(on))

    def hold_turbulence(self, on: bool = True):
        """Freeze k, omega and mu_t in the coupled step (analysis only)."""
        _load().orc_hold_turbulence(self.h, int(on))

    def sst_production_limit(self, factor: float):
        """Limit the k equation's production to factor * beta* rho k omega (0: the reference's unlimited
        production; analysis only)."""
        _load().orc_sst_production_limit(self.h, float(factor))

    def wall_force(self) -> np.ndarray:
        """(Fx, Fy) through the wall faces in the last residual evaluation."""
        f = np.zeros(2)
        _load().orc_wall_force(self.h, f.ctypes.data_as(C.POINTER(C.c_double)))
        return f

    def field(self, name: str) -> np.ndarray:
        """A live numpy view of one oracle array."""
        width, per_face = SHAPE[name]
        n = (self.m.nedge if per_face else self.m.ncell) * width
        p = _load().orc_field(self.h, FIELD[name])
        a = np.ctypeslib.as_array(p, shape=(n,))
        return a.reshape(-1, width) if width > 1 else a

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_free(self.h)
            self.h = None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def nodal_weights(nvert, xv, xp):
    """computeNodalWeight2D for n pairs: nvert[n], xv[n,4,2], xp[n,2] -> (frac[n,4], n_singular)."""
    nv = np.ascontiguousarray(nvert, np.int32)
    x = np.ascontiguousarray(xv, np.float64).reshape(-1)
    p = np.ascontiguousarray(xp, np.float64).reshape(-1)
    out = np.zeros(4 * nv.size)
    bad = _load().orc_nodal_weights(nv.size, _ip(nv), _dp(x), _dp(p), _dp(out))
    return out.reshape(-1, 4), int(bad)


def donor_search(xy, cell_verts, cell_nvert, pts):
    """Brute-force containment: (lowest containing cell, number of containing cells, its weights)."""
    x = np.ascontiguousarray(xy, np.float64).reshape(-1)
    cv = np.ascontiguousarray(cell_verts, np.int32).reshape(-1)
    nv = np.ascontiguousarray(cell_nvert, np.int32)
    p = np.ascontiguousarray(pts, np.float64).reshape(-1)
    n = p.size // 2
    donor = np.zeros(n, np.int32)
    cnt = np.zeros(n, np.int32)
    w = np.zeros(4 * n)
    _load().orc_donor_search(_dp(x), nv.size, _ip(cv), _ip(nv), n, _dp(p), _ip(donor), _ip(cnt), _dp(w))
    return donor, cnt, w.reshape(n, 4)


def adt_search(xy, cell_verts, cell_nvert, pts, unaccept=None, tags=None, res=None):
    """MeshBlock::search as the reference runs it: the donor (mesh cell, -1 for none) of every point, the point
    whose search each took (coincident points share one) and the resolutions merged over coincident points."""
    x = np.ascontiguousarray(xy, np.float64).reshape(-1)
    cv = np.ascontiguousarray(cell_verts, np.int32).reshape(-1)
    nv = np.ascontiguousarray(cell_nvert, np.int32)
    p = np.ascontiguousarray(pts, np.float64).reshape(-1)
    n = p.size // 2
    ua = np.zeros(nv.size, np.uint8) if unaccept is None else np.ascontiguousarray(unaccept, np.uint8)
    tg = np.ones(n, np.int32) if tags is None else np.ascontiguousarray(tags, np.int32)
    rt = np.ones(n) if res is None else np.array(res, np.float64)
    donor = np.zeros(n, np.int32)
    xtag = np.zeros(n, np.int32)
    _load().orc_adt_search(_dp(x), nv.size, _ip(cv), _ip(nv), ua.ctypes.data_as(C.c_char_p), n, _dp(p), _ip(tg),
                           _dp(rt), _ip(donor), _ip(xtag))
    return donor, xtag, rt


def interp_update(recv, nw, inode, w, q, nnodes, qr, nnodes_recv, nvar, layout):
    """getInterpolatedSolution + updateSolnData into qr (modified in place)."""
    r = np.ascontiguousarray(recv, np.int32)
    n_w = np.ascontiguousarray(nw, np.int32)
    i4 = np.ascontiguousarray(inode, np.int32).reshape(-1)
    w4 = np.ascontiguousarray(w, np.float64).reshape(-1)
    qa = np.ascontiguousarray(q, np.float64).reshape(-1)
    assert qr.dtype == np.float64 and qr.flags.c_contiguous
    _load().orc_interp_update(r.size, _ip(r), _ip(n_w), _ip(i4), _dp(w4), _dp(qa), nnodes, _dp(qr), nnodes_recv,
                              nvar, layout)
    return qr


def holemap(xy, cell_verts, cell_nvert, wall_nodes, isym=3):
    """Hole map of one block's walls: (nx[2], extents[4], sam[ny, nx])."""
    x = np.ascontiguousarray(xy, np.float64).reshape(-1)
    cv = np.ascontiguousarray(cell_verts, np.int32).reshape(-1)
    nv = np.ascontiguousarray(cell_nvert, np.int32)
    wn = np.ascontiguousarray(wall_nodes, np.int32)
    nxy = np.zeros(2, np.int32)
    geo = np.zeros(4)
    sam = np.zeros(200_000, np.int32)
    rc = _load().orc_holemap(_dp(x), nv.size, _ip(cv), _ip(nv), wn.size, _ip(wn), isym, _ip(nxy), _dp(geo), _ip(sam),
                             sam.size)
    if rc != 0:
        raise ValueError("hole map larger than 200000 cells")
    return nxy, geo, sam[:nxy[0] * nxy[1]].reshape(nxy[1], nxy[0]).copy()


def holemap_check(nxy, geo, sam, pts):
    p = np.ascontiguousarray(pts, np.float64).reshape(-1)
    n = p.size // 2
    out = np.zeros(n, np.int32)
    nx = np.ascontiguousarray(nxy, np.int32)
    g = np.ascontiguousarray(geo, np.float64)
    s = np.ascontiguousarray(sam, np.int32).reshape(-1)
    _load().orc_holemap_check(_ip(nx), _dp(g), _ip(s), n, _dp(p), _ip(out))
    return out


def blank(self_topo, others, nfringe=1):
    """processDonors' hole test and mandatory fringes (bookkeeping.cpp:88-186).

    others: list of (topo, wall_nodes or None, isym).  Returns (iblank, mandatory)."""
    xy = self_topo.xy.reshape(-1, 2)
    ib = np.ones(len(xy), np.int32)
    for topo, wall, isym in others:
        if wall is None:
            continue
        donor, _, _ = donor_search(topo.xy, topo.cell_verts, topo.cell_nvert, xy)
        nxy, geo, sam = holemap(topo.xy, topo.cell_verts, topo.cell_nvert, wall, isym)
        inside = holemap_check(nxy, geo, sam, xy)
        ib[(donor < 0) & (inside == 1)] = 0
    tag = (ib == 0).astype(np.int32)
    cv = self_topo.cell_verts.reshape(-1, 4)
    for _ in range(nfringe):
        tag1 = tag.copy()
        for c in range(self_topo.ncell):
            vs = cv[c, :self_topo.cell_nvert[c]]
            if np.any(tag[vs] == 1):
                tag1[vs] = 1
        tag = tag1
    return ib, ((tag == 1) & (ib == 1)).astype(np.int32)


def wall_nodes(topo):
    """Ends of the wall faces (right side == wall code), ascending."""
    lr = topo.lr.reshape(-1, 2)
    en = topo.edge_nodes.reshape(-1, 2)
    return np.unique(en[lr[:, 1] == -2].reshape(-1)).astype(np.int32)


def cell_iblank(cell_verts, cell_nvert, node_iblank):
    """MeshBlock::getCellIblanks (bookkeeping.cpp:654-705): 0 if any node is 0,
    else -1 if every node is -1, else 1 (nodes visited in vertex order)."""
    cv = np.asarray(cell_verts).reshape(-1, 4)
    ibl = np.asarray(node_iblank)
    out = np.ones(len(cv), np.int32)
    for c in range(len(cv)):
        n = int(cell_nvert[c])
        vals = ibl[cv[c, :n]]
        if np.any(vals == 0):
            out[c] = 0
        elif np.all(vals == -1):
            out[c] = -1
    return out
