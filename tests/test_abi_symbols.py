"""The C-ABI library loads and exports every function declared in include/*.h
(no compute calls: runs without a GPU)."""
from __future__ import annotations

import ctypes
import re

from conftest import ROOT


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(cfd_\w+)\s*\(", txt, flags=re.M))
    return names


def test_every_declared_symbol_is_exported(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_text(built_lib):
    from tmp_gb300 import abi

    L = abi.lib()
    assert L.cfd_version() >= 10000
    assert L.cfd_mesh_info(None, None, None, None) == -1
    assert b"null" in L.cfd_last_error()


def _defines():
    out = {}
    for h in (ROOT / "include").glob("*.h"):
        for name, val in re.findall(r"^#define\s+(CFD_\w+)\s+(-?\d+)\b", h.read_text(), flags=re.M):
            out[name] = int(val)
    return out


def test_header_constants_match_bindings():
    """The enum values the Python bindings pass across the C ABI are the
    header's (flow, integrator, precision forms, fields, norms, layouts)."""
    from tmp_gb300 import abi

    d = _defines()
    pairs = {"CFD_FLOW_EULER": abi.FLOW_EULER, "CFD_FLOW_LAMINAR": abi.FLOW_LAMINAR, "CFD_FLOW_SST": abi.FLOW_SST,
             "CFD_ADV_RK5": abi.ADV_RK5, "CFD_ADV_LUSGS": abi.ADV_LUSGS,
             "CFD_PREC_FP64": abi.PREC_FP64, "CFD_PREC_FP32": abi.PREC_FP32,
             "CFD_PREC_MIXED": abi.PREC_MIXED, "CFD_PREC_MIXFF": abi.PREC_MIXFF}
    pairs.update({f"CFD_FIELD_{k}": v for k, v in abi.FIELD.items()})
    pairs.update({f"CFD_NORM_{k}": v for k, v in abi.NORM.items()})
    missing = [k for k in pairs if k not in d]
    assert not missing, missing
    wrong = {k: (d[k], v) for k, v in pairs.items() if d[k] != v}
    assert not wrong, wrong


def test_header_compiles_as_c_and_cxx():
    """include/cfdgb.h is a plain C header: it compiles as C99 and as C++17
    with every warning on, so a C, cgo or ctypes caller can include it."""
    import subprocess

    h = str(ROOT / "include" / "cfdgb.h")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c", h],
                ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c++", h]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, (cmd[0], r.stderr)
