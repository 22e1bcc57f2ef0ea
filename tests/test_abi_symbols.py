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
