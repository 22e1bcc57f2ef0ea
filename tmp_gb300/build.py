"""Build the CUDA library (tmp_gb300/libcfdgb.so) and the oracle's C library.

Compiles every translation unit for sm_103a only, in parallel, straight with
nvcc (no cmake, no torch extension machinery).  The binary64 kernel unit gets
``-fmad=false`` so each a*b+c is rounded twice, as in the reference's compiled
code; the binary32 unit keeps fused multiply-adds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcfdgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]

# (source, extra flags)
UNITS = [
    ("mesh.cpp", []),
    ("cfd_abi.cpp", []),
    ("k_fp64.cu", ["-fmad=false"]),
    ("k_fp64fma.cu", []),
    ("k_ff.cu", ["-fmad=false"]),
    ("k_fp32.cu", []),
    ("k_misc.cu", []),
    ("k_overset.cu", ["-fmad=false"]),
    ("k_mlp.cu", []),
    ("k_sst.cu", ["-fmad=false"]),
    ("k_noalloc.cu", []),
    ("k_fringe.cu", ["-fmad=false"]),
    ("adt.cpp", []),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return cand


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + [ROOT / "include" / "cfdgb.h"]
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _compile(src: str, extra: list[str]) -> Path:
    s = CSRC / src
    obj = BUILD / (src.replace(".", "_") + ".o")
    if not _stale(obj, s):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_COMMON, *extra, "-c", str(s), "-o", str(obj)]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *NVCC_COMMON, *extra, "-x", "c++", "-c", str(s), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    if LIB.exists() and all(o.stat().st_mtime <= LIB.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    """Compile the C restatement in oracle/ (test infrastructure only)."""
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob  # noqa: E402

    return ob.build(verbose=verbose)


if __name__ == "__main__":
    build_library(verbose=True)
