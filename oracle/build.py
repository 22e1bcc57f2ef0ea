"""Compile oracle/cfd_oracle.c into oracle/liboracle.so (test infrastructure).

-ffp-contract=off keeps every a*b+c as two rounded operations on both x86-64
and aarch64, matching the reference's compiled arithmetic.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cfd_oracle.c"
LIB = HERE / "liboracle.so"


def build(verbose: bool = False) -> Path:
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", str(SRC), "-o", str(tmp),
           "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def reference_root() -> Path:
    """Where the reference's sources are read from: $REFERENCE_ROOT, else the
    container's read-only mount."""
    return Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))


def build_ref(verbose: bool = False, reference_root: str | os.PathLike | None = None) -> Path | None:
    """Compile the reference's own serial path (oracle/_ref/ref_driver) when its
    sources are present; returns None when they are not."""
    reference_root = str(reference_root or globals()["reference_root"]())
    if not (Path(reference_root) / "src" / "UnstructSolver").is_dir():
        return None
    r = subprocess.run(["bash", str(HERE / "build_ref.sh"), reference_root], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout.strip())
    return HERE / "_ref" / "ref_driver"


if __name__ == "__main__":
    build(verbose=True)
    build_ref(verbose=True)
