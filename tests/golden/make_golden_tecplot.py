"""Generate tests/golden/tecplot.npz: the reference's own Tecplot field dumps.

Runs oracle/_ref/ref_driver (the reference's serial solver path, compiled from
its sources by oracle/build_ref.sh) with WRITE_TECPLOT=1 and no steps on two
golden cases, starting from their fixtures' non-uniform initial fields, and
keeps the bytes of the files that TopologyHolderStrategy::writeCellData,
writeNOdeData and writeTiogaFormat write (node data: node i, variable k =
0.001*i + k; cell integers: cell c -> c % 3 - 1).

usage: python tests/golden/make_golden_tecplot.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
DRV = ROOT / "oracle" / "_ref" / "ref_driver"
CASES = ("mixed_lam_lusgs", "omesh_euler_rk5")


def main():
    man = json.loads((HERE / "manifest.json").read_text())
    out = {}
    for name in CASES:
        c = man[name]
        g = np.load(HERE / f"{name}.npz")
        with tempfile.TemporaryDirectory() as td:
            init = Path(td) / "init.bin"
            np.ascontiguousarray(g["init_U"], np.float64).tofile(init)
            od = Path(td) / "out"
            env = dict(os.environ, WRITE_TECPLOT="1")
            subprocess.run([str(DRV), str(HERE / c["mesh"]), str(c["wall_tag"]), str(c["far_tag"]), c["flow"],
                            c["advance"], str(c["mach"]), str(c["aoa"]), str(c["re"]), str(c["cfl"]), "0", str(od),
                            str(init)], check=True, cwd=td, env=env, stdout=subprocess.DEVNULL)
            for key, fname in (("cells", "cells_1_1"), ("nodes", "nodes_1_1"), ("tioga", "tioga00")):
                data = (od / fname).read_bytes()
                out[f"{name}/{key}"] = np.frombuffer(data, np.uint8)
                print(name, key, len(data), "bytes")
    np.savez_compressed(HERE / "tecplot.npz", **out)


if __name__ == "__main__":
    sys.exit(main())
