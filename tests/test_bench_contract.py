"""bench.py's reference arm, run on the host cores without a GPU: the JSON
line it prints (the fields the benchmark contract names), its rank rule
under torchrun, and its argument checks."""
from __future__ import annotations

import json
import os
import subprocess
import sys

from conftest import ROOT


def run_bench(*args, env=None, timeout=600):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=e, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_line(built_oracle):
    """One RK5 step of C1 (8,192 cells) per copy, after three untimed ones."""
    r = run_bench("--impl", "reference", "--config", "c1", "--steps", "1", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["unit"] == "cell-iters/s" and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["steps"] == 1 and d["warmup"] >= 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"].startswith("C1") and d["config"]["ncell"] == 8192
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == (os.cpu_count() or 1) and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and "copies" in cb["sample"]
    e2e = d["e2e"]
    assert e2e == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly(built_oracle):
    """Under torchrun only rank 0 runs and prints the reference arm."""
    r = run_bench("--impl", "reference", "--config", "c1", "--steps", "1", env={"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_aoa_only_for_c3(built_oracle):
    """--aoa sets the angle of the C3 case and is refused for the others."""
    r = run_bench("--impl", "reference", "--config", "c1", "--aoa", "3", "--steps", "1", timeout=300)
    assert r.returncode != 0
    assert "--aoa applies to the c3 workload only" in r.stderr + r.stdout
