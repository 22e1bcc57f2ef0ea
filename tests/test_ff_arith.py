"""Float-float arithmetic of the MIXFF residual, checked on the host.

tests/ff_check.cpp includes the header the device code uses
(tmp_gb300/csrc/ff_arith.h), runs each pair operation on random operands over
twelve decades and both signs, and reports the largest error against the long
double result of the operands' exact values.  The bounds asserted here are
the ones the header documents: sums within 2^-46 of |x| + |y| (also under
near-cancellation), products and square roots within 2^-46 and quotients
within 2^-44 of the exact result; a binary64 value split into a pair and
summed back is exact to 2^-48.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def report(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path_factory.mktemp("ff") / "ff_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe), str(HERE / "ff_check.cpp")],
                   check=True)
    out = subprocess.run([str(exe), "300000"], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.splitlines())}


@pytest.mark.parametrize("op,bound", [("add", 2.0 ** -46), ("sub", 2.0 ** -46), ("cancel", 2.0 ** -46),
                                      ("mul", 2.0 ** -46), ("div", 2.0 ** -44), ("sqrt", 2.0 ** -46),
                                      ("convert", 2.0 ** -48)])
def test_pair_operation_error_bound(report, op, bound):
    assert report[op] <= bound, f"{op}: {report[op]:.3e} > {bound:.3e}"
    assert report[op] > 0.0  # the check did run on inexact cases


def test_special_values(report):
    assert report["sqrt0"] == 0.0
    assert report["order"] == 1.0
