"""Shared test setup: the `gpu` marker, golden-fixture helpers and library builds."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libcfdgb.so")


def manifest() -> dict:
    return json.loads((GOLDEN / "manifest.json").read_text())


def golden(case: str):
    return np.load(GOLDEN / f"{case}.npz")


@pytest.fixture(scope="session")
def built_lib():
    from tmp_gb300.build import build_library

    return build_library()


@pytest.fixture(scope="session")
def built_oracle():
    import oracle

    return oracle.build()


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
