"""Shared test setup.

`-m "not gpu"` tests run anywhere (oracle vs the reference's golden vectors,
host-side logic, C-ABI symbol exports); `-m gpu` tests need a CUDA device and
call the engine through its C ABI (libd4e.so via ctypes).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


def decode_grid(text: str, width: int, height: int):
    import numpy as np

    return np.array([ord(ch) - 49 for ch in text], dtype=np.int8).reshape(height, width)


def load_cases():
    return json.loads((GOLDEN / "cases.json").read_text())["cases"]


def case_problem(c):
    from d4gb.problem import Problem

    return Problem(c["width"], c["height"], list(c["rows"]), list(c["shapes"]),
                   list(c["counts"]), c["sym"], name=c["name"])


@pytest.fixture(scope="session")
def golden_cases():
    return load_cases()


@pytest.fixture(scope="session")
def catalogue_golden():
    raw = json.loads((GOLDEN / "catalogue.json").read_text())
    return {k: {int(m): v for m, v in d.items()} for k, d in raw.items()}


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def engine():
    """The product library (built in-tree); fails loudly when it cannot load."""
    from d4gb import build

    build.build()
    from d4gb import engine as E

    return E


def has_gpu() -> bool:
    from d4gb import build

    build.build()
    from d4gb import engine as E

    return E.device_count() > 0
