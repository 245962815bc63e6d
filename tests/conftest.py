"""Shared fixtures: the CPU oracle (checker) and the CUDA library under test."""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from fortran8_gb300 import abi  # noqa: E402

ORACLE_SO = ROOT / "oracle" / "liboracle_f8.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def build_oracle() -> Path:
    src = ROOT / "oracle" / "f8_oracle.cpp"
    if not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    return ORACLE_SO


@pytest.fixture(scope="session")
def oracle_lib():
    return C.CDLL(str(build_oracle()))


@pytest.fixture(scope="session")
def oracle(oracle_lib):
    return abi.bind(oracle_lib, "f8o_")


@pytest.fixture(scope="session")
def gpu():
    """ABI functions of the CUDA library; the test fails (not skips) if it cannot load."""
    from fortran8_gb300 import build, lib
    build.build()
    return lib.functions()


def interior(a: np.ndarray) -> np.ndarray:
    """Interior cells of a halo field (NZ+2, NY+2, NX+2[, NC])."""
    return a[1:-1, 1:-1, 1:-1]


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)
