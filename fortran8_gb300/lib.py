"""Loader of the in-tree CUDA library (fortran8_gb300/libf8.so).

There is no CPU fallback: if the library is missing or no GPU is present the
calls fail with an explicit error.
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "libf8.so"


@lru_cache(maxsize=1)
def load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built; run fortran8_gb300.build.build() first")
    return C.CDLL(str(LIB_PATH))


@lru_cache(maxsize=1)
def functions() -> dict:
    return abi.bind(load(), "f8_")
