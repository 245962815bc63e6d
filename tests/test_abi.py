"""The C ABI library loads and exports every entry point that include/f8.h declares."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

from fortran8_gb300 import abi

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"^\s*(?:int|void|const char \*)\s*(f8_\w+)\s*\(", h.read_text(), re.M))
    return sorted(names)


def test_header_declares_the_bound_functions():
    names = declared_functions()
    assert names, "no declarations found"
    for fn in abi.ABI_FUNCTIONS:
        assert "f8_" + fn in names


@pytest.fixture(scope="module")
def cuda_lib():
    from fortran8_gb300 import build, lib
    build.build()
    return lib.load()


def test_library_exports_every_declared_symbol(cuda_lib):
    for name in declared_functions():
        assert hasattr(cuda_lib, name), name


def test_oracle_exports_the_same_abi(oracle_lib):
    """Every entry point but the adjoint (the oracle's gradient reference is the
    differentiable torch restatement, oracle/f8_torch.py)."""
    for name in declared_functions():
        if name[3:] in abi.GPU_FUNCTIONS:
            assert not hasattr(oracle_lib, "f8o_" + name[3:]), name
            continue
        assert hasattr(oracle_lib, "f8o_" + name[3:]), name


def test_grad_is_bound_and_rejects_bad_arguments(cuda_lib):
    fns = abi.bind(cuda_lib, "f8_")
    assert "grad" in fns
    dp = (C.c_double * 3)()
    assert fns["grad"](None, 1, 0, None, None, None, dp, None, None) == abi.F8_ERR_ARG


def test_invalid_arguments_are_rejected_without_a_device(cuda_lib):
    fns = abi.bind(cuda_lib, "f8_")
    h = C.c_void_p()
    ph = abi.Phys()
    fns["default_phys"](C.byref(ph))
    bad = abi.Grid(3, 30, 16, 16, 1.0, 1.0, 1.0, 0, 0.0)  # 30 is not a power of two
    assert fns["create"](C.byref(h), C.byref(bad), C.byref(ph), None, 0, 0, 0) == abi.F8_ERR_ARG
    bad2 = abi.Grid(2, 16, 16, 4, 1.0, 1.0, 1.0, 0, 0.0)  # 2D needs nz == 1
    assert fns["create"](C.byref(h), C.byref(bad2), C.byref(ph), None, 0, 0, 0) == abi.F8_ERR_ARG
    assert fns["step"](None, 1, None) == abi.F8_ERR_ARG
    assert fns["strerror"](abi.F8_ERR_NAN).decode().startswith("NaN")


def test_no_device_is_reported_not_hidden(cuda_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    fns = abi.bind(cuda_lib, "f8_")
    h = C.c_void_p()
    ph = abi.Phys()
    fns["default_phys"](C.byref(ph))
    g = abi.Grid(3, 16, 16, 16, 1.0, 1.0, 1.0, 0, 0.0)
    assert fns["create"](C.byref(h), C.byref(g), C.byref(ph), None, 0, 0, 0) == abi.F8_ERR_NO_DEVICE
