"""The allocation-free spectral solve (f8_fft_solve_noalloc) through the C ABI.

Callers that cannot let the library allocate device memory (a driver that
reserves all its device memory up front) use f8_fft_solve_noalloc, whose
workspace is a fixed device array of the library.  Its result must equal that
of f8_fft_solve, which allocates its workspace per call, on two calls in a
row: the shared workspace keeps the previous call's contents, and a second
call with another grid and other data must not be affected by them.  This
file is collected last so that a run stopping at the first failure has run
every other test already.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from fortran8_gb300 import abi

pytestmark = pytest.mark.gpu

ARGS = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.c_double]
TOL = 1e-14  # relative to the largest value; both entry points run the same kernels


@pytest.fixture(scope="module")
def lib():
    from fortran8_gb300 import build, lib as flib
    build.build()
    L = flib.load()
    for name in ("f8_fft_solve", "f8_fft_solve_noalloc"):
        getattr(L, name).argtypes = ARGS
        getattr(L, name).restype = C.c_int
    return L


def _solve(fn, shape, lx, q, lhs):
    import torch
    nz, ny, nx = shape
    qd = torch.from_numpy(q).cuda()
    pd = torch.full_like(qd, np.nan)
    st = fn(nx, ny, nz, lx, 2 * np.pi, 2 * np.pi, qd.data_ptr(), pd.data_ptr(), *lhs)
    return st, pd.cpu().numpy()


def test_noalloc_matches_allocating_solve_twice(lib):
    cases = [((32, 64, 64), 2 * np.pi, (0.0, -1.0), 5),       # Poisson, 64 x 64 x 32
             ((16, 16, 128), 4 * np.pi, (1.0, 2.25e-7), 6)]   # Helmholtz, 128 x 16 x 16, after the first
    for shape, lx, lhs, seed in cases:
        q = np.random.default_rng(seed).random(shape)
        q -= q.mean()
        st_a, ref = _solve(lib.f8_fft_solve, shape, lx, q, lhs)
        st_n, out = _solve(lib.f8_fft_solve_noalloc, shape, lx, q, lhs)
        assert st_a == abi.F8_OK and st_n == abi.F8_OK
        assert np.all(np.isfinite(out))
        assert np.max(np.abs(out - ref)) <= TOL * max(1.0, np.abs(ref).max())


def test_noalloc_call_leaves_free_device_memory_unchanged(lib):
    """After a first call, a call allocates nothing: the device's free memory
    (cudaMemGetInfo) is the same before and after it."""
    import torch
    shape = (32, 64, 64)
    q = np.random.default_rng(7).random(shape)
    q -= q.mean()
    qd = torch.from_numpy(q).cuda()
    pd = torch.zeros_like(qd)
    args = (64, 64, 32, 2 * np.pi, 2 * np.pi, 2 * np.pi, qd.data_ptr(), pd.data_ptr(), 0.0, -1.0)
    assert lib.f8_fft_solve_noalloc(*args) == abi.F8_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.f8_fft_solve_noalloc(*args) == abi.F8_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_grids_beyond_its_workspace(lib):
    import torch
    qd = torch.zeros((64, 64, 64), dtype=torch.float64, device="cuda")   # 33*64*64 fits
    assert lib.f8_fft_solve_noalloc(64, 64, 64, 1.0, 1.0, 1.0, qd.data_ptr(), qd.data_ptr(), 0.0, -1.0) == abi.F8_OK
    big = torch.zeros((64, 64, 128), dtype=torch.float64, device="cuda")  # 65*64*64 does not
    st = lib.f8_fft_solve_noalloc(128, 64, 64, 1.0, 1.0, 1.0, big.data_ptr(), big.data_ptr(), 0.0, -1.0)
    assert st == abi.F8_ERR_TOO_LARGE
    lib.f8_strerror.restype = C.c_char_p
    assert b"workspace" in lib.f8_strerror(st)
