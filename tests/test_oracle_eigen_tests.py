"""The reference's alternative SPD tests of the face candidates (its
compile-time eigen_method, fenep.f90:21, 187-212) in the CPU oracle:
Cardano's roots (fenep.f90:384-423), Sylvester's criterion (446-461) and the
symmetric eigensolver (LAPACK dsyev, 197-212).  Known answers: the repeated
root of sample5.f90:9 ([[2,1,1],[1,2,1],[1,1,2]], eigenvalues 1, 1, 4: Vieta's
and Cardano's sentinels, the symmetric solver's true 1, Sylvester's +1), and
random symmetric matrices against numpy's eigenvalues."""
from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import F8Error, Solver

from .conftest import interior, rel_l2

dp = C.POINTER(C.c_double)
KATS = __import__("json").load(open(__import__("pathlib").Path(__file__).parent / "golden" / "kats.json"))


@pytest.fixture(scope="module")
def test_fn(oracle_lib):
    oracle_lib.f8o_eigen_test.restype = C.c_double
    oracle_lib.f8o_eigen_test.argtypes = [C.c_int, dp]
    return lambda m, a: oracle_lib.f8o_eigen_test(m, np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(dp))


def sym6(S):
    return np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])


def test_repeated_root_known_answers(test_fn):
    a = KATS["vieta_repeated"]["a"]
    assert test_fn(abi.F8_EIGEN_VIETA, a) == -100.0
    assert test_fn(abi.F8_EIGEN_CARDANO, a) == -1.0
    assert abs(test_fn(abi.F8_EIGEN_SYMMETRIC, a) - 1.0) < 1e-14
    assert test_fn(abi.F8_EIGEN_SYLVESTER, a) == 1.0


def test_smallest_eigenvalue_of_random_symmetric_matrices(test_fn):
    rng = np.random.default_rng(11)
    for _ in range(200):
        M = rng.standard_normal((3, 3))
        S = M @ M.T + rng.standard_normal() * np.eye(3)
        lam = np.linalg.eigvalsh(S)[0]
        a = sym6(S)
        for m in (abi.F8_EIGEN_VIETA, abi.F8_EIGEN_CARDANO, abi.F8_EIGEN_SYMMETRIC):
            assert abs(test_fn(m, a) - lam) <= 1e-12 * max(1.0, abs(lam)), (m, test_fn(m, a), lam)
        assert test_fn(abi.F8_EIGEN_SYLVESTER, a) == (1.0 if lam > 0 else -1.0)


def run(oracle, w, steps):
    with Solver(oracle, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        st, drag = s.step(steps)
        return st, drag, s.store()


def test_steps_with_each_test(oracle):
    """The eigen tests that find the smallest eigenvalue choose Vieta's
    candidates except where candidates tie: from C = I all three candidates'
    faces are close to I and their smallest eigenvalues agree to round-off,
    which each formula breaks differently (fields within 1e-6).  Sylvester's
    +-1 chooses the first positive-definite candidate, a different scheme."""
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    out = {}
    for m in (abi.F8_EIGEN_VIETA, abi.F8_EIGEN_CARDANO, abi.F8_EIGEN_SYLVESTER, abi.F8_EIGEN_SYMMETRIC):
        st, drag, o = run(oracle, replace(w, phys=replace(w.phys, eigen_test=m)), 5)
        assert st == abi.F8_OK
        out[m] = o
    for m in (abi.F8_EIGEN_CARDANO, abi.F8_EIGEN_SYMMETRIC):
        assert rel_l2(interior(out[m]["c"]), interior(out[abi.F8_EIGEN_VIETA]["c"])) < 1e-6
    assert rel_l2(interior(out[abi.F8_EIGEN_SYLVESTER]["c"]), interior(out[abi.F8_EIGEN_VIETA]["c"])) > 0


def test_eigen_test_is_validated(oracle):
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    with pytest.raises(F8Error):
        Solver(oracle, w.grid, replace(w.phys, eigen_test=4), w.cyls)
    w2 = configs.scaled(configs.c1_2d(), 16, 16, 1)
    with pytest.raises(F8Error):
        Solver(oracle, w2.grid, replace(w2.phys, eigen_test=abi.F8_EIGEN_SYLVESTER), w2.cyls)
