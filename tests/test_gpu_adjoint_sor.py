"""Discrete adjoint of the SOR variant of the FP64 step (f8_grad on an
F8_POISSON_SOR context).

The SOR solve maps the right-hand side to the zero-mean pressure correction
through the pseudo-inverse of the symmetric 7-point Laplacian (to its
tolerance), so the adjoint runs the same red-black SOR on the zero-mean part
of the adjoint right-hand side.  The FFT + tridiagonal solve inverts the same
discrete Laplacian exactly, so with a tight SOR tolerance the two variants'
gradients agree; with the reference's tolerance (1e-5) they differ by the
SOR truncation (a few 1e-9 relative on the channel case below).  Segments recomputed from a checkpoint restart the SOR from
the checkpointed Phi, so they repeat the forward's iterates.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi
from fortran8_gb300.solver import F8Error, Solver

from .adjoint_cases import case, param_vector, with_params

pytestmark = pytest.mark.gpu


def grad(fns, w, st, step0, n, poisson, K=0, precision=abi.F8_FP64):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision, poisson=poisson) as s:
        s.load(st, step0)
        status, J, dp, _, drag = s.grad(n, K)
        final = s.store()
    return status, J, dp, drag, final


def tight(w):
    return replace(w, phys=replace(w.phys, sor_eps=1e-13, sor_itrmax=20000))


@pytest.mark.parametrize("name", ["channel", "periodic"])
def test_sor_gradient_matches_fft_gradient_at_tight_tolerance(gpu, oracle, name):
    w, st, step0 = case(name, oracle)
    w = tight(w)
    n = 4
    st1, J1, d1, _, _ = grad(gpu, w, st, step0, n, abi.F8_POISSON_SOR, K=2)
    st2, J2, d2, _, _ = grad(gpu, w, st, step0, n, abi.F8_POISSON_FFT, K=2)
    assert st1 == abi.F8_OK and st2 == abi.F8_OK
    assert abs(J1 - J2) <= 1e-10 * abs(J2)
    for q, (a, b) in enumerate(zip(d1, d2)):
        assert abs(a - b) <= 1e-7 * abs(b) + 1e-11, (q, a, b)


def test_sor_gradient_matches_sor_central_differences(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    w = tight(w)
    n = 3
    _, _, dp, _, _ = grad(gpu, w, st, step0, n, abi.F8_POISSON_SOR)
    base = param_vector(w)
    for q in range(len(base)):
        h = 1e-4 * max(abs(base[q]), 1.0)
        vals = []
        for sgn in (1, -1):
            b = base.copy()
            b[q] += sgn * h
            wq = with_params(w, b)
            with Solver(gpu, wq.grid, wq.phys, wq.cyls, poisson=abi.F8_POISSON_SOR) as s:
                s.load(st, step0)
                _, drag = s.step(n)
            vals.append(drag[:, :, 0].sum() / n)
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(dp[q] - fd) <= 1e-4 * abs(fd) + 1e-8, (q, dp[q], fd)


def test_sor_gradient_at_reference_tolerance(gpu, oracle):
    """At the reference's tolerance (1e-5) the gradient is that of the SOR
    trajectory: within 1e-6 of the exact-solve gradient (measured 7e-9 on this
    case); recomputed segments
    repeat the forward (checkpoint intervals agree to round-off, the state
    left equals f8_step's)."""
    w, st, step0 = case("channel", oracle)
    n = 6
    res = [grad(gpu, w, st, step0, n, abi.F8_POISSON_SOR, K=K) for K in (0, 2, 3)]
    _, _, dfft, _, _ = grad(gpu, w, st, step0, n, abi.F8_POISSON_FFT)
    with Solver(gpu, w.grid, w.phys, w.cyls, poisson=abi.F8_POISSON_SOR) as s:
        s.load(st, step0)
        _, drag = s.step(n)
        out = s.store()
    for status, J, dp, dg, final in res:
        assert status == abi.F8_OK
        assert np.array_equal(dg, drag)
        for f in ("u", "v", "w", "p", "c"):
            assert np.array_equal(final[f], out[f]), f
        for q, (a, b) in enumerate(zip(dp, res[0][2])):
            assert abs(a - b) <= 1e-9 * abs(b) + 1e-12, (q, a, b)
    print("sor", list(res[0][2]), "fft", list(dfft))
    for q, (a, b) in enumerate(zip(res[0][2], dfft)):
        assert abs(a - b) <= 1e-6 * abs(b) + 1e-10, (q, a, b)


def test_mixed_sor_gradient_is_unsupported(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED, poisson=abi.F8_POISSON_SOR) as s:
        s.load(st, step0)
        with pytest.raises(F8Error):
            s.grad(2)
