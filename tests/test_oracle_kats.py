"""The CPU oracle against the reference's known-answer programs and analytic checks.

The reference ships no golden outputs (its data files are git-ignored) and
cannot be compiled here (no Fortran compiler, no FFTW), so the oracle is
pinned by (a) the sample*.f90 known answers (tests/golden/kats.json),
(b) the DFT it replaces (naive DFT and numpy.fft), and (c) analytic
solutions: Taylor-Green decay (fenep.f90:948-979) and a divergence-free
projection.
"""
from __future__ import annotations

import ctypes as C
import json
import math
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import GridSpec, PhysSpec, Solver, empty_state

KATS = json.loads((Path(__file__).parent / "golden" / "kats.json").read_text())
dp = C.POINTER(C.c_double)


def ptr(a):
    return a.ctypes.data_as(dp)


@pytest.fixture(scope="module")
def olib(oracle_lib):
    L = oracle_lib
    L.f8o_vieta.restype = C.c_double
    L.f8o_vieta.argtypes = [dp]
    L.f8o_eig2.argtypes = [dp, dp]
    L.f8o_gauss.argtypes = [C.c_int, dp, dp, dp]
    L.f8o_tdma.argtypes = [C.c_int, dp, dp, dp, dp, dp]
    L.f8o_fft_line.argtypes = [C.c_int, dp, dp, C.c_int]
    L.f8o_fft_solve.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [dp, dp, C.c_double, C.c_double]
    L.f8o_roma.restype = C.c_double
    L.f8o_roma.argtypes = [C.c_double]
    return L


def test_eig2_sample(olib):
    k = KATS["eig2"]
    out = np.zeros(2)
    olib.f8o_eig2(ptr(np.array(k["a"])), ptr(out))
    assert out.tolist() == k["expected"]


def test_tdma_sample6(olib):
    k = KATS["tdma"]
    x = np.zeros(4)
    olib.f8o_tdma(4, *(ptr(np.array(k[n])) for n in "abcd"), ptr(x))
    np.testing.assert_allclose(x, k["expected"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("name", ["gauss3", "gauss3_singular", "gauss6"])
def test_gauss_sample2(olib, name):
    k = KATS[name]
    A = np.array(k["A"], dtype=np.float64)
    n = A.shape[0]
    x = np.zeros(n)
    assert olib.f8o_gauss(n, ptr(np.ascontiguousarray(A)), ptr(np.array(k["b"])), ptr(x)) == 0
    np.testing.assert_allclose(x, k["expected"], rtol=0, atol=1e-13)


def test_vieta_repeated_root_sentinel(olib):
    k = KATS["vieta_repeated"]
    assert olib.f8o_vieta(ptr(np.array(k["a"]))) == k["expected"]


def test_vieta_smallest_eigenvalue(olib):
    rng = np.random.default_rng(7)
    for _ in range(200):
        M = rng.standard_normal((3, 3))
        S = M @ M.T + 0.1 * np.eye(3)
        a = np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])
        lam = np.linalg.eigvalsh(S)[0]
        assert abs(olib.f8o_vieta(ptr(a)) - lam) <= 1e-9 * max(1.0, abs(np.linalg.eigvalsh(S)).max())


def test_roma_kernel_partition_of_unity(olib):
    # the 3-point kernel sums to one over any three consecutive grid points
    for s in np.linspace(-0.5, 0.5, 41):
        tot = sum(olib.f8o_roma(s + d) for d in (-1.0, 0.0, 1.0))
        assert abs(tot - 1.0) < 1e-14


@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 64, 128, 512])
def test_fft_line_vs_dft(olib, n):
    rng = np.random.default_rng(n)
    z = rng.random(n) + 1j * rng.random(n)
    for sign in (-1, 1):
        re, im = z.real.copy(), z.imag.copy()
        olib.f8o_fft_line(n, ptr(re), ptr(im), sign)
        m = np.arange(n)
        dft = np.exp(sign * 2j * np.pi * np.outer(m, m) / n) @ z  # naive DFT, FFTW's convention
        assert np.max(np.abs(re + 1j * im - dft)) <= 1e-13 * max(1.0, np.abs(dft).max())
        ref = np.fft.fft(z) if sign < 0 else np.fft.ifft(z) * n
        assert np.max(np.abs(re + 1j * im - ref)) <= 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("shape,lx", [((8, 16, 32), 4 * math.pi), ((1, 32, 32), 2 * math.pi), ((16, 16, 16), 2 * math.pi)])
@pytest.mark.parametrize("kind", ["poisson", "helmholtz"])
def test_fft_solve_vs_numpy(olib, shape, lx, kind):
    nz, ny, nx = shape
    L = 2 * math.pi
    q = np.random.default_rng(3).random(shape)
    q -= q.mean()
    out = np.zeros_like(q)
    dt_b_re_2 = 1e-3 * 0.9 / 100 / 2
    lhs0, lhs1 = (0.0, -1.0) if kind == "poisson" else (1.0, dt_b_re_2)
    olib.f8o_fft_solve(nx, ny, nz, lx, L, L, ptr(q), ptr(out), lhs0, lhs1)
    dx, dy, dz = lx / nx, L / ny, L / nz
    k2 = lambda n, d: 2 * (1 - np.cos(np.arange(n) * 2 * np.pi / n)) / d ** 2
    kk = k2(nx, dx)[None, None, :] + k2(ny, dy)[None, :, None] + (k2(nz, dz)[:, None, None] if nz > 1 else 0)
    lhs = lhs0 + lhs1 * kk
    qh = np.fft.fftn(q)
    ph = np.where(np.abs(lhs) < 1e-16, 0.0, qh / np.where(np.abs(lhs) < 1e-16, 1.0, lhs))
    ref = np.fft.ifftn(ph).real
    assert np.max(np.abs(out - ref)) <= 1e-13 * max(1.0, np.abs(ref).max())


def _tg2d(n, steps, re=10.0, dt=1e-3):
    g = GridSpec(2, n, n, 1, 2 * math.pi, 2 * math.pi, 2 * math.pi / n)
    ph = PhysSpec(re=re, wi=1.0, beta=1.0, lp2=100.0, dt=dt)
    st = empty_state(g)
    dX = 2 * math.pi / n
    i = np.arange(1, n + 1)[None, :]
    j = np.arange(1, n + 1)[:, None]
    st.arrays["u"][1, 1:-1, 1:-1] = -np.sin(i * dX) * np.cos((j - 0.5) * dX)  # fenep_2d.f90:104-105
    st.arrays["v"][1, 1:-1, 1:-1] = np.cos((i - 0.5) * dX) * np.sin(j * dX)
    return g, ph, st


def test_taylor_green_decay_2d(oracle):
    # Taylor-Green decay check of the reference (fenep_2d.f90:612-639): the
    # discrete mode decays at the rate of the modified wavenumber under CN.
    n, steps, re, dt = 32, 200, 10.0, 1e-3
    g, ph, st = _tg2d(n, steps, re, dt)
    with Solver(oracle, g, ph) as s:
        s.load(st)
        s.step(steps, want_drag=False)
        out = s.store()
    dX = 2 * math.pi / n
    lam = 2 * (2 * (1 - math.cos(dX)) / dX ** 2)
    amp = ((1 - dt * lam / re / 2) / (1 + dt * lam / re / 2)) ** steps
    u0 = st.arrays["u"][1, 1:-1, 1:-1]
    u1 = out["u"][1, 1:-1, 1:-1]
    # the discrete TG mode is an exact eigenfunction of the scheme (the
    # nonlinear term is balanced by the pressure), up to roundoff
    np.testing.assert_allclose(u1, amp * u0, rtol=0, atol=2e-10)
    # continuous decay exp(-2 nu t) differs by the O(dX^2) modified-wavenumber error
    assert abs(u1.max() / u0.max() - math.exp(-2 * steps * dt / re)) < 5e-4


@pytest.mark.parametrize("wl", ["c2", "c3", "c1"])
def test_projection_is_divergence_free(oracle, wl):
    w = {"c2": configs.scaled(configs.c2_3d(), 16, 16, 16),
         "c3": configs.scaled(configs.c3_channel(), 32, 16, 16),
         "c1": configs.scaled(configs.c1_2d(), 32, 32, 1)}[wl]
    with Solver(oracle, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        st, drag = s.step(3)
        d = s.diagnostics()
    assert st == abi.F8_OK
    assert d.div_max < 1e-11
    assert np.all(np.isfinite(drag))


def test_oracle_golden_regression(oracle):
    """Pins the oracle's full step to the committed fixture (tests/golden/make_step_golden.py)."""
    path = Path(__file__).parent / "golden" / "step_golden.npz"
    gold = np.load(path)
    for name in ("c2", "c3", "c1"):
        w = _golden_workload(name)
        with Solver(oracle, w.grid, w.phys, w.cyls) as s:
            s.load(configs.initial_state(w))
            _, drag = s.step(int(gold[f"{name}_steps"]))
            out = s.store()
        for f in ("u", "v", "p"):
            np.testing.assert_allclose(out[f], gold[f"{name}_{f}"], rtol=0, atol=1e-12 * max(1.0, np.abs(gold[f"{name}_{f}"]).max()))
        np.testing.assert_allclose(out["c"], gold[f"{name}_c"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(drag, gold[f"{name}_drag"], rtol=1e-11, atol=1e-11)


def _golden_workload(name):
    from tests.golden.make_step_golden import golden_workload
    return golden_workload(name)


def test_taylor_green_3d_energy_decreases(oracle):
    w = replace(configs.scaled(configs.c2_3d(), 16, 16, 16), cyls=())
    with Solver(oracle, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        e0 = None
        for _ in range(4):
            s.step(5)
            e = s.diagnostics().ke
            if e0 is not None:
                assert e < e0
            e0 = e
