"""Discrete adjoint of the 2D FP64 step (f8_grad on a 2D context,
fenep_2d.f90:1912-1966), against central differences of the GPU forward.

Cases: the 2D periodic box with a filled cylinder (the 2D benchmark
configuration at 32^2) and a 2D wall channel (Poiseuille base flow, filled
cylinder, the reference's wall mode with the polymer update on the ghost
rows), each advanced by the CPU oracle from a stretched polymer field and with
the cylinder off the grid lines; the FENE-P step and the Newtonian one
(beta = 1).  Checked: dJ/d(Wi, beta, L^2, centre) of the time-averaged drag
against central differences (relative step 1e-4, 1e-6 for the centres) within
1e-4; the adjoint of
the initial state along a random direction against the directional central
difference; checkpoint intervals agree and the state left equals f8_step's;
the SOR variant's gradient equals the FFT one at a tight SOR tolerance.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import CylSpec, GridSpec, Solver

from .adjoint_cases import param_vector, with_params

pytestmark = pytest.mark.gpu

PI = np.pi


def case2d(name, oracle, spinup=8, beta=None):
    if name == "periodic":
        w = configs.c1_2d(32)
        w = replace(w, cyls=(replace(w.cyls[0], xc=PI + 0.0123, yc=PI + 0.0371),))
    else:
        n = 32
        g = GridSpec(2, n, n // 2, 1, 2 * PI, PI, 2 * PI / n, abi.F8_BC_WALLS, 0.0)
        w = configs.Workload("channel2d", g, replace(configs.c1_2d().phys, re=20.0, dt=2e-3), (CylSpec(PI + 0.0123, PI / 2 + 0.0371, 0.4),),
                             10, 5, 1e-2, "poiseuille")
    if beta is not None:
        w = replace(w, phys=replace(w.phys, beta=beta))
    st = configs.initial_state(w)
    g = w.grid
    dX = g.lx / g.nx
    i = np.arange(0, g.nx + 2)[None, None, :]
    j = np.arange(0, g.ny + 2)[None, :, None]
    cxx = 1.0 + 20.0 * (1.0 + 0.5 * np.sin((i - 0.5) * dX) * np.cos((j - 0.5) * dX))
    st.arrays["c"][..., 0] = np.broadcast_to(cxx, st.arrays["c"].shape[:3])
    st.arrays["c"][..., 1] = 0.5 * np.broadcast_to(np.cos((i - 0.5) * dX), st.arrays["c"].shape[:3])
    with Solver(oracle, w.grid, w.phys, w.cyls) as o:
        o.load(st)
        o.step(spinup)
        out = o.store()
    return w, out, spinup


def grad(gpu, w, st, step0, n, K=0, seed=None, want_dstate=False):
    with Solver(gpu, w.grid, w.phys, w.cyls) as s:
        s.load(st, step0)
        status, J, dp, ds, drag = s.grad(n, K, None, seed, want_dstate)
        final = s.store()
    assert status == abi.F8_OK, status
    return J, dp, ds, drag, final


def mean_drag(gpu, w, st, step0, n):
    with Solver(gpu, w.grid, w.phys, w.cyls) as s:
        s.load(st, step0)
        _, drag = s.step(n)
    return drag[:, :, 0].sum() / n


@pytest.mark.parametrize("name,beta", [("periodic", None), ("channel", None), ("channel", 1.0)])
def test_2d_gradient_matches_central_differences(gpu, oracle, name, beta):
    w, st, step0 = case2d(name, oracle, beta=beta)
    n = 4
    _, dp, _, _, _ = grad(gpu, w, st, step0, n)
    base = param_vector(w)
    fds = []
    for q in range(len(base)):
        if beta == 1.0 and q < 3:
            continue          # Newtonian: Wi and L^2 do not enter, and beta = 1 switches the polymer off
        # Roma's kernel is C1: a stencil weight whose offset crosses one of its
        # break points (|r| = 0.5, 1.5) within +-h makes the central difference
        # converge at O(h) only; the filled cylinder's many markers make such
        # a crossing likely at h = 1e-4 |p|, so the centres use 1e-6 |p|
        h = (1e-4 if q < 3 else 1e-6) * max(abs(base[q]), 1.0)
        vals = []
        for sgn in (1, -1):
            b = base.copy()
            b[q] += sgn * h
            vals.append(mean_drag(gpu, with_params(w, b), st, step0, n))
        fd = (vals[0] - vals[1]) / (2 * h)
        fds.append((q, dp[q], fd))
    print(name, beta, fds)
    for q, a, fd in fds:
        assert abs(a - fd) <= 1e-4 * abs(fd) + 1e-8, (q, a, fd)


def test_2d_state_adjoint_along_a_direction(gpu, oracle):
    w, st, step0 = case2d("channel", oracle)
    n = 3
    _, _, ds, _, _ = grad(gpu, w, st, step0, n, want_dstate=True)
    rng = np.random.default_rng(5)
    g = w.grid
    d = {name: np.zeros_like(st.arrays[name]) for name in ("u", "v", "c")}
    for name in ("u", "v"):
        d[name][1:-1, 1:-1, 1:-1] = rng.standard_normal((1, g.ny, g.nx))
    d["c"][1:-1, 1:-1, 1:-1, 0] = rng.standard_normal((1, g.ny, g.nx))
    d["c"][1:-1, 1:-1, 1:-1, 1] = rng.standard_normal((1, g.ny, g.nx))
    lin = sum(np.sum(ds[name] * d[name]) for name in d)
    h = 1e-5
    vals = []
    for sgn in (1, -1):
        sp = st.copy()
        for name in d:
            sp.arrays[name] = sp.arrays[name] + sgn * h * d[name]
        vals.append(mean_drag(gpu, w, sp, step0, n))
    fd = (vals[0] - vals[1]) / (2 * h)
    print("directional", lin, fd)
    assert abs(lin - fd) <= 1e-4 * abs(fd) + 1e-9


def test_2d_checkpoints_agree_and_state_advances(gpu, oracle):
    w, st, step0 = case2d("channel", oracle)
    n = 6
    res = [grad(gpu, w, st, step0, n, K=K) for K in (1, 4, 0)]
    with Solver(gpu, w.grid, w.phys, w.cyls) as s:
        s.load(st, step0)
        _, drag = s.step(n)
        out = s.store()
    for J, dp, _, dg, final in res:
        assert np.array_equal(dg, drag)
        for name in ("u", "v", "p", "c"):
            assert np.array_equal(final[name], out[name]), name
        for q, (a, b) in enumerate(zip(dp, res[0][1])):
            assert abs(a - b) <= 1e-9 * abs(b) + 1e-12, (q, a, b)


def test_2d_sor_gradient_matches_fft_gradient(gpu, oracle):
    """The SOR variant's adjoint in 2D: at a tight SOR tolerance the gradient
    equals the FFT + tridiagonal one (the same discrete Laplacian)."""
    w, st, step0 = case2d("channel", oracle)
    w = replace(w, phys=replace(w.phys, sor_eps=1e-13, sor_itrmax=20000))
    out = []
    for poisson in (abi.F8_POISSON_SOR, abi.F8_POISSON_FFT):
        with Solver(gpu, w.grid, w.phys, w.cyls, poisson=poisson) as s:
            s.load(st, step0)
            status, J, dp, _, _ = s.grad(3, 0)
        assert status == abi.F8_OK
        out.append(dp)
    for q, (a, b) in enumerate(zip(*out)):
        assert abs(a - b) <= 1e-7 * abs(b) + 1e-11, (q, a, b)
