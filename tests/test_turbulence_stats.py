"""Turbulence statistics (all_time_dif) and the energy spectrum (energy_single)
of the oracle: Parseval, a single Fourier mode, and a numpy restatement."""
from __future__ import annotations

import math

import numpy as np
import pytest

from fortran8_gb300 import configs
from fortran8_gb300.solver import Solver


def periodic_box(oracle, n=16):
    w = configs.scaled(configs.c2_3d(), n, n, n)
    return w, Solver(oracle, w.grid, w.phys, ())


def test_spectrum_parseval(oracle):
    w, s = periodic_box(oracle)
    with s:
        s.load(configs.initial_state(w))
        s.step(2)
        e = s.spectrum()
        st = s.store()
    it = (slice(1, -1),) * 3
    k_stag = sum(float(np.sum(st[f][it] ** 2)) for f in ("u", "v", "w")) / 2 / w.grid.cells
    assert abs(e.sum() - k_stag) <= 1e-12 * k_stag


def test_spectrum_single_mode(oracle):
    w, s = periodic_box(oracle)
    st = configs.initial_state(w)
    g = w.grid
    for f in ("u", "v", "w"):
        st.arrays[f][...] = 0.0
    x = (np.arange(1, g.nx + 1)) * (g.lx / g.nx)
    st.arrays["u"][1:-1, 1:-1, 1:-1] = np.cos(3 * 2 * math.pi * x / g.lx)[None, None, :]
    with s:
        s.load(st)
        e = s.spectrum()
    assert np.argmax(e) == 3
    assert abs(e[3] - 0.25) < 1e-12 and abs(e.sum() - 0.25) < 1e-12   # <cos^2>/2


def numpy_turb(st, g, phys, mean=None):
    U, V, W = (st[f][1:-1, 1:-1, 1:-1] - (mean[q] if mean is not None else 0.0)
               for q, f in enumerate(("u", "v", "w")))
    dX, dY, dZ = g.lx / g.nx, g.ly / g.ny, g.lz / g.nz
    sh = lambda a, ax, d: np.roll(a, d, axis=ax)   # a(i - d) along ax (periodic wrap)
    Ur, Vr, Wr = (U + sh(U, 2, 1)) / 2, (V + sh(V, 1, 1)) / 2, (W + sh(W, 0, 1)) / 2
    N = g.cells
    urms, vrms, wrms = (np.sum(a ** 2) / N for a in (Ur, Vr, Wr))
    gu, gv, gw = (U - sh(U, 2, 1)) / dX, (V - sh(V, 1, 1)) / dY, (W - sh(W, 0, 1)) / dZ
    D = np.zeros((3, 3) + U.shape)
    D[0, 0] = gu
    D[0, 1] = (sh(U, 1, -1) - sh(U, 1, 1) + sh(sh(U, 2, 1), 1, -1) - sh(sh(U, 2, 1), 1, 1)) / (4 * dY)
    D[0, 2] = (sh(U, 0, -1) - sh(U, 0, 1) + sh(sh(U, 2, 1), 0, -1) - sh(sh(U, 2, 1), 0, 1)) / (4 * dZ)
    D[1, 0] = (sh(V, 2, -1) - sh(V, 2, 1) + sh(sh(V, 1, 1), 2, -1) - sh(sh(V, 1, 1), 2, 1)) / (4 * dX)
    D[1, 1] = gv
    D[1, 2] = (sh(V, 0, -1) - sh(V, 0, 1) + sh(sh(V, 1, 1), 0, -1) - sh(sh(V, 1, 1), 0, 1)) / (4 * dZ)
    D[2, 0] = (sh(W, 2, -1) - sh(W, 2, 1) + sh(sh(W, 0, 1), 2, -1) - sh(sh(W, 0, 1), 2, 1)) / (4 * dX)
    D[2, 1] = (sh(W, 1, -1) - sh(W, 1, 1) + sh(sh(W, 0, 1), 1, -1) - sh(sh(W, 0, 1), 1, 1)) / (4 * dY)
    D[2, 2] = gw
    S = D + D.transpose(1, 0, 2, 3, 4)
    nu = 1.0 / phys.re
    eps = nu / 2 * np.sum(S ** 2) / N
    all_rms = (urms + vrms + wrms) / 3
    all_grad = (np.sum(gu ** 2) + np.sum(gv ** 2) + np.sum(gw ** 2)) / N / 3
    lam = math.sqrt(all_rms / all_grad)
    return {"k_energy": (urms + vrms + wrms) / 2, "epsilon": eps, "lambda_": lam,
            "re_lambda": math.sqrt(all_rms) * lam / nu, "l_kolmogorov": (nu ** 3 / eps) ** 0.25}


@pytest.mark.parametrize("with_mean", [False, True])
def test_turbulence_matches_restatement(oracle, with_mean):
    w, s = periodic_box(oracle)
    rng = np.random.default_rng(7)
    mean = tuple(0.1 * rng.random(w.grid.interior_shape) for _ in range(3)) if with_mean else None
    with s:
        s.load(configs.initial_state(w))
        s.step(2)
        t = s.turbulence(mean)
        ref = numpy_turb(s.store(), w.grid, w.phys, mean)
    for k, v in ref.items():
        assert abs(getattr(t, k) - v) <= 1e-11 * abs(v), (k, getattr(t, k), v)
    assert t.ep_energy > 0 and t.trc_mean > 2.9
