"""Running statistics of the step loop (fenep_mpi.f90:2934-2941, 3054-3056)
and their post-processing (ave_mean, power_spectrum), on the oracle."""
from __future__ import annotations

import numpy as np

from fortran8_gb300 import configs, stats
from fortran8_gb300.solver import Solver


def test_sums_and_probes_follow_the_stored_states(oracle):
    w = configs.scaled(configs.c3_channel(), 16, 8, 8)
    g = w.grid
    with Solver(oracle, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        s.stats_begin(1, max_steps=4)
        stored = []
        for _ in range(3):
            s.step(1)
            stored.append(s.store())
        sums, probes, n = s.stats_read(max_steps=4)
        assert n == 3 and probes.shape == (3, 3, g.nz)
        it = (slice(1, -1),) * 3
        for q, f in enumerate(("u", "v", "w")):
            np.testing.assert_allclose(sums[q], sum(st[f][it] for st in stored), rtol=1e-14, atol=1e-15)
        i, j = g.nx // 2, g.ny // 2
        for n_, st in enumerate(stored):
            U, V, W = st["u"], st["v"], st["w"]
            np.testing.assert_allclose(probes[0, n_], (U[1:-1, j, i] + U[1:-1, j, i - 1]) / 2, rtol=1e-14)
            np.testing.assert_allclose(probes[1, n_], (V[1:-1, j, i] + V[1:-1, j - 1, i]) / 2, rtol=1e-14)
            np.testing.assert_allclose(probes[2, n_], (W[1:-1, j, i] + W[:-2, j, i]) / 2, rtol=1e-14)
        # second pass: squared fluctuations about the z-averaged time mean
        mean = stats.ave_mean(stats.time_mean(sums, n))
        s.stats_begin(2, mean=mean)
        s.step(2)
        sq, _, n2 = s.stats_read()
        assert n2 == 2 and all(np.all(a >= 0) for a in sq)


def test_power_spectrum_of_a_tone():
    nstep, nz = 64, 4
    t = np.arange(nstep)
    probes = np.zeros((3, nstep, nz))
    probes[0] = np.cos(2 * np.pi * 5 * t / nstep)[:, None]
    ps = stats.power_spectrum(probes)
    assert ps.shape == (3, nstep // 2 + 1)
    assert np.argmax(ps[0]) == 5 and abs(ps[0, 5] - nz * 0.125) < 1e-12   # |1/2|^2 / 2 per k
    assert np.allclose(ps[1:], 0.0)
