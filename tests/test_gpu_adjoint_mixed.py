"""Discrete adjoint of the FP32-mixed step (f8_grad on an F8_MIXED context).

The mixed step computes the FP64 step's discrete operator in other
arithmetic, so its adjoint is checked against the FP64 adjoint (itself pinned
to the torch gradient oracle and to central differences in
tests/test_gpu_adjoint.py) and against central differences of the FP64
forward.

Each adjoint is the exact transpose of its own forward with that forward's
SPD face-candidate choices held fixed (fenep.f90:220-230).  Where C is smooth
the three candidates nearly coincide, and the FP32 and FP64 eigen tests break
those near-ties differently (in most cells of the strongly stretched small
cases below); the forwards hardly notice (the face values agree to O(dx^2)),
but the two linearisations differ.  The small stretched cases are therefore
compared at 1e-3 (parameters) and 5e-3 (state adjoints); the adjoint workload
itself, the 128 x 64 x 64 channel over 400 steps from C = I, at 1e-4:

* dJ/d(Wi, beta, L^2, centres) of the time-averaged drag against the FP64
  adjoint, per parameter, with and without the AB2 start step, on the channel
  and the periodic box, and at full size on the adjoint workload;
* the adjoint of the whole initial state (seeded final-state adjoints);
* checkpoint intervals agree, with the tapes of the earlier segments kept
  from the first forward pass or recomputed, and the state f8_grad leaves
  equals f8_step's bit for bit;
* central differences of the FP64 forward (relative step 1e-4).
"""
from __future__ import annotations

import numpy as np
import pytest

from fortran8_gb300 import abi
from fortran8_gb300.solver import Solver

from .adjoint_cases import case, param_vector, with_params
from .conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4           # adjoint workload, and the Newtonian case (no candidate choice)
TOL_SMALL = 1e-3     # small stretched cases: near-tie candidate choices differ
TOL_STATE = 5e-3


def grad(fns, w, st, step0, n, precision, K=0, weights=None, seed=None, want_dstate=False):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(st, step0)
        status, J, dp, ds, drag = s.grad(n, K, weights, seed, want_dstate)
        final = s.store()
    assert status == abi.F8_OK, status
    return J, dp, ds, drag, final


def assert_params_close(dm, d64, tol):
    for q, (a, b) in enumerate(zip(dm, d64)):
        assert abs(a - b) <= tol * abs(b) + 1e-12, (q, a, b, list(dm), list(d64))


@pytest.mark.parametrize("name,spinup", [("channel", 10), ("channel", 0), ("periodic", 10), ("newtonian", 10)])
def test_mixed_grad_matches_fp64_adjoint(gpu, oracle, name, spinup):
    w, st, step0 = case(name, oracle, spinup=spinup)
    n = 6
    Jm, dm, _, dragm, _ = grad(gpu, w, st, step0, n, abi.F8_MIXED, K=3)
    J6, d6, _, drag6, _ = grad(gpu, w, st, step0, n, abi.F8_FP64, K=3)
    assert abs(Jm - J6) <= 1e-5 * abs(J6)
    assert_params_close(dm, d6, TOL if name == "newtonian" else TOL_SMALL)


def test_mixed_grad_matches_fp64_adjoint_on_the_adjoint_workload(gpu):
    """The 128 x 64 x 64 channel with two cylinders from its seeded initial
    state, 400 steps with a checkpoint every 20: every parameter within 1e-4
    of the FP64 adjoint."""
    from dataclasses import replace
    from fortran8_gb300 import configs
    w = configs.c4_adjoint()
    w = replace(w, cyls=tuple(replace(c, xc=c.xc + 0.0123, yc=c.yc + 0.0371) for c in w.cyls))
    st = configs.initial_state(w)
    Jm, dm, _, _, _ = grad(gpu, w, st, 0, w.steps, abi.F8_MIXED, K=20)
    J6, d6, _, _, _ = grad(gpu, w, st, 0, w.steps, abi.F8_FP64, K=20)
    print("mixed", list(dm), "fp64", list(d6))
    assert abs(Jm - J6) <= 1e-6 * abs(J6)
    assert_params_close(dm, d6, TOL)


def test_mixed_state_vjp_matches_fp64(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    g = w.grid
    rng = np.random.default_rng(7)
    seed = st.copy()
    for n in ("u", "v", "w", "p"):
        seed.arrays[n] = rng.standard_normal(g.halo_shape)
    seed.arrays["c"] = rng.standard_normal(g.halo_shape + (6,))
    for n in ("ax0", "ay0", "az0", "tx0", "ty0", "tz0"):
        seed.arrays[n] = rng.standard_normal(g.interior_shape)
    for n in ("phi", "fx", "fy", "fz"):
        seed.arrays[n] = np.zeros_like(seed.arrays[n])
    n = 3
    zero_w = np.zeros((n, len(w.cyls), 3))
    _, dm, dsm, _, _ = grad(gpu, w, st, step0, n, abi.F8_MIXED, weights=zero_w, seed=seed, want_dstate=True)
    _, d6, ds6, _, _ = grad(gpu, w, st, step0, n, abi.F8_FP64, weights=zero_w, seed=seed, want_dstate=True)
    assert_params_close(dm, d6, TOL_SMALL)
    errs = {name: rel_l2(dsm[name], ds6[name]) for name in ("u", "v", "w", "p", "c", "ax0", "ay0", "az0", "tx0",
                                                             "ty0", "tz0")}
    assert max(errs.values()) < TOL_STATE, errs


def test_mixed_checkpoints_agree_and_state_advances(gpu, oracle, monkeypatch):
    w, st, step0 = case("channel", oracle)
    n = 6
    # the first forward pass keeps the tape of every segment that fits in
    # memory (here all of them); F8_GRAD_KEEP_TAPE=0 keeps the last one only,
    # so that the others are recomputed from their checkpoints
    res = [grad(gpu, w, st, step0, n, abi.F8_MIXED, K=K) for K in (1, 4, 0)]
    monkeypatch.setenv("F8_GRAD_KEEP_TAPE", "0")
    res += [grad(gpu, w, st, step0, n, abi.F8_MIXED, K=K) for K in (1, 4)]
    monkeypatch.delenv("F8_GRAD_KEEP_TAPE")
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(st, step0)
        _, drag = s.step(n)
        out = s.store()
    for J, dp, _, dg, final in res:
        assert np.array_equal(dg, drag)
        for name in ("u", "v", "w", "p", "c"):
            assert np.array_equal(final[name], out[name]), name
        assert_params_close(dp, res[0][1], 1e-4)


def test_mixed_grad_matches_fp64_central_differences(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    n = 4
    _, dm, _, _, _ = grad(gpu, w, st, step0, n, abi.F8_MIXED)
    base = param_vector(w)
    for q in range(len(base)):
        h = 1e-4 * max(abs(base[q]), 1.0)
        vals = []
        for sgn in (1, -1):
            b = base.copy()
            b[q] += sgn * h
            wq = with_params(w, b)
            with Solver(gpu, wq.grid, wq.phys, wq.cyls) as s:
                s.load(st, step0)
                _, drag = s.step(n)
            vals.append(drag[:, :, 0].sum() / n)
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(dm[q] - fd) <= TOL_SMALL * abs(fd) + 1e-10, (q, dm[q], fd)
