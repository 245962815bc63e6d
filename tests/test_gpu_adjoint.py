"""Discrete adjoint of the FP64 step (f8_grad) on the GPU, through the C ABI.

* Against the torch restatement (oracle/f8_torch.py, pinned to the C++ oracle
  and to its own central differences): the gradient of the time-averaged
  total drag with respect to Wi, beta, L^2 and the cylinder centres to 1e-8
  relative, with and without the AB2 start step, channel and periodic box,
  spinning surface-ring cylinders under a moving wall, and beta = 1.
* The vector-Jacobian product of the whole state: seeded adjoints of the final
  state give the adjoint of the initial state and the parameters to 1e-8.
* Checkpointing: every checkpoint interval gives the same gradient, and the
  state f8_grad leaves equals f8_step's bit for bit.
* Central differences of the GPU forward agree with the adjoint: on a
  32 x 16 x 16 channel over 3 steps (h = 1e-4, within 1e-4), and on the
  adjoint workload itself, the 128 x 64 x 64 channel with two cylinders from
  its seeded initial state, over 400 steps with a checkpoint every 20 steps
  (relative steps; see the two workload tests for the tolerances).
"""
from __future__ import annotations

import numpy as np
import pytest

from fortran8_gb300.solver import Solver

from .adjoint_cases import case, param_vector, torch_grad, with_params
from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def gpu_grad(fns, w, st, step0, nsteps, K=0, weights=None, seed=None, want_dstate=False):
    with Solver(fns, w.grid, w.phys, w.cyls) as s:
        s.load(st, step0)
        _, J, dp, ds, drag = s.grad(nsteps, K, weights, seed, want_dstate)
        final = s.store()
    return J, dp, ds, drag, final


def close(a, b, rel):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).max()
    return np.all(np.abs(a - b) <= rel * np.abs(b) + 1e-3 * rel * scale)


@pytest.mark.parametrize("name,spinup", [("channel", 10), ("channel", 0), ("periodic", 10), ("moving", 10), ("arc", 10),
                                         ("newtonian", 10)])
def test_grad_matches_torch(gpu, oracle, name, spinup):
    w, st, step0 = case(name, oracle, spinup=spinup)
    n = 4
    J, dp, _, drag, _ = gpu_grad(gpu, w, st, step0, n, K=2)
    Jt, gt, _, Dt = torch_grad(w, st, step0, n)
    assert rel_l2(drag, Dt) < 1e-11
    assert abs(J - Jt) <= 1e-11 * abs(Jt)
    assert close(dp, gt, 1e-8), (dp, gt)


def test_grad_matches_torch_over_tens_of_steps(gpu, oracle):
    """A horizon of 24 steps (6 checkpoint segments) against the torch gradient."""
    w, st, step0 = case("channel", oracle)
    n = 24
    J, dp, _, drag, _ = gpu_grad(gpu, w, st, step0, n, K=4)
    Jt, gt, _, Dt = torch_grad(w, st, step0, n)
    assert rel_l2(drag, Dt) < 1e-11
    assert abs(J - Jt) <= 1e-11 * abs(Jt)
    assert close(dp, gt, 1e-8), (dp, gt)


def test_state_vjp_matches_torch(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    g = w.grid
    rng = np.random.default_rng(7)
    seed = {n: rng.standard_normal(g.halo_shape) for n in ("u", "v", "w", "p")}
    seed["c"] = rng.standard_normal(g.halo_shape + (6,))
    for n in ("ax0", "ay0", "az0", "tx0", "ty0", "tz0"):
        seed[n] = rng.standard_normal(g.interior_shape)
    seed_state = st.copy()
    for n, a in seed.items():
        seed_state.arrays[n] = np.ascontiguousarray(a)
    for n in ("phi", "fx", "fy", "fz"):
        seed_state.arrays[n] = np.zeros_like(seed_state.arrays[n])
    n = 2
    zero_w = np.zeros((n, len(w.cyls), 3))
    J, dp, ds, _, _ = gpu_grad(gpu, w, st, step0, n, weights=zero_w, seed=seed_state, want_dstate=True)
    Jt, gt, dst, _ = torch_grad(w, st, step0, n, weights=zero_w, seed=seed)
    assert close(dp, gt, 1e-8), (dp, gt)
    for name in ("u", "v", "w", "p", "c", "ax0", "ay0", "az0", "tx0", "ty0", "tz0"):
        assert rel_l2(ds[name], dst[name]) < 1e-9, name


def test_checkpoint_intervals_agree_and_state_advances(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    n = 6
    res = [gpu_grad(gpu, w, st, step0, n, K=K) for K in (1, 4, 0)]
    for J, dp, _, drag, final in res[1:]:
        assert J == res[0][0]
        assert np.array_equal(drag, res[0][3])
        assert close(dp, res[0][1], 1e-12)
    with Solver(gpu, w.grid, w.phys, w.cyls) as s:
        s.load(st, step0)
        _, drag = s.step(n)
        out = s.store()
    for J, dp, _, dg, final in res:
        assert np.array_equal(dg, drag)
        for name in ("u", "v", "w", "p", "c"):
            assert np.array_equal(final[name], out[name]), name


def test_grad_matches_gpu_central_differences(gpu, oracle):
    w, st, step0 = case("channel", oracle)
    n = 3
    J, dp, _, _, _ = gpu_grad(gpu, w, st, step0, n)
    base = param_vector(w)
    h = 1e-4
    for q in range(len(base)):
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
        assert abs(dp[q] - fd) <= 1e-4 * abs(fd) + 1e-8, (q, dp[q], fd)


def _workload_fd(gpu, w, st, n, qs_rel):
    """Central differences of the mean x drag over n steps from st, with the
    relative step h_q = rel * |p_q| for each parameter index q in qs_rel."""
    base = param_vector(w)
    fds = {}
    for q, rel in qs_rel.items():
        h = rel * max(abs(base[q]), 1.0)
        vals = []
        for sgn in (1, -1):
            b = base.copy()
            b[q] += sgn * h
            wq = with_params(w, b)
            with Solver(gpu, wq.grid, wq.phys, wq.cyls) as s:
                s.load(st, 0)
                _, drag = s.step(n)
            vals.append(drag[:, :, 0].sum() / n)
        fds[q] = (vals[0] - vals[1]) / (2 * h)
    return fds


def _adjoint_workload(beta=None):
    from dataclasses import replace
    from fortran8_gb300 import configs
    w = configs.c4_adjoint()
    assert (w.grid.nx, w.grid.ny, w.grid.nz, w.steps) == (128, 64, 64, 400)
    w = replace(w, cyls=tuple(replace(c, xc=c.xc + 0.0123, yc=c.yc + 0.0371) for c in w.cyls))
    if beta is not None:
        w = replace(w, phys=replace(w.phys, beta=beta))
    return w, configs.initial_state(w)


def test_grad_adjoint_workload_matches_central_differences(gpu):
    """The 128 x 64 x 64 channel with 2 cylinders (r = 0.3), Re 300, Wi 3,
    beta 0.85, L^2 400, dt 5e-4, from its seeded initial state (seed 3, C = I):
    the gradient of the drag averaged over 400 steps, with a checkpoint every
    20 steps, against FP64 central differences (14 perturbed forward runs).

    The steps are relative, because the parameters differ in scale by 10^3
    (beta 0.85, L^2 400): h = 1e-4 |p| for Wi, beta and L^2, within 1e-4 (plus
    1e-10 absolute for L^2, whose sensitivity of ~6e-8 moves the differenced
    drag by ~1e-10 of J).  The centre differences need h = 1e-5 |p|: the Roma
    kernel is only C^1, and at h = 1e-4 their own truncation error is ~1e-3
    (the Newtonian test below shows it vanishing as h decreases).  At that
    step the perturbed runs of this 400-step FENE-P flow also differ in some
    SPD face-candidate choices (a discontinuous function of C whose derivative
    the adjoint takes as zero), which moves the differences by ~2e-4, so the
    centres are held to 1e-3 here and to 1e-4 in the Newtonian test.
    The centres are moved off the grid lines by a fraction of a cell so that no
    marker sits on a break point of the Roma kernel."""
    w, st = _adjoint_workload()
    n, K = w.steps, 20
    J, dp, _, _, _ = gpu_grad(gpu, w, st, 0, n, K=K)
    fds = _workload_fd(gpu, w, st, n, {0: 1e-4, 1: 1e-4, 2: 1e-4, 3: 1e-5, 4: 1e-5, 5: 1e-5, 6: 1e-5})
    print("adjoint", list(dp), "central differences", fds)
    for q, fd in fds.items():
        tol = 1e-4 if q < 3 else 1e-3
        assert abs(dp[q] - fd) <= tol * abs(fd) + 1e-10, (q, dp[q], fd)


def test_grad_newtonian_adjoint_workload_matches_central_differences(gpu):
    """The same workload with beta = 1 (no polymer stage, hence no candidate
    choice): the centre gradients over 400 steps within 1e-4 of central
    differences with h = 1e-5 |centre|.  beta is not differenced here: at
    beta = 1 the step zeroes C and skips the polymer stage (fenep.f90:2479-2485),
    while any beta != 1 runs it, so J is not differentiable in beta there."""
    w, st = _adjoint_workload(beta=1.0)
    n, K = w.steps, 20
    J, dp, _, _, _ = gpu_grad(gpu, w, st, 0, n, K=K)
    fds = _workload_fd(gpu, w, st, n, {3: 1e-5, 4: 1e-5, 5: 1e-5, 6: 1e-5})
    print("adjoint", list(dp), "central differences", fds)
    for q, fd in fds.items():
        assert abs(dp[q] - fd) <= 1e-4 * abs(fd), (q, dp[q], fd)


def test_autograd_function_returns_the_adjoint_gradient(gpu, oracle):
    import torch
    from fortran8_gb300.autograd import DragProblem, drag_objective
    w, st, step0 = case("channel", oracle)
    n = 3
    prob = DragProblem(w.grid, w.phys, w.cyls, st, n, step0=step0, checkpoint_every=2)
    p = prob.params().requires_grad_(True)
    J = drag_objective(p, prob)
    loss = (J - 1.0) ** 2
    loss.backward()
    Jg, dp, _, _, _ = gpu_grad(gpu, w, st, step0, n, K=2)
    assert J.item() == Jg
    assert np.allclose(p.grad.numpy(), 2.0 * (Jg - 1.0) * dp, rtol=1e-12, atol=0.0)
