"""The differentiable torch restatement (oracle/f8_torch.py), the gradient
reference of the discrete adjoint, is pinned here on the CPU:

* its forward against the C++ oracle on identical seeded inputs (relative L2
  <= 1e-12 on U, V, P, drag; <= 1e-10 on W and C: the Newton iterates agree to
  the solver's round-off, C - I and W are small);
* its autograd gradient against central differences of its own forward
  (h = 1e-4 absolute, the step size BASELINE's check names) to 1e-5 relative.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from fortran8_gb300.solver import Solver

from .adjoint_cases import case, params_of, param_vector, torch_grad, with_params
from .conftest import interior, rel_l2

import f8_torch as ft  # noqa: E402  (path set by adjoint_cases)


@pytest.mark.parametrize("name", ["channel", "periodic", "moving", "newtonian", "arc"])
def test_forward_matches_oracle(oracle, name):
    w, st, step0 = case(name, oracle, spinup=0)
    n = 3
    with Solver(oracle, w.grid, w.phys, w.cyls) as o:
        o.load(st)
        _, drag = o.step(n)
        out = o.store()
    J, D, s = ft.run(st.arrays, w.grid, w.phys, w.cyls, params_of(w), n, first_step=True)
    I = interior
    assert rel_l2(I(s["U"].detach().numpy()), I(out["u"])) < 1e-12
    assert rel_l2(I(s["V"].detach().numpy()), I(out["v"])) < 1e-12
    assert rel_l2(I(s["W"].detach().numpy()), I(out["w"])) < 1e-10
    assert rel_l2(I(s["P"].detach().numpy()), I(out["p"])) < 1e-12
    assert rel_l2(I(np.moveaxis(s["C"].detach().numpy(), 0, -1)), I(out["c"])) < 1e-10
    assert rel_l2(D.detach().numpy(), drag) < 1e-12


def test_gradient_matches_central_differences(oracle):
    w, st, step0 = case("channel", oracle, spinup=10)
    n = 3
    J, g, _, _ = torch_grad(w, st, step0, n)
    base = param_vector(w)
    h = 1e-4
    for q in range(len(base)):
        vals = []
        for sgn in (1, -1):
            b = base.copy()
            b[q] += sgn * h
            wq = with_params(w, b)
            with torch.no_grad():
                Jq, _, _ = ft.run(st.arrays, wq.grid, wq.phys, wq.cyls, params_of(wq), n, first_step=step0 == 0)
            vals.append(Jq.item())
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(g[q] - fd) <= 1e-5 * abs(fd) + 1e-7, (q, g[q], fd)
