"""torch.autograd front end of the discrete adjoint (f8_grad).

``drag_objective(params, problem)`` returns the drag objective of ``problem``
(by default the time-averaged total drag over ``nsteps`` FP64 GPU steps from
``problem.state``) as a differentiable function of

    params = (Wi, beta, L^2, xc_0, yc_0, xc_1, yc_1, ...)

(the cylinder centres move their markers).  Its forward runs one f8_grad
call, which advances the step, stores the checkpoints and runs the adjoint
sweep, so the gradient is ready when ``backward`` asks for it: backward only
scales the stored gradient by the incoming one.  The computation runs in the
CUDA library; there is no CPU path.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np
import torch

from . import abi, lib
from .solver import Solver, State


@dataclass
class DragProblem:
    """A fixed initial state and the objective's definition; params vary."""
    grid: object                 # solver.GridSpec (3D)
    phys: object                 # solver.PhysSpec; wi, beta, lp2 are replaced by params
    cyls: tuple                  # solver.CylSpec; xc, yc are replaced by params
    state: State
    nsteps: int
    step0: int = 0
    checkpoint_every: int = 0
    weights: object = None       # (nsteps, ncyl, 3) drag weights; None: time-averaged total x drag

    def params(self) -> torch.Tensor:
        v = [self.phys.wi, self.phys.beta, self.phys.lp2]
        for c in self.cyls:
            v += [c.xc, c.yc]
        return torch.tensor(v, dtype=torch.float64)

    def evaluate(self, vec: np.ndarray):
        """(J, dJ/dparams) at params = vec, from the CUDA library."""
        ph = replace(self.phys, wi=float(vec[0]), beta=float(vec[1]), lp2=float(vec[2]))
        cyls = tuple(replace(c, xc=float(vec[3 + 2 * l]), yc=float(vec[4 + 2 * l]))
                     for l, c in enumerate(self.cyls))
        with Solver(lib.functions(), self.grid, ph, cyls, precision=abi.F8_FP64,
                    poisson=abi.F8_POISSON_FFT) as s:
            s.load(self.state, self.step0)
            _, J, dp, _, _ = s.grad(self.nsteps, self.checkpoint_every, self.weights)
        return J, dp


class _DragObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, problem):
        J, dp = problem.evaluate(params.detach().cpu().numpy().astype(np.float64))
        ctx.save_for_backward(torch.as_tensor(dp, dtype=params.dtype, device=params.device))
        return torch.tensor(J, dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        (dp,) = ctx.saved_tensors
        return grad_out * dp, None


def drag_objective(params: torch.Tensor, problem: DragProblem) -> torch.Tensor:
    """Differentiable drag objective J(params) of ``problem`` (see module docstring)."""
    return _DragObjective.apply(params, problem)
