"""The reference's analytic validation of the wall-bounded step (koide_theory).

The reference checks its 2D wall-bounded solver (fenep_2d.f90, method 3) on a
Poiseuille channel driven by Fx = 1 between walls at NY/4 and 3 NY/4 of its
2 pi box against Koide's analytic FENE-P profile, and reports the RMSE of U over
the channel (koide_theory, fenep_2d.f90:1385-1437).  The same channel here is
the 2D wall grid NX x NX/2 of 2 pi x pi (walls at the domain boundary, so row j
of this grid is row NY/4 + j of the reference's).
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .solver import GridSpec, PhysSpec, State, empty_state

PI = math.pi


def koide_profile(nx: int, beta: float, wi: float, lp: float, re: float = 1.0, fx: float = 1.0) -> np.ndarray:
    """u_theory at the NX/2 cell centres of the channel (koide_theory,
    fenep_2d.f90:1393-1422): the Newtonian parabola plus the FENE-P
    correction in Cardano form, in the reference's scaling (half-height pi/2)."""
    dy = 2 * PI / nx
    a = lp ** 2 / (6.0 * beta * wi ** 2)
    re_t = re * (PI / 2.0)
    b = -lp ** 2 * fx * re_t / (4.0 * beta * wi ** 2)

    def parts(y):
        root = math.sqrt(b ** 2 * y ** 2 + a ** 3)
        fp = (b * y + root) ** (1.0 / 3.0)
        t = b * y - root
        fn = math.copysign(abs(t) ** (1.0 / 3.0), t)
        return fp, fn, 3 * b * y + root, 3 * b * y - root

    fp0, fn0, gp0, gn0 = parts(-1.0)
    out = np.empty(nx // 2)
    for jj in range(nx // 2):
        y = ((jj + 0.5) * dy - PI / 2.0) / (PI / 2.0)
        fp, fn, gp, gn = parts(y)
        u = re_t / (2.0 * beta) * fx * (1.0 - y ** 2) - (1.0 - beta) / beta * 3.0 / (8.0 * b) * (
            fp * gn - fp0 * gn0 + fn * gp - fn0 * gp0)
        out[jj] = u * (PI / 2.0)
    return out


def koide_case(nx: int, beta: float, wi: float, lp: float = 55.0, re: float = 1.0, dt: float = 0.005,
               nz: int = 0):
    """(grid, phys, initial state) of the validation channel: U = V = 0, C = I,
    Fx = 1 (flow_type 2, fenep_2d.f90:86-90).  nz = 0: the 2D channel with the
    2D Newton parameters of fenep_2d.f90:291-293; nz > 0: the same channel
    extruded over nz cells in z (periodic), a 3D grid whose steady Newtonian
    flow is the 2D one."""
    if nz:
        g = GridSpec(3, nx, nx // 2, nz, 2 * PI, PI, nz * 2 * PI / nx, abi.F8_BC_WALLS, 0.0)
        ph = PhysSpec(re=re, wi=wi, beta=beta, lp2=lp * lp, dt=dt)
    else:
        g = GridSpec(2, nx, nx // 2, 1, 2 * PI, PI, 2 * PI / nx, abi.F8_BC_WALLS, 0.0)
        ph = PhysSpec(re=re, wi=wi, beta=beta, lp2=lp * lp, dt=dt, newton_dc=1.0e-10, newton_eps=1.0e-10)
    st = empty_state(g)
    c = st.arrays["c"]
    c[..., 0] = 1.0
    c[..., 3 if nz else 2] = 1.0
    if nz:
        c[..., 5] = 1.0
    st.arrays["fx"][:] = 1.0
    return g, ph, st


def koide_rmse(state: State, nx: int, beta: float, wi: float, lp: float = 55.0, re: float = 1.0) -> float:
    """RMSE of U against the analytic profile over the channel cells, as
    koide_theory sums it (fenep_2d.f90:1426-1432); for a 3D grid over every
    z plane."""
    u = state["u"][1:-1, 1:-1, 1:-1]
    ut = koide_profile(nx, beta, wi, lp, re)
    return math.sqrt(float(((u - ut[None, :, None]) ** 2).sum()) / u.size)


def run_to_steady(solver, nx: int, beta: float, wi: float, lp: float = 55.0, chunk: int = 2000,
                  max_steps: int = 200000, rtol: float = 1e-12):
    """Advance a loaded solver until the RMSE changes by less than rtol between
    chunks; returns (rmse, steps)."""
    prev, steps = None, 0
    while steps < max_steps:
        solver.step(chunk, want_drag=False)
        steps += chunk
        r = koide_rmse(solver.store(), nx, beta, wi, lp)
        if prev is not None and abs(r - prev) <= rtol * r:
            return r, steps
        prev = r
    return prev, steps
