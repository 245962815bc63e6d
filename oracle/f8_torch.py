"""FP64 PyTorch restatement of the 3D SMAC + FENE-P + IBM step (gradient oracle).

TEST INFRASTRUCTURE ONLY.  This module is the reference for the gradients of
the discrete adjoint (``f8_grad``): the whole 3D step is written with plain
differentiable torch operations, so ``torch.autograd`` gives the exact
derivative of the same discretisation.  Only ``tests/`` import it.  Its forward
is pinned against the C++ oracle (``oracle/f8_oracle.cpp``, itself pinned by
the reference's known-answer programs) to round-off.

The step follows machapin/fortran8 as the oracle restates it:

* halo fill: PBM (fenep.f90:147-166) and the wall rules of
  fenep_2d.f90:1098-1143 (x, then y, then z); with walls the polymer update
  also covers the ghost rows (zero C and velocity beyond them), which keep
  their updated values through the stress and are extrapolated at the end of
  the step, as the reference's wall mode does;
* polymer: candidate faces and the Vieta eigen test (fenep.f90:169-242,
  425-444), Cstar (464-507), the Lyapunov Newton solve with its central
  difference Jacobian (518-643), stress divergence (645-691);
* convection and viscous terms (694-770), the AB2 predictor with the IBM
  explicit velocity (1430-1474, 1970-2037), direct forcing with the Roma
  kernel (fenep_mpi.f90:1794-1929, fenep.f90:2039-2055, fold 2195-2205);
* Helmholtz and Poisson solves: FFT (fenep.f90:1400-1428, 1529-1560) or FFT in
  x, z with the tridiagonal wall systems in y (fenep_2d.f90:1179-1342);
* projection and pressure update (fenep.f90:1562-1604).

Differentiation conventions (the same as the CUDA adjoint's):

* the SPD candidate choice is a discrete decision, evaluated on detached
  values, so the derivative flows through the chosen candidate only;
* the Newton solution C* of G(C) = A C + C A^T - b = 0 is differentiated by
  the implicit-function theorem: the value is the Newton iterate, the
  derivative that of C* - J^-1 G(C*) with the exact Jacobian J held fixed;
* |u| has derivative sign(u) (0 at 0).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

F64 = torch.float64
PI = 3.141592653589793238462643383279502884
E6 = (1.0, 0.0, 0.0, 1.0, 0.0, 1.0)


@dataclass
class TGrid:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    walls: bool
    uwall: float = 0.0

    @classmethod
    def from_spec(cls, g) -> "TGrid":
        """From fortran8_gb300.solver.GridSpec (3D)."""
        assert g.dim == 3
        return cls(g.nx, g.ny, g.nz, g.lx / g.nx, g.ly / g.ny, g.lz / g.nz, g.bc_y == 1, g.uwall)


# ---------------------------------------------------------------------------
# halo fill (functional)

def bc(A: torch.Tensor, kind: str, g: TGrid) -> torch.Tensor:
    """Boundary values of a halo field (..., NZ+2, NY+2, NX+2) from its interior.

    kind: 'u', 'v', 'w', 'p' or 'c' (conformation tensor extrapolation).
    """
    NX, NY, NZ = g.nx, g.ny, g.nz
    A = torch.cat([A[..., NX:NX + 1], A[..., 1:NX + 1], A[..., 1:2]], dim=-1)
    if not g.walls:
        A = torch.cat([A[..., NY:NY + 1, :], A[..., 1:NY + 1, :], A[..., 1:2, :]], dim=-2)
    else:
        r1, rn = A[..., 1:2, :], A[..., NY:NY + 1, :]
        mid = A[..., 1:NY + 1, :]
        if kind == "u":
            lo, hi = -r1, 2 * g.uwall - rn
        elif kind == "w":
            lo, hi = -r1, -rn
        elif kind == "v":
            z = torch.zeros_like(r1)
            lo, hi = z, z
            mid = torch.cat([A[..., 1:NY, :], z], dim=-2)
        elif kind == "p":
            lo, hi = r1, rn
        else:
            lo = 2 * r1 - A[..., 2:3, :]
            hi = 2 * rn - A[..., NY - 1:NY, :]
        A = torch.cat([lo, mid, hi], dim=-2)
    A = torch.cat([A[..., NZ:NZ + 1, :, :], A[..., 1:NZ + 1, :, :], A[..., 1:2, :, :]], dim=-3)
    return A


def bc_xz(A: torch.Tensor, g: TGrid) -> torch.Tensor:
    """Periodic x and z halo copies only (every y row, ghost rows included)."""
    NX, NZ = g.nx, g.nz
    A = torch.cat([A[..., NX:NX + 1], A[..., 1:NX + 1], A[..., 1:2]], dim=-1)
    return torch.cat([A[..., NZ:NZ + 1, :, :], A[..., 1:NZ + 1, :, :], A[..., 1:2, :, :]], dim=-3)


def sh(A: torch.Tensor, g: TGrid, di=0, dj=0, dk=0) -> torch.Tensor:
    """Values at (i+di, j+dj, k+dk) for every interior cell (i, j, k)."""
    return A[..., 1 + dk:1 + dk + g.nz, 1 + dj:1 + dj + g.ny, 1 + di:1 + di + g.nx]


def embed(I: torch.Tensor, g: TGrid) -> torch.Tensor:
    """Interior field -> halo field with zero halo (to be filled by bc)."""
    return torch.nn.functional.pad(I, (1, 1, 1, 1, 1, 1))


# ---------------------------------------------------------------------------
# polymer

def vieta(a):
    a0, a1, a2, a3, a4, a5 = a
    A2 = -(a0 + a3 + a5)
    A1 = a0 * a3 + a3 * a5 + a5 * a0 - a4 * a4 - a2 * a2 - a1 * a1
    A0 = -(a0 * a3 * a5 + a1 * a4 * a2 + a1 * a4 * a2 - a0 * a4 * a4 - a1 * a1 * a5 - a2 * a3 * a2)
    p = A1 - (A2 * A2) / 3.0
    q = A0 - A1 * A2 / 3.0 + 2.0 * (A2 * A2 * A2) / 27.0
    qh, p3 = q / 2.0, p / 3.0
    t = qh * qh + p3 * p3 * p3
    two_pi_3 = 2.0 * PI / 3.0
    val = 2.0 * torch.sqrt(-p / 3.0) * torch.cos(torch.acos(3.0 * q / (2.0 * p) * torch.sqrt(-3.0 / p)) / 3.0
                                                  + two_pi_3) - A2 / 3.0
    return torch.where(t >= 0.0, torch.full_like(val, -100.0), val)


def face_p(idx, cm, c0, cp):
    return torch.where(idx == 0, c0 * 3 / 2 - cp / 2,
                       torch.where(idx == 1, cm / 2 + c0 / 2,
                                   torch.where(idx == 2, cm / 4 + c0 - cp / 4, c0)))


def face_n(idx, cm, c0, cp):
    return torch.where(idx == 0, c0 / 2 + cp / 2,
                       torch.where(idx == 1, -cm / 2 + c0 * 3 / 2,
                                   torch.where(idx == 2, -cm / 4 + c0 + cp / 4, c0)))


def select(cm, c0, cp):
    """Chosen candidate (0..2) or 3 for the cell value, per cell (detached)."""
    with torch.no_grad():
        mins = []
        for l in range(3):
            li = torch.full(c0[0].shape, l, dtype=torch.long)
            pt = [face_p(li, cm[m], c0[m], cp[m]) for m in range(6)]
            nt = [face_n(li, cm[m], c0[m], cp[m]) for m in range(6)]
            mins.append(torch.fmin(vieta(pt), vieta(nt)))
        mins.append(torch.zeros_like(mins[0]))
        st = torch.stack(mins, 0)
        st = torch.where(torch.isnan(st), torch.full_like(st, -math.inf), st)
        return torch.argmax(st, dim=0)


def lyap(AT, b, x, lp2, dt, wi):
    """l = A X + X A^T - b with A = AT + (1 + f(X) dt/Wi)/2 I (fenep.f90:588-605)."""
    fx = (lp2 - 3) / (lp2 - x[0] - x[3] - x[5])
    dd = (1.0 + fx * dt / wi) / 2.0
    A = [[AT[r][q] for q in range(3)] for r in range(3)]
    for r in range(3):
        A[r][r] = A[r][r] + dd
    l0 = (A[0][0] + A[0][0]) * x[0] + A[0][1] * x[1] + A[0][2] * x[2] + A[0][1] * x[1] + A[0][2] * x[2] - b[0]
    l1 = A[1][0] * x[0] + (A[1][1] + A[0][0]) * x[1] + A[1][2] * x[2] + A[0][1] * x[3] + A[0][2] * x[4] - b[1]
    l2 = A[2][0] * x[0] + A[2][1] * x[1] + (A[2][2] + A[0][0]) * x[2] + A[0][1] * x[4] + A[0][2] * x[5] - b[2]
    l3 = A[1][0] * x[1] + A[1][0] * x[1] + (A[1][1] + A[1][1]) * x[3] + A[1][2] * x[4] + A[1][2] * x[4] - b[3]
    l4 = A[1][0] * x[2] + A[2][0] * x[1] + A[2][1] * x[3] + (A[2][2] + A[1][1]) * x[4] + A[1][2] * x[5] - b[4]
    l5 = A[2][0] * x[2] + A[2][1] * x[4] + A[2][0] * x[2] + A[2][1] * x[4] + (A[2][2] + A[2][2]) * x[5] - b[5]
    return [l0, l1, l2, l3, l4, l5]


def newton(AT, b, x0, lp2, dt, wi, dc, eps, itrmax):
    """Newton of fenep.f90:518-585 on detached values, every cell at once:
    central-difference Jacobian, solve, stop at |r|/|x| < eps per cell."""
    with torch.no_grad():
        x = torch.stack(x0, 0).clone()          # (6, N)
        n = x.shape[1]
        active = torch.ones(n, dtype=torch.bool)
        iters = torch.zeros(n, dtype=torch.long)
        for _ in range(itrmax):
            idx = torch.nonzero(active).flatten()
            if idx.numel() == 0:
                break
            xa = x[:, idx]
            ATa = [[AT[r][q][idx] for q in range(3)] for r in range(3)]
            ba = [bb[idx] for bb in b]
            J = torch.empty(idx.numel(), 6, 6, dtype=F64)
            for col in range(6):
                x1 = xa.clone(); x2 = xa.clone()
                x1[col] = x1[col] + dc
                x2[col] = x2[col] - dc
                l1 = lyap(ATa, ba, list(x1), lp2, dt, wi)
                l2 = lyap(ATa, ba, list(x2), lp2, dt, wi)
                for row in range(6):
                    J[:, row, col] = (l1[row] - l2[row]) / (2.0 * dc)
            l = torch.stack(lyap(ATa, ba, list(xa), lp2, dt, wi), 1)
            r = torch.linalg.solve(J, l.unsqueeze(-1)).squeeze(-1).T   # (6, na)
            xa = xa - r
            x[:, idx] = xa
            iters[idx] += 1
            sr = r[0] * r[0]
            sx = xa[0] * xa[0]
            for m in range(1, 6):
                sr = sr + r[m] * r[m]
                sx = sx + xa[m] * xa[m]
            done = torch.sqrt(sr / sx) < eps
            active[idx[done]] = False
        return x, iters


def _num(x) -> float:
    return float(x.detach()) if torch.is_tensor(x) else float(x)


def polymer(C, U, V, W, g: TGrid, dt, wi, lp2, dc, eps, itrmax):
    """C^{n+1} of the updated cells (list of 6) from C^n (halo, (6, ...)) and the
    velocity.  Periodic: the interior cells.  With walls also the ghost rows
    (rows 0..NY+1, shape (NZ, NY+2, NX)): the reference's wall mode updates C on
    every row of its box, the rows beyond the walls holding zero C and velocity
    (fenep_2d.f90:138-348, 1097-1143, 1912-1929)."""
    if g.walls:
        pad = lambda A: torch.nn.functional.pad(A, (0, 0, 1, 1, 0, 0))
        C, U, V, W = pad(C), pad(U), pad(V), pad(W)
        g = TGrid(g.nx, g.ny + 2, g.nz, g.dx, g.dy, g.dz, True, g.uwall)
    dX, dY, dZ = g.dx, g.dy, g.dz
    c0 = [sh(C[m], g) for m in range(6)]
    faces = []
    for d, (di, dj, dk) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
        cm = [sh(C[m], g, -di, -dj, -dk) for m in range(6)]
        cp = [sh(C[m], g, di, dj, dk) for m in range(6)]
        idx = select(cm, c0, cp)
        fp = [face_p(idx, cm[m], c0[m], cp[m]) for m in range(6)]
        fn = [face_n(idx, cm[m], c0[m], cp[m]) for m in range(6)]
        faces.append((fp, fn))
    (fpx, fnx), (fpy, fny), (fpz, fnz) = faces
    pxm, nxp = fpx, fnx
    pxp = [torch.roll(f, -1, -1) for f in fpx]
    nxm = [torch.roll(f, 1, -1) for f in fnx]
    pzm, nzp = fpz, fnz
    pzp = [torch.roll(f, -1, -3) for f in fpz]
    nzm = [torch.roll(f, 1, -3) for f in fnz]
    pym, nyp = fpy, fny
    if not g.walls:
        pyp = [torch.roll(f, -1, -2) for f in fpy]
        nym = [torch.roll(f, 1, -2) for f in fny]
    else:
        # faces of the cells beyond the ghost rows: multiplied by exactly zero
        # (the wall-normal velocity vanishes there)
        zrow = torch.zeros_like(fpy[0][:, :1, :])
        pyp = [torch.cat([fpy[m][:, 1:, :], zrow], dim=-2) for m in range(6)]
        nym = [torch.cat([zrow, fny[m][:, :-1, :]], dim=-2) for m in range(6)]
    u1, u2 = sh(U, g, -1), sh(U, g)
    v1, v2 = sh(V, g, 0, -1), sh(V, g)
    w1, w2 = sh(W, g, 0, 0, -1), sh(W, g)
    s1 = (-u2 + torch.abs(u2)) * dt / (2 * dX)
    s2 = 1.0 / 6 + (-u2 - torch.abs(u2)) * dt / (2 * dX)
    s3 = 1.0 / 6 + (u1 - torch.abs(u1)) * dt / (2 * dX)
    s4 = (u1 + torch.abs(u1)) * dt / (2 * dX)
    s5 = (-v2 + torch.abs(v2)) * dt / (2 * dY)
    s6 = 1.0 / 6 + (-v2 - torch.abs(v2)) * dt / (2 * dY)
    s7 = 1.0 / 6 + (v1 - torch.abs(v1)) * dt / (2 * dY)
    s8 = (v1 + torch.abs(v1)) * dt / (2 * dY)
    s9 = (-w2 + torch.abs(w2)) * dt / (2 * dZ)
    s10 = 1.0 / 6 + (-w2 - torch.abs(w2)) * dt / (2 * dZ)
    s11 = 1.0 / 6 + (w1 - torch.abs(w1)) * dt / (2 * dZ)
    s12 = (w1 + torch.abs(w1)) * dt / (2 * dZ)
    b = [s3 * pxm[m] + s1 * pxp[m] + s4 * nxm[m] + s2 * nxp[m] + s7 * pym[m] + s5 * pyp[m] + s8 * nym[m]
         + s6 * nyp[m] + s11 * pzm[m] + s9 * pzp[m] + s12 * nzm[m] + s10 * nzp[m] for m in range(6)]
    b[0] = b[0] + dt / wi
    b[3] = b[3] + dt / wi
    b[5] = b[5] + dt / wi

    def u(a, bb, cc):
        return sh(U, g, a, bb, cc)

    def v(a, bb, cc):
        return sh(V, g, a, bb, cc)

    def w(a, bb, cc):
        return sh(W, g, a, bb, cc)
    A0 = [[None] * 3 for _ in range(3)]
    A0[0][0] = -dt * (-u(-1, 0, 0) + u(0, 0, 0)) / dX
    A0[0][1] = -dt * (-v(-1, -1, 0) + v(1, -1, 0) - v(-1, 0, 0) + v(1, 0, 0)) / (4 * dX)
    A0[0][2] = -dt * (-w(-1, 0, -1) + w(1, 0, -1) - w(-1, 0, 0) + w(1, 0, 0)) / (4 * dX)
    A0[1][0] = -dt * (-u(-1, -1, 0) - u(0, -1, 0) + u(-1, 1, 0) + u(0, 1, 0)) / (4 * dY)
    A0[1][1] = -dt * (-v(0, -1, 0) + v(0, 0, 0)) / dY
    A0[1][2] = -dt * (-w(0, -1, -1) + w(0, 1, -1) - w(0, -1, 0) + w(0, 1, 0)) / (4 * dY)
    A0[2][0] = -dt * (-u(-1, 0, -1) - u(0, 0, -1) + u(-1, 0, 1) + u(0, 0, 1)) / (4 * dZ)
    A0[2][1] = -dt * (-v(0, -1, -1) - v(0, 0, -1) + v(0, -1, 1) + v(0, 0, 1)) / (4 * dZ)
    A0[2][2] = -dt * (-w(0, 0, -1) + w(0, 0, 0)) / dZ
    AT = [[A0[q][r].reshape(-1) for q in range(3)] for r in range(3)]
    bf = [bb.reshape(-1) for bb in b]
    xs, iters = newton([[a.detach() for a in row] for row in AT], [bb.detach() for bb in bf],
                       [c.detach().reshape(-1) for c in c0], _num(lp2), dt, _num(wi), dc, eps, itrmax)
    # implicit-function derivative: x = x* - J^-1 G(x*; b, A, Wi, L^2), J exact and fixed
    xstar = [xs[m] for m in range(6)]
    with torch.no_grad():
        J = torch.func.vmap(torch.func.jacrev(
            lambda xv, at, bv: torch.stack(lyap([[at[r * 3 + q] for q in range(3)] for r in range(3)],
                                                list(bv), list(xv), _num(lp2), dt, _num(wi)))))(
            xs.T, torch.stack([AT[r][q].detach() for r in range(3) for q in range(3)], 1),
            torch.stack([bb.detach() for bb in bf], 1))
    G = torch.stack(lyap(AT, bf, xstar, lp2, dt, wi), 1)          # (N, 6), differentiable in b, A, wi, lp2
    corr = -torch.linalg.solve(J, G.unsqueeze(-1)).squeeze(-1)    # (N, 6)
    corr = corr - corr.detach()
    shape = c0[0].shape
    out = [(xstar[m] + corr[:, m]).reshape(shape) for m in range(6)]
    return out, iters


def stress(Cn, g: TGrid, lp2, coef):
    """Polymer stress divergence (fenep.f90:645-691) from C (halo, filled)."""
    dX, dY, dZ = g.dx, g.dy, g.dz
    f = (lp2 - 3) / (lp2 - Cn[0] - Cn[3] - Cn[5])
    C0 = [f * Cn[m] - E6[m] for m in range(6)]

    def c(m, a, b, cc):
        return sh(C0[m - 1], g, a, b, cc)
    tx = ((-c(1, 0, 0, 0) + c(1, 1, 0, 0)) / dX
          + (-c(2, 0, -1, 0) - c(2, 1, -1, 0) + c(2, 0, 1, 0) + c(2, 1, 1, 0)) / (4 * dY)
          + (-c(3, 0, 0, -1) - c(3, 1, 0, -1) + c(3, 0, 0, 1) + c(3, 1, 0, 1)) / (4 * dZ))
    ty = ((-c(2, -1, 0, 0) + c(2, 1, 0, 0) - c(2, -1, 1, 0) + c(2, 1, 1, 0)) / (4 * dX)
          + (-c(4, 0, 0, 0) + c(4, 0, 1, 0)) / dY
          + (-c(5, 0, 0, -1) - c(5, 0, 1, -1) + c(5, 0, 0, 1) + c(5, 0, 1, 1)) / (4 * dZ))
    tz = ((-c(3, -1, 0, 0) + c(3, 1, 0, 0) - c(3, -1, 0, 1) + c(3, 1, 0, 1)) / (4 * dX)
          + (-c(5, 0, -1, 0) + c(5, 0, 1, 0) - c(5, 0, -1, 1) + c(5, 0, 1, 1)) / (4 * dY)
          + (-c(6, 0, 0, 0) + c(6, 0, 0, 1)) / dZ)
    return [coef * tx, coef * ty, coef * tz]


def conv_visc(U, V, W, g: TGrid, vis):
    dX, dY, dZ = g.dx, g.dy, g.dz

    def u(a, b, c):
        return sh(U, g, a, b, c)

    def v(a, b, c):
        return sh(V, g, a, b, c)

    def w(a, b, c):
        return sh(W, g, a, b, c)
    t1 = (u(-1, 0, 0) + u(0, 0, 0)) / 2
    t2 = (u(0, 0, 0) + u(1, 0, 0)) / 2
    ax = ((-(t1 * t1) + t2 * t2) / dX
          + (-(v(0, -1, 0) + v(1, -1, 0)) / 2 * (u(0, -1, 0) + u(0, 0, 0)) / 2
             + (v(0, 0, 0) + v(1, 0, 0)) / 2 * (u(0, 0, 0) + u(0, 1, 0)) / 2) / dY)
    t3 = (v(0, -1, 0) + v(0, 0, 0)) / 2
    t4 = (v(0, 0, 0) + v(0, 1, 0)) / 2
    ay = ((-(u(-1, 0, 0) + u(-1, 1, 0)) / 2 * (v(-1, 0, 0) + v(0, 0, 0)) / 2
           + (u(0, 0, 0) + u(0, 1, 0)) / 2 * (v(0, 0, 0) + v(1, 0, 0)) / 2) / dX
          + (-(t3 * t3) + t4 * t4) / dY)
    bx = ((u(-1, 0, 0) - 2 * u(0, 0, 0) + u(1, 0, 0)) / (dX * dX)
          + (u(0, -1, 0) - 2 * u(0, 0, 0) + u(0, 1, 0)) / (dY * dY))
    by = ((v(-1, 0, 0) - 2 * v(0, 0, 0) + v(1, 0, 0)) / (dX * dX)
          + (v(0, -1, 0) - 2 * v(0, 0, 0) + v(0, 1, 0)) / (dY * dY))
    ax = ax + (-(w(0, 0, -1) + w(1, 0, -1)) / 2 * (u(0, 0, -1) + u(0, 0, 0)) / 2
               + (w(0, 0, 0) + w(1, 0, 0)) / 2 * (u(0, 0, 0) + u(0, 0, 1)) / 2) / dZ
    ay = ay + (-(w(0, 0, -1) + w(0, 1, -1)) / 2 * (v(0, 0, -1) + v(0, 0, 0)) / 2
               + (w(0, 0, 0) + w(0, 1, 0)) / 2 * (v(0, 0, 0) + v(0, 0, 1)) / 2) / dZ
    t5 = (w(0, 0, -1) + w(0, 0, 0)) / 2
    t6 = (w(0, 0, 0) + w(0, 0, 1)) / 2
    az = ((-(u(-1, 0, 0) + u(-1, 0, 1)) / 2 * (w(-1, 0, 0) + w(0, 0, 0)) / 2
           + (u(0, 0, 0) + u(0, 0, 1)) / 2 * (w(0, 0, 0) + w(1, 0, 0)) / 2) / dX
          + (-(v(0, -1, 0) + v(0, -1, 1)) / 2 * (w(0, -1, 0) + w(0, 0, 0)) / 2
             + (v(0, 0, 0) + v(0, 0, 1)) / 2 * (w(0, 0, 0) + w(0, 1, 0)) / 2) / dY
          + (-(t5 * t5) + t6 * t6) / dZ)
    bx = bx + (u(0, 0, -1) - 2 * u(0, 0, 0) + u(0, 0, 1)) / (dZ * dZ)
    by = by + (v(0, 0, -1) - 2 * v(0, 0, 0) + v(0, 0, 1)) / (dZ * dZ)
    bz = ((w(-1, 0, 0) - 2 * w(0, 0, 0) + w(1, 0, 0)) / (dX * dX)
          + (w(0, -1, 0) - 2 * w(0, 0, 0) + w(0, 1, 0)) / (dY * dY)
          + (w(0, 0, -1) - 2 * w(0, 0, 0) + w(0, 0, 1)) / (dZ * dZ))
    return [-ax, -ay, -az], [vis * bx, vis * by, vis * bz]


# ---------------------------------------------------------------------------
# spectral solves

def _kmod(n, d):
    th = 2 * PI / n
    return np.array([2 * (1 - math.cos(m * th)) / (d * d) for m in range(n)])


def solve_periodic(Q, g: TGrid, lhs0, lhs1):
    """fft_solve: IFFT(FFT(Q) / LHS), 0 where |LHS| < 1e-16.  Q (NZ, NY, NX)."""
    kx2 = torch.tensor(_kmod(g.nx, g.dx)[: g.nx // 2 + 1], dtype=F64)
    ky2 = torch.tensor(_kmod(g.ny, g.dy), dtype=F64)
    kz2 = torch.tensor(_kmod(g.nz, g.dz), dtype=F64)
    lam = kx2[None, None, :] + ky2[None, :, None] + kz2[:, None, None]
    lhs = lhs0 + lhs1 * lam
    H = torch.fft.rfftn(Q, dim=(0, 1, 2))
    with torch.no_grad():
        zero = torch.abs(lhs) < 1.0e-16
    H = torch.where(zero, torch.zeros_like(H), H / torch.where(zero, torch.ones_like(lhs), lhs))
    return torch.fft.irfftn(H, s=(g.nz, g.ny, g.nx), dim=(0, 1, 2))


def solve_walls(Q, g: TGrid, sys: str, kap, uwall=0.0):
    """FFT in x, z of rows 1..NY; per (kx, kz) the tridiagonal system over rows
    0..NY+1 (fenep_2d.f90:1179-1342); returns rows 0..NY+1, shape (NZ, NY+2, NX).
    sys 'u' (U, W), 'v' or 'p'; kap = dt beta / (2 Re) for 'u', 'v'."""
    NX, NY, NZ = g.nx, g.ny, g.nz
    NXH, n = NX // 2 + 1, NY + 2
    kx2 = torch.tensor(_kmod(NX, g.dx)[:NXH], dtype=F64)
    kz2 = torch.tensor(_kmod(NZ, g.dz), dtype=F64)
    lam = kz2[:, None] + kx2[None, :]                       # (NZ, NXH)
    H = torch.fft.fft(torch.fft.rfft(Q, dim=2), dim=0)       # (NZ, NY, NXH)
    rhs = torch.zeros(NZ, NXH, n, dtype=torch.complex128)
    rhs = rhs + torch.nn.functional.pad(H.permute(0, 2, 1), (1, 1))
    idy2 = 1.0 / (g.dy * g.dy)
    M = torch.zeros(NZ, NXH, n, n, dtype=F64)
    ar = torch.arange(n)
    if sys in ("u", "v"):
        a_int = 1.0 + kap * (lam[..., None] + 2.0 * idy2) * torch.ones(n, dtype=F64)
        b_int = -kap * idy2
    else:
        a_int = -(lam[..., None] + 2.0 * idy2) * torch.ones(n, dtype=F64)
        b_int = idy2
    rows_int = torch.zeros(n, dtype=torch.bool)
    if sys == "v":
        rows_int[1:NY] = True
    else:
        rows_int[1:NY + 1] = True
    Mi = torch.diag_embed(a_int) + b_int * (torch.diag(torch.ones(n - 1, dtype=F64), 1)
                                           + torch.diag(torch.ones(n - 1, dtype=F64), -1))
    M = torch.where(rows_int[:, None], Mi, M)
    fixed = torch.zeros(n, n, dtype=F64)
    if sys == "u":
        fixed[0, 0], fixed[0, 1] = 1.0, 1.0
        fixed[n - 1, n - 1], fixed[n - 1, n - 2] = 1.0, 1.0
    elif sys == "v":
        fixed[0, 0] = 1.0
        for j in range(NY, n):
            fixed[j, j] = 1.0
    else:
        fixed[0, 0], fixed[0, 1] = 1.0, -1.0
        fixed[n - 1, n - 1], fixed[n - 1, n - 2] = 1.0, -1.0
    M = torch.where(rows_int[:, None], M, fixed)
    keep = rows_int.clone()
    rhs = torch.where(keep, rhs, torch.zeros_like(rhs))
    if sys == "u" and uwall != 0.0:
        top = torch.zeros(NZ, NXH, n, dtype=torch.complex128)
        top[0, 0, n - 1] = 2 * uwall * NX * NZ
        rhs = rhs + top
    if sys == "p":
        # mode (0, 0) is singular; the Thomas guard of the reference pins the
        # top ghost row to 0 (fenep_2d.f90:1157-1160)
        pin = torch.zeros(n, n, dtype=F64)
        pin[n - 1, n - 1] = 1.0
        M = M.clone()
        M[0, 0] = torch.where((ar == n - 1)[:, None], pin, M[0, 0])
    X = torch.linalg.solve(M.to(torch.complex128), rhs.unsqueeze(-1)).squeeze(-1)   # (NZ, NXH, n)
    X = torch.fft.ifft(X, dim=0)
    return torch.fft.irfft(X.permute(0, 2, 1), n=NX, dim=2)    # (NZ, n, NX)


# ---------------------------------------------------------------------------
# IBM

def roma(r):
    """Roma kernel (fenep.f90:2045-2055).  The square roots of the branches not
    taken get a dummy argument 1, so that their (masked) gradients stay finite."""
    ar = torch.abs(r)
    is_in = ar < 0.5
    is_out = (ar >= 0.5) & (ar < 1.5)
    one = torch.ones_like(r)
    outer = (5.0 - 3.0 * ar - torch.sqrt(torch.where(is_out, -3.0 * ((1 - ar) * (1 - ar)) + 1.0, one))) / 6.0
    inner = (1.0 + torch.sqrt(torch.where(is_in, -3.0 * (r * r) + 1.0, one))) / 3.0
    return torch.where(is_in, inner, torch.where(is_out, outer, torch.zeros_like(r)))


def marker_geometry(cyls, dX):
    """Per marker (cylinder, dx, dy offsets from the centre, u, v), ordered as
    build_markers of the library (marker-major, cylinder-minor)."""
    per = []
    for l, cy in enumerate(cyls):
        DC = 2.0 * cy.r
        lst = []
        if not cy.filled:
            NL = max(int(round(PI * DC / dX)), 1)
            for j in range(1, NL + 1):
                ang = 2 * PI / NL * j
                lst.append((l, DC / 2 * math.cos(ang), DC / 2 * math.sin(ang),
                            cy.spin * math.sin(ang), -cy.spin * math.cos(ang)))
        else:
            NL_lap = int(DC / (2 * dX))
            shell = [int(math.floor(PI * (DC - 2 * i * dX) / dX + 0.5)) for i in range(NL_lap + 1)]
            if shell[NL_lap] == 0:
                shell[NL_lap] = 1
            for i in range(NL_lap + 1):
                for j in range(1, shell[i] + 1):
                    ang = 2 * PI / shell[i] * j
                    rr = (DC - 2 * i * dX) / 2
                    lst.append((l, rr * math.cos(ang), rr * math.sin(ang),
                                cy.spin * ((DC - 2 * i * dX) / DC * math.sin(ang)),
                                -cy.spin * ((DC - 2 * i * dX) / DC * math.cos(ang))))
        per.append(lst)
    out = []
    for m in range(max((len(p) for p in per), default=0)):
        for p in per:
            if m < len(p):
                out.append(p[m])
    return out


def ibm(Uas, centres, geom, g: TGrid, dt, cylvol=None):
    """Marker forces Fc[comp] (NZ, nm) and the folded spread forces (interior).
    Markers spread over dX^3 (fenep_mpi.f90:1794-1929), or over their
    cylinder's cylvol[l] when given."""
    dX, dY, dZ = g.dx, g.dy, g.dz
    NX, NY, NZ = g.nx, g.ny, g.nz
    SX, SY, SZ = NX + 2, NY + 2, NZ + 2
    nm = len(geom)
    cyl = torch.tensor([m[0] for m in geom])
    mx = centres[cyl, 0] + torch.tensor([m[1] for m in geom], dtype=F64)
    my = centres[cyl, 1] + torch.tensor([m[2] for m in geom], dtype=F64)
    mu = torch.tensor([m[3] for m in geom], dtype=F64)
    mv = torch.tensor([m[4] for m in geom], dtype=F64)
    dvol = (dX * dY) * dZ
    dxn = dX * dX * dX
    mvol = (torch.full((nm,), dxn, dtype=F64) if cylvol is None
            else torch.tensor([cylvol[m[0]] for m in geom], dtype=F64))
    n = torch.arange(1, NZ + 1, dtype=F64)
    zc = (n - 0.25) * dZ                                   # (NZ,)
    Fcs, fints = [], []
    for comp in range(3):
        with torch.no_grad():
            xd, yd = mx.detach(), my.detach()
            if comp == 0:
                j0 = torch.trunc(yd / dY).long(); i0 = torch.trunc(xd / dX - 0.5).long()
            elif comp == 1:
                j0 = torch.trunc(yd / dY - 0.5).long(); i0 = torch.trunc(xd / dX).long()
            else:
                j0 = torch.trunc(yd / dY).long(); i0 = torch.trunc(xd / dX).long()
        a = torch.arange(3)
        ii = i0[:, None] + a[None, :]                      # (nm, 3)
        jj = j0[:, None] + a[None, :]
        xg = (ii.to(F64) - 0.5) * dX + (0.5 * dX if comp == 0 else 0.0)
        yg = (jj.to(F64) - 0.5) * dY + (0.5 * dY if comp == 1 else 0.0)
        wx = roma((xg - mx[:, None]) / dX)                 # (nm, 3)
        wy = roma((yg - my[:, None]) / dY)
        kk = torch.arange(1, NZ + 1)[:, None] + torch.tensor([-1, 0, 1])[None, :]    # (NZ, 3)
        zg = (kk.to(F64) - 0.5) * dZ + (0.5 * dZ if comp == 2 else 0.0)
        wz = roma((zg - zc[:, None]) / dZ)                 # (NZ, 3)
        # delta of (plane n, marker m, kz, jy, ix)
        dlt = (wx[None, :, None, None, :] * wy[None, :, None, :, None] * wz[:, None, :, None, None]) / dvol
        flat = (ii[None, :, None, None, :] + SX * (jj[None, :, None, :, None] + SY * kk[:, None, :, None, None]))
        flat = flat.expand(NZ, nm, 3, 3, 3)
        Uf = Uas[comp].reshape(-1)
        ub = (Uf[flat] * dlt * dxn).sum(dim=(2, 3, 4))     # (NZ, nm)
        uc = mu if comp == 0 else (mv if comp == 1 else torch.zeros_like(mu))
        Fc = 0.0 + (uc[None, :] - ub) / dt
        Fcs.append(Fc)
        ftmp = torch.zeros(SZ * SY * SX, dtype=F64).index_add(
            0, flat.reshape(-1), (Fc[:, :, None, None, None] * dlt * mvol[None, :, None, None, None]).reshape(-1)
        ).reshape(SZ, SY, SX)
        # periodic fold (fenep.f90:2195-2205); y only when periodic
        ftmp = torch.cat([ftmp[:, :, 0:1], ftmp[:, :, 1:2] + ftmp[:, :, NX + 1:NX + 2], ftmp[:, :, 2:NX],
                          ftmp[:, :, NX:NX + 1] + ftmp[:, :, 0:1], ftmp[:, :, NX + 1:]], dim=2)
        if not g.walls:
            ftmp = torch.cat([ftmp[:, 0:1], ftmp[:, 1:2] + ftmp[:, NY + 1:NY + 2], ftmp[:, 2:NY],
                              ftmp[:, NY:NY + 1] + ftmp[:, 0:1], ftmp[:, NY + 1:]], dim=1)
        ftmp = torch.cat([ftmp[0:1], ftmp[1:2] + ftmp[NZ + 1:NZ + 2], ftmp[2:NZ],
                          ftmp[NZ:NZ + 1] + ftmp[0:1], ftmp[NZ + 1:]], dim=0)
        fints.append(ftmp[1:NZ + 1, 1:NY + 1, 1:NX + 1])
    return Fcs, fints, cyl


# ---------------------------------------------------------------------------
# the step

@dataclass
class TPhys:
    re: float
    dt: float
    newton_dc: float = 1.0e-5
    newton_eps: float = 1.0e-6
    newton_itrmax: int = 10000
    cylvol: tuple | None = None    # per-cylinder spreading volume; None: the cell volume


def arc_volumes(cyls, dX):
    """Spreading volume of each cylinder's markers under the arc element of
    smac.f90 (smac.f90:1128-1129, 1428-1446): dV = pi*DC/NL * dX * dX."""
    out = []
    for cy in cyls:
        DC = 2.0 * cy.r
        NL = max(int(round(PI * DC / dX)), 1)
        out.append(PI * DC / NL * dX * dX)
    return tuple(out)


def tphys(phys_spec, cyls, dX):
    """TPhys of a PhysSpec, with the arc-element volumes when it selects them."""
    arc = getattr(phys_spec, "ibm_volume", 0) == 1
    return TPhys(phys_spec.re, phys_spec.dt, phys_spec.newton_dc, phys_spec.newton_eps, phys_spec.newton_itrmax,
                 arc_volumes(cyls, dX) if arc else None)


def step(st: dict, prm: dict, g: TGrid, ph: TPhys, geom, first: bool):
    """One step.  st: U, V, W, P (halo), C (6, halo), A0, T0, F (3, interior).
    prm: wi, beta, lp2 (0-d tensors), centres (ncyl, 2).
    Returns (new state, drag (ncyl, 3))."""
    dt, re = ph.dt, ph.re
    wi, beta, lp2 = prm["wi"], prm["beta"], prm["lp2"]
    U, V, W, P, C = st["U"], st["V"], st["W"], st["P"], st["C"]
    if _num(beta) == 1.0:
        # Newtonian: C and T vanish and the polymer stage is skipped (fenep.f90:2479-2485)
        Cn = torch.zeros_like(C)
        T = [torch.zeros_like(sh(U, g)) for _ in range(3)]
        iters = None
    else:
        Cn_cells, iters = polymer(C, U, V, W, g, dt, wi, lp2, ph.newton_dc, ph.newton_eps, ph.newton_itrmax)
        if g.walls:
            # updated ghost rows kept through the stress (C_PBM in x, z only);
            # extrapolated at the end of the step (fenep_2d.f90:1371-1374)
            Cn = bc_xz(torch.stack([torch.nn.functional.pad(c, (1, 1, 0, 0, 1, 1)) for c in Cn_cells], 0), g)
        else:
            Cn = bc(torch.stack([embed(c, g) for c in Cn_cells], 0), "c", g)
        T = stress(Cn, g, lp2, (1.0 - beta) / (re * wi))
    A, B = conv_visc(U, V, W, g, beta / re)
    A0 = A if first else st["A0"]
    T0 = T if first else st["T0"]
    d = (g.dx, g.dy, g.dz)
    Us = (U, V, W)
    kinds = ("u", "v", "w")
    Ua = []
    for c in range(3):
        di = (1 if c == 0 else 0, 1 if c == 1 else 0, 1 if c == 2 else 0)
        gp = -dt * (-sh(P, g) + sh(P, g, *di)) / d[c]
        val = (sh(Us[c], g) + gp + dt * (3.0 * A[c] - A0[c]) / 2.0 + dt * B[c]
               + dt * (T[c] + T0[c]) / 2.0 + dt * st["F"][c])
        Ua.append(bc(embed(val, g), kinds[c], g))
    Fc, fint, cyl = ibm(Ua, prm["centres"], geom, g, dt, ph.cylvol)
    ncyl = prm["centres"].shape[0]
    dv = (torch.full((ncyl,), (g.dx * g.dy) * g.dz, dtype=F64) if ph.cylvol is None
          else torch.tensor(ph.cylvol, dtype=F64))
    drag = torch.stack([-torch.zeros(ncyl, dtype=F64).index_add(0, cyl, Fc[c].sum(0)) * dv for c in range(3)], 1)
    Q = [sh(Ua[c], g) + dt * fint[c] - dt * B[c] / 2 for c in range(3)]
    kap = dt * beta / re / 2.0
    Up = []
    for c in range(3):
        if not g.walls:
            x = embed(solve_periodic(Q[c], g, 1.0, kap), g)
        else:
            rows = solve_walls(Q[c], g, "v" if c == 1 else "u", kap, g.uwall if c == 0 else 0.0)
            x = torch.nn.functional.pad(rows, (1, 1, 0, 0, 1, 1))
        Up.append(bc(x, kinds[c], g))
    dX, dY, dZ = d
    rhs = ((-sh(Up[0], g, -1) + sh(Up[0], g)) / dX + (-sh(Up[1], g, 0, -1) + sh(Up[1], g)) / dY
           + (-sh(Up[2], g, 0, 0, -1) + sh(Up[2], g)) / dZ) / dt
    if not g.walls:
        Phi = embed(solve_periodic(rhs, g, 0.0, -1.0), g)
    else:
        Phi = torch.nn.functional.pad(solve_walls(rhs, g, "p", 0.0), (1, 1, 0, 0, 1, 1))
    Phi = bc(Phi, "p", g)
    ph0 = sh(Phi, g)
    Un = sh(Up[0], g) - dt * (-ph0 + sh(Phi, g, 1)) / dX
    Vn = sh(Up[1], g) - dt * (-ph0 + sh(Phi, g, 0, 1)) / dY
    Wn = sh(Up[2], g) - dt * (-ph0 + sh(Phi, g, 0, 0, 1)) / dZ
    lap = ((sh(Phi, g, -1) - 2 * ph0 + sh(Phi, g, 1)) / (dX * dX)
           + (sh(Phi, g, 0, -1) - 2 * ph0 + sh(Phi, g, 0, 1)) / (dY * dY)
           + (sh(Phi, g, 0, 0, -1) - 2 * ph0 + sh(Phi, g, 0, 0, 1)) / (dZ * dZ))
    Pn = sh(P, g) + ph0 - kap * lap
    new = {"U": bc(embed(Un, g), "u", g), "V": bc(embed(Vn, g), "v", g), "W": bc(embed(Wn, g), "w", g),
           "P": bc(embed(Pn, g), "p", g), "C": bc(Cn, "c", g) if g.walls else Cn, "A0": A, "T0": T, "F": st["F"],
           "Phi": Phi}
    return new, drag, iters


def state_from_numpy(arrs: dict, g: TGrid) -> dict:
    """Reference-layout numpy state (fortran8_gb300.solver.State.arrays) -> tensors
    with boundary values filled (as f8_load does)."""
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=F64)
    st = {"U": bc(t(arrs["u"]), "u", g), "V": bc(t(arrs["v"]), "v", g), "W": bc(t(arrs["w"]), "w", g),
          "P": bc(t(arrs["p"]), "p", g),
          "C": bc(t(np.moveaxis(arrs["c"], -1, 0)), "c", g),
          "A0": [t(arrs[n]) for n in ("ax0", "ay0", "az0")],
          "T0": [t(arrs[n]) for n in ("tx0", "ty0", "tz0")],
          "F": [t(arrs[n]) for n in ("fx", "fy", "fz")]}
    return st


def run(arrs: dict, grid_spec, phys_spec, cyls, params: dict, nsteps: int, weights=None, first_step=True):
    """Run nsteps from a numpy state; returns (J, drag history (nsteps, ncyl, 3),
    final state).  params: tensors wi, beta, lp2, centres (ncyl, 2), which may
    require grad.  J = sum(weights * drag); by default the time-averaged total
    x-drag, J = (1/nsteps) sum_n sum_l drag[n, l, 0]."""
    g = TGrid.from_spec(grid_spec)
    if getattr(phys_spec, "ibm_repeats", 1) != 1:
        raise ValueError("the torch step has one direct-forcing iteration")
    ph = tphys(phys_spec, cyls, g.dx)
    geom = marker_geometry(cyls, g.dx)
    st = state_from_numpy(arrs, g)
    drags = []
    for s in range(nsteps):
        st, drag, _ = step(st, params, g, ph, geom, first_step and s == 0 and phys_spec.ab2_start)
        drags.append(drag)
    D = torch.stack(drags, 0)
    if weights is None:
        w = torch.zeros_like(D)
        w[:, :, 0] = 1.0 / nsteps
    else:
        w = torch.as_tensor(weights, dtype=F64)
    J = (w * D).sum()
    return J, D, st
