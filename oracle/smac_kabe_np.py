"""CPU restatement (numpy, FP64) of the z-walled Newtonian channel step of
smac_kabe.f90 (method 1, pattern 1) — test infrastructure: the oracle of
the library's walls-normal-to-z mode (f8_grid.wall_axis = F8_WALL_Z).

Arrays are indexed [k, j, i] (x fastest in memory, the reference's
(0:NX+1, 0:NY+1, 0:NZ+1) Fortran layout); halo fields have shape
(NZ+2, NY+2, NX+2), interior fields (NZ, NY, NX).  The step, in the
reference's order (smac_kabe.f90:1740-1760):

* convection (divergence form) and viscous terms, smac_kabe.f90:159-235;
* fft_navier_kabe, smac_kabe.f90:757-973: the right-hand side with the AB2
  convection (the first step copies A into A0) and half the viscous term,
  2D FFT over (x, y), and per (kx, ky) mode a Gauss-Seidel / SOR sweep along
  z of the Crank-Nicolson system until sqrt(sum|E|^2 / sum|Q|^2) < eps; the
  wall rows: U, V ghost = -interior (2 Uwall - interior for the mean mode of
  U at the top), W = 0 on the wall faces (the W system runs over k < NZ);
* fft_poisson_kabe, smac_kabe.f90:975-1053: the same sweeps for the pressure
  correction with Neumann rows, then the zero-mean shift;
* fft_march, smac_kabe.f90:1055-1104, and the wall / periodic halo fills
  U_kabe .. P_kabe, smac_kabe.f90:118-157.

The sweep tolerance `eps` and relaxation `omega` are parameters: the
reference uses eps = 1e-5 and omega = 2 / (1 + sin(pi dX)) with dX = 1/NX
(smac_kabe.f90:24-25); a tight eps makes the sweeps converge to the direct
tridiagonal solution.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class KabeGrid:
    nx: int
    ny: int
    nz: int
    lx: float = 1.0
    ly: float = 1.0
    lz: float = 1.0
    re: float = 5.0
    dt: float = 0.01
    uwall: float = 0.0
    eps: float = 1.0e-5
    omega: float | None = None
    itrmax: int = 10000

    @property
    def dx(self):
        return self.lx / self.nx

    @property
    def dy(self):
        return self.ly / self.ny

    @property
    def dz(self):
        return self.lz / self.nz

    @property
    def sor(self):
        # smac_kabe.f90:24, dX normalised by Xmax
        return self.omega if self.omega is not None else 2.0 / (1.0 + math.sin(math.pi / self.nx))


def _xy_periodic(A, g):
    # x, y periodic halo (smac_kabe.f90:119-122)
    A[:, :, 0] = A[:, :, g.nx]
    A[:, :, g.nx + 1] = A[:, :, 1]
    A[:, 0, :] = A[:, g.ny, :]
    A[:, g.ny + 1, :] = A[:, 1, :]


def u_kabe(U, g):
    _xy_periodic(U, g)
    U[0] = -U[1]
    U[g.nz + 1] = 2 * g.uwall - U[g.nz]


def v_kabe(V, g):
    _xy_periodic(V, g)
    V[0] = -V[1]
    V[g.nz + 1] = -V[g.nz]


def w_kabe(W, g):
    _xy_periodic(W, g)
    W[0] = 0.0
    W[g.nz] = 0.0
    W[g.nz + 1] = 0.0


def p_kabe(P, g):
    _xy_periodic(P, g)
    P[0] = P[1]
    P[g.nz + 1] = P[g.nz]


def _s(A, di=0, dj=0, dk=0):
    """interior view of a halo field shifted by (di, dj, dk)"""
    nz, ny, nx = A.shape[0] - 2, A.shape[1] - 2, A.shape[2] - 2
    return A[1 + dk:1 + dk + nz, 1 + dj:1 + dj + ny, 1 + di:1 + di + nx]


def convection(U, V, W, g):
    """smac_kabe.f90:159-199 (divergence form, sign flipped at the end)"""
    dX, dY, dZ = g.dx, g.dy, g.dz
    s = _s
    Ax = ((-((s(U, -1) + s(U)) / 2) ** 2 + ((s(U) + s(U, 1)) / 2) ** 2) / dX
          + (-(s(V, 0, -1) + s(V, 1, -1)) / 2 * (s(U, 0, -1) + s(U)) / 2
             + (s(V) + s(V, 1)) / 2 * (s(U) + s(U, 0, 1)) / 2) / dY
          + (-(s(W, 0, 0, -1) + s(W, 1, 0, -1)) / 2 * (s(U, 0, 0, -1) + s(U)) / 2
             + (s(W) + s(W, 1)) / 2 * (s(U) + s(U, 0, 0, 1)) / 2) / dZ)
    Ay = ((-(s(U, -1) + s(U, -1, 1)) / 2 * (s(V, -1) + s(V)) / 2
           + (s(U) + s(U, 0, 1)) / 2 * (s(V) + s(V, 1)) / 2) / dX
          + (-((s(V, 0, -1) + s(V)) / 2) ** 2 + ((s(V) + s(V, 0, 1)) / 2) ** 2) / dY
          + (-(s(W, 0, 0, -1) + s(W, 0, 1, -1)) / 2 * (s(V, 0, 0, -1) + s(V)) / 2
             + (s(W) + s(W, 0, 1)) / 2 * (s(V) + s(V, 0, 0, 1)) / 2) / dZ)
    Az = ((-(s(U, -1) + s(U, -1, 0, 1)) / 2 * (s(W, -1) + s(W)) / 2
           + (s(U) + s(U, 0, 0, 1)) / 2 * (s(W) + s(W, 1)) / 2) / dX
          + (-(s(V, 0, -1) + s(V, 0, -1, 1)) / 2 * (s(W, 0, -1) + s(W)) / 2
             + (s(V) + s(V, 0, 0, 1)) / 2 * (s(W) + s(W, 0, 1)) / 2) / dY
          + (-((s(W, 0, 0, -1) + s(W)) / 2) ** 2 + ((s(W) + s(W, 0, 0, 1)) / 2) ** 2) / dZ)
    return -Ax, -Ay, -Az


def viscous(U, V, W, g):
    """smac_kabe.f90:201-235 (nu constant: 1/Re times the 7-point Laplacian)"""
    out = []
    for A in (U, V, W):
        lap = ((_s(A, -1) - 2 * _s(A) + _s(A, 1)) / g.dx ** 2
               + (_s(A, 0, -1) - 2 * _s(A) + _s(A, 0, 1)) / g.dy ** 2
               + (_s(A, 0, 0, -1) - 2 * _s(A) + _s(A, 0, 0, 1)) / g.dz ** 2)
        out.append(1.0 / g.re * lap)
    return out


def _modes(g):
    """2 (1 - cos) / d^2 of every (ky, kx) mode of the (y, x) real transform"""
    kx = 2 * (1 - np.cos(np.arange(g.nx // 2 + 1) * (1.0 / g.nx) * 2 * math.pi)) / g.dx ** 2
    ky = 2 * (1 - np.cos(np.arange(g.ny) * (1.0 / g.ny) * 2 * math.pi)) / g.dy ** 2
    return ky[:, None] + kx[None, :]


def _sweeps(Qh, B0, BZ, g, kind):
    """Gauss-Seidel / SOR sweeps along z of every mode, each until its own
    residual passes (smac_kabe.f90:800-834, 1013-1039).  Qh: (NZ, NY, NX/2+1)
    right-hand sides; B0: (NY, NX/2+1) centre coefficients; BZ: off-diagonal.
    kind: 'u' (-ghost, moving top wall for the mean mode), 'v' (-ghost),
    'w' (zero on the wall faces, rows k < NZ) or 'p' (Neumann)."""
    nz = g.nz
    X = np.zeros((nz + 2,) + Qh.shape[1:], dtype=complex)
    Q = Qh.copy()
    if kind == "w":
        Q[nz - 1] = 0.0
    er0 = np.sum(np.abs(Q) ** 2, axis=0) + 1.0e-16
    active = np.ones(Qh.shape[1:], dtype=bool)
    E = np.zeros_like(Q)
    kmax = nz - 1 if kind == "w" else nz
    for _ in range(g.itrmax):
        if not active.any():
            break
        for k in range(1, kmax + 1):
            e = BZ * X[k - 1] - B0 * X[k] + BZ * X[k + 1] - Q[k - 1]
            E[k - 1] = np.where(active, e, E[k - 1])
            X[k] = np.where(active, X[k] + g.sor * e / B0, X[k])
        if kind == "u":
            X[0] = np.where(active, -X[1], X[0])
            top = -X[nz]
            top[0, 0] = 2 * g.uwall - X[nz][0, 0]
            X[nz + 1] = np.where(active, top, X[nz + 1])
        elif kind == "v":
            X[0] = np.where(active, -X[1], X[0])
            X[nz + 1] = np.where(active, -X[nz], X[nz + 1])
        elif kind == "p":
            X[0] = np.where(active, X[1], X[0])
            X[nz + 1] = np.where(active, X[nz], X[nz + 1])
        else:
            E[nz - 1] = 0.0
        er = np.sum(np.abs(E) ** 2, axis=0)
        active &= ~(np.sqrt(er / er0) < g.eps)
    return X


def _to_real(X, g):
    """fftc2r_2d of every plane k = 0 .. NZ+1 (unnormalised) into a halo field"""
    A = np.zeros((g.nz + 2, g.ny + 2, g.nx + 2))
    A[:, 1:g.ny + 1, 1:g.nx + 1] = np.fft.irfft2(X, s=(g.ny, g.nx), axes=(1, 2)) * (g.nx * g.ny)
    return A


def _to_modes(Q, g):
    return np.fft.rfft2(Q, axes=(1, 2)) / (g.nx * g.ny)


def step(st: dict, g: KabeGrid, first: bool) -> dict:
    """One step; st: U, V, W, P (halo), A0 = (Ax0, Ay0, Az0), F = (Fx, Fy, Fz)
    (interior).  Returns the new state (A0 updated)."""
    U, V, W, P = st["U"], st["V"], st["W"], st["P"]
    A = convection(U, V, W, g)
    B = viscous(U, V, W, g)
    A0 = [a.copy() for a in A] if first else st["A0"]
    dt = g.dt
    grads = ((1, 0, 0, g.dx), (0, 1, 0, g.dy), (0, 0, 1, g.dz))
    B0 = -(1 + dt / g.re / 2.0 * (_modes(g) + 2.0 / g.dz ** 2))
    BZ = -dt / g.re / 2.0 / g.dz ** 2
    vel = []
    for c, (Uc, kind) in enumerate(((U, "u"), (V, "v"), (W, "w"))):
        di, dj, dk, d = grads[c]
        Q = (_s(Uc) - dt * (-_s(P) + _s(P, di, dj, dk)) / d + dt * (3.0 * A[c] - A0[c]) / 2.0
             + dt * B[c] / 2.0 + dt * st["F"][c])
        X = _sweeps(_to_modes(Q, g), B0, BZ, g, kind)
        vel.append(_to_real(X, g))
    Up, Vp, Wp = vel
    u_kabe(Up, g)
    v_kabe(Vp, g)
    w_kabe(Wp, g)
    # fft_poisson_kabe
    Q = ((-_s(Up, -1) + _s(Up)) / g.dx + (-_s(Vp, 0, -1) + _s(Vp)) / g.dy + (-_s(Wp, 0, 0, -1) + _s(Wp)) / g.dz) / dt
    X = _sweeps(_to_modes(Q, g), _modes(g) + 2.0 / g.dz ** 2, 1.0 / g.dz ** 2, g, "p")
    # the centre coefficient enters the sweep as -B0 (E = BZ X- - B0 X + BZ X+ - Q)
    Phi = _to_real(X, g)
    Phi -= Phi[1:g.nz + 1, 1:g.ny + 1, 1:g.nx + 1].mean()
    p_kabe(Phi, g)
    # fft_march
    Un, Vn, Wn, Pn = (np.zeros_like(U) for _ in range(4))
    Un[1:-1, 1:-1, 1:-1] = _s(Up) - dt * (-_s(Phi) + _s(Phi, 1)) / g.dx
    Vn[1:-1, 1:-1, 1:-1] = _s(Vp) - dt * (-_s(Phi) + _s(Phi, 0, 1)) / g.dy
    Wn[1:-1, 1:-1, 1:-1] = _s(Wp) - dt * (-_s(Phi) + _s(Phi, 0, 0, 1)) / g.dz
    lap = ((_s(Phi, -1) - 2 * _s(Phi) + _s(Phi, 1)) / g.dx ** 2
           + (_s(Phi, 0, -1) - 2 * _s(Phi) + _s(Phi, 0, 1)) / g.dy ** 2
           + (_s(Phi, 0, 0, -1) - 2 * _s(Phi) + _s(Phi, 0, 0, 1)) / g.dz ** 2)
    Pn[1:-1, 1:-1, 1:-1] = _s(P) + _s(Phi) - dt / g.re / 2.0 * lap
    u_kabe(Un, g)
    v_kabe(Vn, g)
    w_kabe(Wn, g)
    p_kabe(Pn, g)
    return {"U": Un, "V": Vn, "W": Wn, "P": Pn, "A0": list(A), "F": st["F"], "Phi": Phi}


def run(st: dict, g: KabeGrid, nsteps: int, first_step: bool = True) -> dict:
    for s in range(nsteps):
        st = step(st, g, first_step and s == 0)
    return st
