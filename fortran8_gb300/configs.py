"""Seeded initial states and parameters of the benchmark workloads.

The reference generates its initial noise with Fortran ``random_number``
(fenep.f90:88-103), which is not reproducible across compilers, so the state
is generated here with numpy ``default_rng(seed)`` in the reference's form
``amp * (rand - 0.5)`` and handed to both the GPU library and the oracle
through the same ``load`` call.

Workloads (sizes and physics as stated for the benchmark; box lengths are
chosen so that dX = dY = dZ, which the IBM requires, fenep.f90:1808-1810):

* ``c1_2d``     2D periodic 2pi x 2pi, 128^2, one filled cylinder r = 0.5 at the
                centre, U = 1 + noise, Re 100, Wi 1, beta 0.9, L^2 100, dt 1e-3.
* ``c2_3d``     3D periodic (2pi)^3, 64^3, Taylor-Green + noise, one spanwise
                cylinder r = 0.4, Re 200, Wi 2, beta 0.8, L^2 400, dt 5e-4.
* ``c3_channel`` 256 x 128 x 128, box 4pi x 2pi x 2pi, no-slip walls in y,
                Poiseuille base flow + noise 1e-2, 2 x 2 spanwise cylinders
                r = 0.3, Re 500, Wi 5, beta 0.9, L^2 900, dt 2e-4.
* ``c4_adjoint`` 128 x 64 x 64 channel, 2 cylinders r = 0.3, Re 300, Wi 3,
                beta 0.85, L^2 400, dt 5e-4.
* ``c5_large``  512 x 256 x 256 channel, 4 x 2 cylinders r = 0.25, Re 1000,
                Wi 8, beta 0.9, L^2 1600, dt 1e-4.
* ``smac_rotating`` the Newtonian IBM case of smac.f90 (smac.f90:13-27,
                1156-1196): (2pi)^3 periodic box, 64^3 (smac.f90 uses 144^3,
                which the radix-2 transforms do not take), four rotating
                surface-ring cylinders of diameter 2pi/6 at (pi/2 | 3pi/2)^2
                with unit surface speed and alternating sense, Re =
                U_C L_C / nu = 5400 for f_C = 2 rps, D_C = 0.03 m, nu = 1e-6,
                dt 8e-5, markers spread with the arc element of their ring
                (smac.f90:1129), noise 1e-3 on a fluid at rest.
* ``smac_kabe``  the z-walled Newtonian channel of smac_kabe.f90
                (smac_kabe.f90:4-37): 16^3 cells in the box normalised by
                Xmax (1 x 1 x 1), walls normal to z, Re 5, dt = dt_C U_C / Xmax
                with dt_C = 0.01 and U_C = Zmax^2 Re / 8, noise 1e-3 on a fluid
                at rest; the upper wall speed is a parameter (0 in the
                reference).

The channel is driven by the uniform body force Fx = 2 / (Re h^2), h = Ly/2,
under which the laminar Newtonian profile is the Poiseuille base flow with
centre-line speed 1 (the reference drives its Poiseuille case with Fx = 1,
fenep_2d.f90:88-90).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

from . import abi
from .solver import CylSpec, GridSpec, PhysSpec, State, empty_state

PI = math.pi


@dataclass
class Workload:
    name: str
    grid: GridSpec
    phys: PhysSpec
    cyls: tuple
    steps: int
    seed: int
    noise: float
    flow: str  # "uniform", "taylor_green", "poiseuille"

    @property
    def cells(self) -> int:
        return self.grid.cells


def _phys(re, wi, beta, lp2, dt, dim):
    if dim == 2:  # fenep_2d.f90:291-293
        return PhysSpec(re=re, wi=wi, beta=beta, lp2=lp2, dt=dt, newton_dc=1.0e-10,
                        newton_eps=1.0e-10, newton_itrmax=10000)
    return PhysSpec(re=re, wi=wi, beta=beta, lp2=lp2, dt=dt)  # fenep.f90:526-528


def c1_2d(n=128):
    g = GridSpec(2, n, n, 1, 2 * PI, 2 * PI, 2 * PI / n)
    return Workload("c1_2d", g, _phys(100.0, 1.0, 0.9, 100.0, 1.0e-3, 2),
                    (CylSpec(PI, PI, 0.5),), 1000, 0, 1.0e-3, "uniform")


def c2_3d(n=64):
    g = GridSpec(3, n, n, n, 2 * PI, 2 * PI, 2 * PI)
    return Workload("c2_3d", g, _phys(200.0, 2.0, 0.8, 400.0, 5.0e-4, 3),
                    (CylSpec(PI, PI, 0.4),), 500, 1, 1.0e-3, "taylor_green")


def _channel(name, nx, ny, nz, re, wi, beta, lp2, dt, cyls, steps, seed, noise):
    g = GridSpec(3, nx, ny, nz, 4 * PI, 2 * PI, 2 * PI * nz / ny, abi.F8_BC_WALLS, 0.0)
    return Workload(name, g, _phys(re, wi, beta, lp2, dt, 3), tuple(cyls), steps, seed, noise,
                    "poiseuille")


def c3_channel(nx=256, ny=128, nz=128, r=0.3):
    lx, ly = 4 * PI, 2 * PI
    cyls = [CylSpec(x, y, r) for y in (ly / 4, 3 * ly / 4) for x in (lx / 4, 3 * lx / 4)]
    return _channel("c3_channel", nx, ny, nz, 500.0, 5.0, 0.9, 900.0, 2.0e-4, cyls, 2000, 2, 1.0e-2)


def c4_adjoint(nx=128, ny=64, nz=64):
    lx, ly = 4 * PI, 2 * PI
    cyls = [CylSpec(lx / 4, ly / 2, 0.3), CylSpec(3 * lx / 4, ly / 2, 0.3)]
    return _channel("c4_adjoint", nx, ny, nz, 300.0, 3.0, 0.85, 400.0, 5.0e-4, cyls, 400, 3, 1.0e-2)


def c5_large(nx=512, ny=256, nz=256):
    lx, ly = 4 * PI, 2 * PI
    cyls = [CylSpec(x, y, 0.25) for y in (ly / 4, 3 * ly / 4) for x in (lx / 8, 3 * lx / 8, 5 * lx / 8, 7 * lx / 8)]
    return _channel("c5_large", nx, ny, nz, 1000.0, 8.0, 0.9, 1600.0, 1.0e-4, cyls, 200, 4, 1.0e-2)


def smac_rotating(n=64, repeats=1):
    g = GridSpec(3, n, n, n, 2 * PI, 2 * PI, 2 * PI)
    dc = 2 * PI / 6.0
    f_c, d_c, nu = 2.0, 0.03, 1.0e-6
    re = (f_c * PI * d_c) * (d_c / dc) / nu
    ph = PhysSpec(re=re, wi=1.0, beta=1.0, lp2=100.0, dt=8.0e-5, ibm_volume=abi.F8_IBM_ARC_VOLUME,
                  ibm_repeats=repeats)
    pos = ((PI / 2, PI / 2, 1.0), (3 * PI / 2, PI / 2, -1.0), (PI / 2, 3 * PI / 2, -1.0), (3 * PI / 2, 3 * PI / 2, 1.0))
    cyls = tuple(CylSpec(x, y, dc / 2, spin=s, filled=0) for x, y, s in pos)
    return Workload("smac_rotating", g, ph, cyls, 10, 5, 1.0e-3, "rest")


def smac_kabe(n=16, uwall=0.0):
    g = GridSpec(3, n, n, n, 1.0, 1.0, 1.0, bc_y=abi.F8_BC_WALLS_Z, uwall=uwall)
    re = 5.0
    u_c = (2 * PI) ** 2 * re / 8.0
    ph = PhysSpec(re=re, wi=1.0, beta=1.0, lp2=100.0, dt=0.01 * u_c / (2 * PI))
    return Workload("smac_kabe", g, ph, (), 10, 11, 1.0e-3, "rest")


WORKLOADS = {"c1_2d": c1_2d, "c2_3d": c2_3d, "c3_channel": c3_channel,
             "c4_adjoint": c4_adjoint, "c5_large": c5_large, "smac_rotating": smac_rotating, "smac_kabe": smac_kabe}


def initial_state(w: Workload) -> State:
    """Seeded initial state of a workload in the reference layouts."""
    g = w.grid
    st = empty_state(g)
    rng = np.random.default_rng(w.seed)
    nx, ny, nz = g.nx, g.ny, g.nz
    dX, dY, dZ = g.lx / nx, g.ly / ny, (g.lz / nz if g.dim == 3 else g.lx / nx)
    shp = g.interior_shape
    noise = {}
    for name in ("u", "v", "w") if g.dim == 3 else ("u", "v"):
        noise[name] = w.noise * (rng.random(shp) - 0.5)
    i = np.arange(1, nx + 1)[None, None, :]
    j = np.arange(1, ny + 1)[None, :, None]
    k = np.arange(1, nz + 1)[:, None, None]
    u = np.zeros(shp); v = np.zeros(shp); wv = np.zeros(shp)
    if w.flow == "uniform":
        u[:] = 1.0
    elif w.flow == "rest":
        pass
    elif w.flow == "taylor_green":
        # u at (i dX, (j-1/2) dY, (k-1/2) dZ), v at ((i-1/2) dX, j dY, (k-1/2) dZ)
        u[:] = np.sin(i * dX) * np.cos((j - 0.5) * dY) * np.cos((k - 0.5) * dZ)
        v[:] = -np.cos((i - 0.5) * dX) * np.sin(j * dY) * np.cos((k - 0.5) * dZ)
    elif w.flow == "poiseuille":
        h = g.ly / 2
        y = (j - 0.5) * dY
        u[:] = (1.0 - ((y - h) / h) ** 2) * np.ones(shp)
        st.arrays["fx"][:] = 2.0 / (w.phys.re * h * h)
    u += noise["u"]
    v += noise["v"]
    if g.dim == 3:
        wv += noise["w"]
    st.arrays["u"][1:-1, 1:-1, 1:-1] = u
    st.arrays["v"][1:-1, 1:-1, 1:-1] = v
    if g.dim == 3:
        st.arrays["w"][1:-1, 1:-1, 1:-1] = wv
    cc = st.arrays["c"]
    if g.dim == 3:
        cc[..., 0] = 1.0
        cc[..., 3] = 1.0
        cc[..., 5] = 1.0
    else:
        cc[..., 0] = 1.0
        cc[..., 2] = 1.0
    return st


def scaled(w: Workload, nx: int, ny: int, nz: int) -> Workload:
    """Same physics on a smaller grid (for tests that the oracle finishes in seconds)."""
    g = replace(w.grid, nx=nx, ny=ny, nz=nz)
    if g.bc_y == abi.F8_BC_WALLS:
        g = replace(g, lz=g.ly * nz / ny)
    elif g.dim == 2:
        g = replace(g, lz=g.lx / nx)
    return replace(w, grid=g)
