"""Shared helpers of the z-walled channel tests (smac_kabe.f90): the seeded
state with the reference's halo fills, the exchange of y and z that maps
the z-walled box onto the y-walled one, and the numpy restatement's run."""
from __future__ import annotations

import sys
from dataclasses import replace
from pathlib import Path

import numpy as np

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import GridSpec, State

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT / "oracle") not in sys.path:
    sys.path.insert(0, str(ROOT / "oracle"))

import smac_kabe_np as sk  # noqa: E402


def workload(n=16, uwall=1.0, force=0.5):
    """smac_kabe's channel with a moving upper wall and a uniform x force
    (the reference's defaults are uwall = 0 and no force, a decaying noise)."""
    w = configs.smac_kabe(n, uwall)
    return w, force


def state(w, force):
    st = configs.initial_state(w)
    st.arrays["fx"][:] = force
    kg = kabe_grid(w, 1e-13)
    # the reference's halo fills of the initial state (smac_kabe.f90:98-103)
    for name, fill in (("u", sk.u_kabe), ("v", sk.v_kabe), ("w", sk.w_kabe), ("p", sk.p_kabe)):
        fill(st.arrays[name], kg)
    return st


def kabe_grid(w, eps, itrmax=3000):
    # the mean mode's pressure right-hand side is round-off (the plane means
    # of div u vanish), so its sweeps never meet a relative tolerance and run
    # to the cap, in the reference too; 3000 sweeps converge every other mode
    # to 1e-13
    g = w.grid
    return sk.KabeGrid(g.nx, g.ny, g.nz, g.lx, g.ly, g.lz, re=w.phys.re, dt=w.phys.dt, uwall=g.uwall, eps=eps,
                       itrmax=itrmax)


def restatement(w, st, steps, eps=1e-13):
    kg = kabe_grid(w, eps)
    a = st.arrays
    s = {"U": a["u"].copy(), "V": a["v"].copy(), "W": a["w"].copy(), "P": a["p"].copy(),
         "A0": [a["ax0"].copy(), a["ay0"].copy(), a["az0"].copy()], "F": [a["fx"], a["fy"], a["fz"]]}
    return sk.run(s, kg, steps, first_step=True)


# y <-> z exchange of the caller's fields (axis 0 is k, axis 1 is j)
def swap_state(st: State) -> State:
    a = st.arrays
    out = {}
    sw = lambda x: np.ascontiguousarray(np.swapaxes(x, 0, 1))
    out["u"], out["v"], out["w"] = sw(a["u"]), sw(a["w"]), sw(a["v"])
    out["p"], out["phi"] = sw(a["p"]), sw(a["phi"])
    c = sw(a["c"])
    out["c"] = np.ascontiguousarray(c[..., [0, 2, 1, 5, 4, 3]])
    for base in ("a", "t", "f"):
        x, y, z = (f"{base}x0", f"{base}y0", f"{base}z0") if base != "f" else ("fx", "fy", "fz")
        out[x], out[y], out[z] = sw(a[x]), sw(a[z]), sw(a[y])
    return State(out)


def swapped_grid(g: GridSpec) -> GridSpec:
    return replace(g, ny=g.nz, nz=g.ny, ly=g.lz, lz=g.ly, bc_y=abi.F8_BC_WALLS)
