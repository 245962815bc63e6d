"""Seeded states for the gradient tests (shared by the CPU and GPU tests).

Each case is a small 3D workload whose flow has been advanced by the CPU
oracle for a few steps from the seeded initial state, with a stretched
polymer (C_xx up to ~60 at L^2 = 400) so that the L^2 and Wi sensitivities are
well above round-off, and cylinder centres moved off the grid lines so that
no marker sits on a break point of the Roma kernel (where the drag is only
once differentiable and central differences lose an order).
"""
from __future__ import annotations

import sys
from dataclasses import replace
from pathlib import Path

import numpy as np

from fortran8_gb300 import configs
from fortran8_gb300.solver import Solver

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT / "oracle") not in sys.path:
    sys.path.insert(0, str(ROOT / "oracle"))


def case(name: str, oracle_fns, spinup: int = 10):
    """(workload, state, step0) of a gradient case: 'channel' (32x16x16, y walls,
    two filled cylinders), 'periodic' (16^3, one cylinder), 'moving' (the channel
    with surface-ring cylinders spinning and the upper wall moving), 'arc' (the
    moving case with markers spread over the arc element of their ring) or
    'newtonian' (the channel with beta = 1: no polymer stage)."""
    if name in ("channel", "moving", "newtonian", "arc"):
        w = configs.scaled(configs.c4_adjoint(), 32, 16, 16)
    else:
        w = configs.scaled(configs.c2_3d(), 16, 16, 16)
    cyls = tuple(replace(c, xc=c.xc + 0.0123, yc=c.yc + 0.0371) for c in w.cyls)
    if name in ("moving", "arc"):
        cyls = tuple(replace(c, filled=0, spin=0.4 * (1 - 2 * l)) for l, c in enumerate(cyls))
        w = replace(w, grid=replace(w.grid, uwall=0.3))
    if name == "newtonian":
        w = replace(w, phys=replace(w.phys, beta=1.0))
    if name == "arc":
        from fortran8_gb300 import abi
        w = replace(w, phys=replace(w.phys, ibm_volume=abi.F8_IBM_ARC_VOLUME))
    w = replace(w, cyls=cyls)
    st = configs.initial_state(w)
    g = w.grid
    dX, dZ = g.lx / g.nx, g.lz / g.nz
    i = np.arange(0, g.nx + 2)[None, None, :]
    k = np.arange(0, g.nz + 2)[:, None, None]
    cxx = 1.0 + 30.0 * (1.0 + 0.5 * np.sin((i - 0.5) * dX) * np.cos((k - 0.5) * dZ))
    st.arrays["c"][..., 0] = np.broadcast_to(cxx, st.arrays["c"].shape[:3])
    st.arrays["c"][..., 1] = 0.5 * np.broadcast_to(np.cos((i - 0.5) * dX), st.arrays["c"].shape[:3])
    if spinup == 0:
        return w, st, 0
    with Solver(oracle_fns, w.grid, w.phys, w.cyls) as o:
        o.load(st)
        o.step(spinup)
        out = o.store()
    return w, out, spinup


def params_of(w):
    import torch
    return {"wi": torch.tensor(w.phys.wi, dtype=torch.float64),
            "beta": torch.tensor(w.phys.beta, dtype=torch.float64),
            "lp2": torch.tensor(w.phys.lp2, dtype=torch.float64),
            "centres": torch.tensor([[c.xc, c.yc] for c in w.cyls], dtype=torch.float64)}


def with_params(w, vec):
    """Workload with (Wi, beta, L^2, xc0, yc0, ...) = vec."""
    ph = replace(w.phys, wi=float(vec[0]), beta=float(vec[1]), lp2=float(vec[2]))
    cyls = tuple(replace(c, xc=float(vec[3 + 2 * l]), yc=float(vec[4 + 2 * l])) for l, c in enumerate(w.cyls))
    return replace(w, phys=ph, cyls=cyls)


def param_vector(w):
    v = [w.phys.wi, w.phys.beta, w.phys.lp2]
    for c in w.cyls:
        v += [c.xc, c.yc]
    return np.array(v)


def torch_grad(w, st, step0, nsteps, weights=None, seed=None):
    """(J, dJ/dparams vector, dJ/d(initial interior state) dict) from the torch
    restatement.  seed: dict of adjoint arrays of the final state (reference
    layouts) added to J as <seed, final state> over interior cells."""
    import torch
    import f8_torch as ft
    prm = params_of(w)
    for v in prm.values():
        v.requires_grad_(True)
    g = ft.TGrid.from_spec(w.grid)
    leaves = {}
    arrs = dict(st.arrays)
    st_t = {}
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    for n, kind in (("u", "u"), ("v", "v"), ("w", "w"), ("p", "p")):
        leaves[n] = t(arrs[n]).requires_grad_(True)
    leaves["c"] = t(np.moveaxis(arrs["c"], -1, 0)).requires_grad_(True)
    for n in ("ax0", "ay0", "az0", "tx0", "ty0", "tz0"):
        leaves[n] = t(arrs[n]).requires_grad_(True)
    st_t["U"] = ft.bc(leaves["u"], "u", g)
    st_t["V"] = ft.bc(leaves["v"], "v", g)
    st_t["W"] = ft.bc(leaves["w"], "w", g)
    st_t["P"] = ft.bc(leaves["p"], "p", g)
    st_t["C"] = ft.bc(leaves["c"], "c", g)
    st_t["A0"] = [leaves[n] for n in ("ax0", "ay0", "az0")]
    st_t["T0"] = [leaves[n] for n in ("tx0", "ty0", "tz0")]
    st_t["F"] = [t(arrs[n]) for n in ("fx", "fy", "fz")]
    ph = ft.tphys(w.phys, w.cyls, g.dx)
    geom = ft.marker_geometry(w.cyls, g.dx)
    drags = []
    cur = st_t
    for s in range(nsteps):
        cur, drag, _ = ft.step(cur, prm, g, ph, geom, step0 + s == 0 and bool(w.phys.ab2_start))
        drags.append(drag)
    D = torch.stack(drags, 0)
    if weights is None:
        wt = torch.zeros_like(D)
        wt[:, :, 0] = 1.0 / nsteps
    else:
        wt = torch.as_tensor(np.broadcast_to(weights, D.shape).copy(), dtype=torch.float64)
    Jd = (wt * D).sum()
    J = Jd
    if seed is not None:
        I = lambda a: a[..., 1:-1, 1:-1, 1:-1]
        for n, key in (("u", "U"), ("v", "V"), ("w", "W"), ("p", "P")):
            if n in seed:
                J = J + (I(cur[key]) * I(t(seed[n]))).sum()
        if "c" in seed:
            J = J + (I(cur["C"]) * I(t(np.moveaxis(seed["c"], -1, 0)))).sum()
        for q, n in enumerate(("ax0", "ay0", "az0")):
            if n in seed:
                J = J + (cur["A0"][q] * t(seed[n])).sum()
        for q, n in enumerate(("tx0", "ty0", "tz0")):
            if n in seed:
                J = J + (cur["T0"][q] * t(seed[n])).sum()
    J.backward()
    val = lambda v: v.grad.numpy() if v.grad is not None else np.zeros(tuple(v.shape))
    gp = [float(val(prm["wi"])), float(val(prm["beta"])), float(val(prm["lp2"]))]
    gp += list(val(prm["centres"]).ravel())
    dstate = {}
    for n, v in leaves.items():
        a = v.grad.numpy() if v.grad is not None else np.zeros(tuple(v.shape))
        if n == "c":
            a = np.moveaxis(a, 0, -1)
        if a.ndim >= 3 and n in ("u", "v", "w", "p", "c"):
            a = a.copy()
            # halo entries of the leaves do not reach the state (bc overwrites them)
            mask = np.zeros(a.shape[:3], dtype=bool)
            mask[1:-1, 1:-1, 1:-1] = True
            a[~mask] = 0.0
        dstate[n] = a
    return Jd.item(), np.array(gp), dstate, D.detach().numpy()
