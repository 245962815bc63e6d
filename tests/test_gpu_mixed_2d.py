"""FP32-mixed 2D step (fenep_2d.f90:1912-1966) vs the FP64 oracle and the FP64
GPU step, through the C ABI.

The 2D mixed step keeps the velocity and pressure as double-float pairs and
computes the conformation tensor (c11, c12, c22), the momentum increments and
the FP32 solves in FP32, with the FP64 defect correction of the pressure, as
the 3D mixed step does.  Cases: the 2D periodic benchmark box with its filled
cylinder (scaled to 32^2 and at its full 128^2 for 200 steps against the FP64
GPU step), and a 2D wall channel (Poiseuille base flow, filled cylinder, the
reference's wall mode with the polymer update on the ghost rows), each from a
stretched polymer field; the Newtonian variant (beta = 1) of each.

Gate as for 3D: drag within 1e-5 relative of the FP64 result, velocity within
1e-5 relative L2, C within 1e-5, the projected velocity divergence-free to
FP64 round-off.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import CylSpec, F8Error, GridSpec, Solver

from .conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

PI = np.pi
DRAG_TOL = 1e-5
VEL_TOL = 1e-5


def workload(name, n=32, beta=None):
    if name == "periodic":
        w = configs.c1_2d(n)
    else:
        g = GridSpec(2, n, n // 2, 1, 2 * PI, PI, 2 * PI / n, abi.F8_BC_WALLS, 0.0)
        w = configs.Workload("channel2d", g, replace(configs.c1_2d().phys, re=20.0, dt=2e-3),
                             (CylSpec(PI + 0.0123, PI / 2 + 0.0371, 0.4),), 10, 5, 1e-2, "poiseuille")
    if beta is not None:
        w = replace(w, phys=replace(w.phys, beta=beta))
    return w


def stretched(w):
    """The workload's initial state with a stretched, non-uniform C."""
    st = configs.initial_state(w)
    g = w.grid
    dX = g.lx / g.nx
    i = np.arange(0, g.nx + 2)[None, None, :]
    j = np.arange(0, g.ny + 2)[None, :, None]
    shape = st.arrays["c"].shape[:3]
    st.arrays["c"][..., 0] = np.broadcast_to(1.0 + 20.0 * (1.0 + 0.5 * np.sin((i - 0.5) * dX) * np.cos((j - 0.5) * dX)), shape)
    st.arrays["c"][..., 1] = 0.5 * np.broadcast_to(np.cos((i - 0.5) * dX), shape)
    return st


def run(fns, w, st, steps, precision):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(st)
        status, drag = s.step(steps)
        return status, drag, s.store(), s.diagnostics()


def drag_rel(dm, d64):
    return float(np.max(np.abs(dm[..., 0] - d64[..., 0])) / np.max(np.abs(d64[..., 0])))


@pytest.mark.parametrize("name,beta", [("periodic", None), ("channel", None), ("periodic", 1.0), ("channel", 1.0)])
def test_mixed_2d_matches_fp64_oracle(gpu, oracle, name, beta):
    w = workload(name, beta=beta)
    st = stretched(w)
    steps = 30
    sm, dm, om, diag = run(gpu, w, st, steps, abi.F8_MIXED)
    so, do, oo, diag_o = run(oracle, w, st, steps, abi.F8_FP64)
    assert sm == abi.F8_OK, sm
    assert drag_rel(dm, do) <= DRAG_TOL
    for f in ("u", "v"):
        assert rel_l2(interior(om[f]), interior(oo[f])) <= VEL_TOL, f
    pm, po = interior(om["p"]), interior(oo["p"])
    assert rel_l2(pm - pm.mean(), po - po.mean()) <= 1e-4
    if w.phys.beta != 1.0:
        assert rel_l2(interior(om["c"]), interior(oo["c"])) <= 1e-5
        for f in ("trc_mean", "trc_max"):
            a, b = getattr(diag, f), getattr(diag_o, f)
            assert abs(a - b) <= 1e-5 * abs(b), (f, a, b)
    assert abs(diag.ke - diag_o.ke) <= 1e-5 * abs(diag_o.ke)
    assert diag.div_max < 1e-9


def test_mixed_2d_benchmark_box_matches_fp64_gpu(gpu):
    """The 2D benchmark configuration at its full 128^2, 200 steps: the mixed
    step against the FP64 GPU step (itself pinned to the oracle)."""
    w = configs.c1_2d()
    st = configs.initial_state(w)
    sm, dm, om, _ = run(gpu, w, st, 200, abi.F8_MIXED)
    s6, d6, o6, _ = run(gpu, w, st, 200, abi.F8_FP64)
    assert sm == abi.F8_OK and s6 == abi.F8_OK
    assert drag_rel(dm, d6) <= DRAG_TOL
    for f in ("u", "v"):
        assert rel_l2(interior(om[f]), interior(o6[f])) <= VEL_TOL, f
    assert rel_l2(interior(om["c"]), interior(o6["c"])) <= 1e-5


def test_mixed_2d_store_load_resumes(gpu):
    """Store, load and continue equals stepping straight through (the 2D
    mixed state round-trips through the FP64 fields exactly)."""
    w = workload("channel")
    st = stretched(w)
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(st)
        s.step(10)
        mid = s.store()
        _, d_a = s.step(5)
        end_a = s.store()
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(mid, 10)
        _, d_b = s.step(5)
        end_b = s.store()
    assert np.array_equal(d_a, d_b)
    for f in ("u", "v", "p", "c"):
        assert np.array_equal(end_a[f], end_b[f]), f


def test_mixed_2d_gradient_is_unsupported(gpu):
    w = workload("periodic")
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(configs.initial_state(w))
        with pytest.raises(F8Error) as err:
            s.grad(2, 0)
    assert err.value.status == abi.F8_ERR_UNSUPPORTED
