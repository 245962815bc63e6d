"""The smac.f90 options of the immersed-boundary forcing on the GPU, through the
C ABI, against the CPU oracle:

* markers spread with the arc element of their ring, dV = pi*DC/NL * dX * dX
  (smac.f90:1128-1129, 1428-1446), and the drag integrated with it;
* NS direct-forcing iterations per step (smac.f90:20, 1607-1611): the marker
  force accumulates over the iterations, each interpolating the last
  Helmholtz solution.

The workload is smac.f90's Newtonian rotating-cylinder box at 32^3 (four
surface-ring cylinders, alternating spin, fluid at rest plus noise).  FP64:
relative L2 <= 1e-10 on u, v, w, p and <= 1e-12 on the drag history (beta = 1:
no polymer stage, so no eigen-test choices).  FP32-mixed against the FP64
step over 50 steps: drag within 5e-5 of its largest component, the velocity
vector within 1e-5 (at Re 5400 the marker slip is a small difference of O(1)
velocities, so the FP32 interpolation weights' rounding shows in the force
at a few 1e-5).  The gradient of the arc-element
forcing is checked in tests/test_gpu_adjoint.py (case 'arc'); f8_grad refuses
NS > 1.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import F8Error, Solver

from .conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-10
DRAG_TOL = 1e-12


def workload(repeats, volume=abi.F8_IBM_ARC_VOLUME, n=32):
    w = configs.smac_rotating(n, repeats)
    return replace(w, phys=replace(w.phys, ibm_volume=volume))


def run(fns, w, steps, precision=abi.F8_FP64):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(configs.initial_state(w))
        st, drag = s.step(steps)
        out = s.store()
    assert st == abi.F8_OK, st
    return drag, out


def drag_err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("repeats,volume", [(1, abi.F8_IBM_ARC_VOLUME), (3, abi.F8_IBM_ARC_VOLUME),
                                            (4, abi.F8_IBM_CELL_VOLUME)])
def test_fp64_matches_oracle(gpu, oracle, repeats, volume):
    w = workload(repeats, volume)
    dg, og = run(gpu, w, 20)
    do, oo = run(oracle, w, 20)
    for f in ("u", "v", "w", "p"):
        assert rel_l2(interior(og[f]), interior(oo[f])) <= FIELD_TOL, f
    assert drag_err(dg, do) <= DRAG_TOL


@pytest.mark.parametrize("repeats", [1, 3])
def test_mixed_matches_fp64(gpu, repeats):
    w = workload(repeats)
    dm, om = run(gpu, w, 50, abi.F8_MIXED)
    d6, o6 = run(gpu, w, 50, abi.F8_FP64)
    assert drag_err(dm, d6) <= 5e-5
    # the velocity vector as a whole: w is noise-level (the cylinders spin
    # about z), so its own relative error is ill-posed
    diff = sum(np.sum((interior(om[f]) - interior(o6[f])) ** 2) for f in ("u", "v", "w"))
    ref = sum(np.sum(interior(o6[f]) ** 2) for f in ("u", "v", "w"))
    assert np.sqrt(diff / ref) <= 1e-5


def test_forcing_iterations_reduce_the_marker_slip(gpu):
    """With NS iterations the drag moves towards its limit: the first step's
    drag at NS = 2, 4 approaches NS = 8 monotonically."""
    d = {ns: run(gpu, workload(ns), 1)[0] for ns in (1, 2, 4, 8)}
    e = [np.max(np.abs(d[ns] - d[8])) for ns in (1, 2, 4)]
    assert e[0] > e[1] > e[2] > 0.0, e


@pytest.mark.parametrize("precision", [abi.F8_FP64, abi.F8_MIXED])
def test_grad_refuses_repeated_forcing(gpu, precision):
    w = workload(2, n=16)
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(configs.initial_state(w))
        with pytest.raises(F8Error):
            s.grad(2)
