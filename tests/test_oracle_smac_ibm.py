"""The smac.f90 variant of the immersed-boundary forcing in the CPU oracle:
markers spread with the arc element of their ring, dV = pi*DC/NL * dX * dX
(smac.f90:1128-1129, 1428-1446), and NS direct-forcing iterations per step
(smac.f90:20, 1607-1611).  The GPU library's counterpart is
tests/test_gpu_smac_ibm.py."""
from __future__ import annotations

import math
from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import F8Error, Solver


def small(repeats=1, volume=abi.F8_IBM_ARC_VOLUME):
    w = configs.smac_rotating(16, repeats)
    return replace(w, phys=replace(w.phys, ibm_volume=volume))


def drag_of(fns, w, steps):
    with Solver(fns, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        _, d = s.step(steps)
    return d


def test_arc_volume_scales_the_first_drag_by_the_ring_element(oracle):
    """From the same state the first iteration's marker forces do not depend on
    the spreading volume, so the first step's drag scales by dV / (dX dY dZ)."""
    wa, wc = small(), small(volume=abi.F8_IBM_CELL_VOLUME)
    da, dc = drag_of(oracle, wa, 1), drag_of(oracle, wc, 1)
    g = wa.grid
    dx = g.lx / g.nx
    for l, cy in enumerate(wa.cyls):
        nl = max(1, round(math.pi * 2 * cy.r / dx))
        ratio = (math.pi * 2 * cy.r / nl * dx * dx) / (dx * dx * dx)
        assert np.allclose(da[0, l], dc[0, l] * ratio, rtol=1e-13, atol=1e-300)


def test_forcing_iterations_converge(oracle):
    """More forcing iterations move the drag towards a limit (the marker no-slip
    residual shrinks), and NS = 1 is the single-iteration step."""
    d = {ns: drag_of(oracle, small(ns), 2) for ns in (1, 2, 4, 8)}
    assert np.array_equal(drag_of(oracle, small(), 2), d[1])
    e = {ns: np.max(np.abs(d[ns] - d[8])) for ns in (1, 2, 4)}
    assert e[1] > e[2] > e[4] > 0.0, e


def test_options_are_validated(oracle):
    w = small()
    with pytest.raises(F8Error):
        Solver(oracle, w.grid, replace(w.phys, ibm_repeats=0), w.cyls)
    with pytest.raises(F8Error):   # the arc element belongs to surface rings
        Solver(oracle, w.grid, w.phys, tuple(replace(c, filled=1) for c in w.cyls))
    w2 = configs.scaled(configs.c1_2d(), 16, 16, 1)
    with pytest.raises(F8Error):   # 3D only
        Solver(oracle, w2.grid, replace(w2.phys, ibm_volume=abi.F8_IBM_ARC_VOLUME),
               tuple(replace(c, filled=0) for c in w2.cyls))
