"""Device iteration caps run out and are reported, in both precisions.

The reference continues silently when its Newton or SOR loop reaches itrmax
(fenep.f90:556-577, 885-901).  The library finishes the step the same way and
reports it: F8_WARN_NEWTON with the number of cell-steps that reached
newton_itrmax, and F8_WARN_SOR with poisson_iters = sor_itrmax + 1, the value
of the reference's loop counter after a DO loop that did not exit.  The caps
are made to run out by small limits (no GPU fault is involved).
"""
from __future__ import annotations

from dataclasses import replace

import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import Solver

pytestmark = pytest.mark.gpu

PRECISIONS = [abi.F8_FP64, abi.F8_MIXED]


def channel():
    return configs.scaled(configs.c3_channel(), 32, 16, 16)


def run(fns, w, steps, precision, poisson=abi.F8_POISSON_FFT):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision, poisson=poisson) as s:
        s.load(configs.initial_state(w))
        st, _ = s.step(steps)
        diag = s.diagnostics()
    return st, diag


@pytest.mark.parametrize("precision", PRECISIONS)
def test_newton_cap_reports_unconverged_cells(gpu, precision):
    w = channel()
    w = replace(w, phys=replace(w.phys, newton_itrmax=1))
    st, diag = run(gpu, w, 2, precision)
    assert st == abi.F8_WARN_NEWTON, st
    # cells of the update (interior and wall ghost rows) that stopped at the cap
    assert 0 < diag.newton_unconverged <= 2 * w.grid.nx * (w.grid.ny + 2) * w.grid.nz
    assert diag.nan_found == 0


@pytest.mark.parametrize("precision", PRECISIONS)
def test_newton_without_cap_is_ok(gpu, precision):
    st, diag = run(gpu, channel(), 2, precision)
    assert st == abi.F8_OK
    assert diag.newton_unconverged == 0


@pytest.mark.parametrize("precision", PRECISIONS)
def test_sor_cap_reports_warning(gpu, precision):
    w = channel()
    w = replace(w, phys=replace(w.phys, sor_itrmax=2, sor_eps=1e-12))
    st, diag = run(gpu, w, 1, precision, poisson=abi.F8_POISSON_SOR)
    assert st == abi.F8_WARN_SOR, st
    assert diag.poisson_iters == w.phys.sor_itrmax + 1


@pytest.mark.parametrize("precision", PRECISIONS)
def test_sor_converging_within_cap_reports_its_count(gpu, precision):
    w = channel()
    w = replace(w, phys=replace(w.phys, sor_itrmax=5000))
    st, diag = run(gpu, w, 1, precision, poisson=abi.F8_POISSON_SOR)
    assert st == abi.F8_OK, st
    assert 1 <= diag.poisson_iters <= w.phys.sor_itrmax
