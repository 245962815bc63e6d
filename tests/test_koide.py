"""The wall-bounded step against the reference's own accuracy table.

The reference reports the steady RMSE of its 2D wall-bounded solver against
Koide's analytic Poiseuille profile for NX = 16 ... 128 (_theory.py:44-49,
koide_theory fenep_2d.f90:1385-1437; tests/golden/koide_rmse.json).  The
steady discrete solution does not depend on dt, so the numbers are a pin of
the whole step.  The oracle (CPU) and the FP64 GPU path reproduce the
Newtonian column and both FENE-P columns (beta = 0.9, Wi = 1 and 10, with
the table's Lp = 10, tests/golden/make_koide.py) to 1e-10 relative.  The 3D
step (FP64 and FP32-mixed) reproduces the Newtonian column on the channel
extruded in z.
"""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from fortran8_gb300 import abi, validation
from fortran8_gb300.solver import Solver

GOLD = json.loads((Path(__file__).parent / "golden" / "koide_rmse.json").read_text())


def _case(fns, nx, pattern, nz=0, precision=abi.F8_FP64, steps=0):
    """(steady RMSE, the table's RMSE); steps = 0: run until the RMSE is
    stationary to 1e-12, else exactly that many steps."""
    p = GOLD["patterns"][pattern]
    g, ph, st = validation.koide_case(nx, p["beta"], p["wi"], GOLD["lp"], GOLD["re"], nz=nz)
    with Solver(fns, g, ph, (), precision=precision) as s:
        s.load(st)
        if steps:
            s.step(steps, want_drag=False)
            r = validation.koide_rmse(s.store(), nx, p["beta"], p["wi"], GOLD["lp"])
        else:
            r, _ = validation.run_to_steady(s, nx, p["beta"], p["wi"], GOLD["lp"])
    return r, GOLD["patterns"][pattern]["rmse"][GOLD["nx"].index(nx)]


@pytest.mark.parametrize("nx,pattern", [(16, "1"), (32, "1"), (16, "2"), (32, "2"), (16, "3")])
def test_oracle_channel_matches_reference_rmse(oracle, nx, pattern):
    r, ref = _case(oracle, nx, pattern)
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)


# The table's Wi = 10 entry at NX = 128 is typed as 0.000348 (3 digits) and lies
# 4.7 % above the converged value (3.323e-4; its three neighbours in the
# column agree to 12 digits), so that entry is not compared.  Wi = 10 takes
# about 50000 steps to converge; the GPU checks it at NX = 16 and 64.
GPU_CASES = [(nx, p) for p in ("1", "2") for nx in (16, 32, 64, 128)] + [(16, "3"), (64, "3")]


@pytest.mark.gpu
@pytest.mark.parametrize("nx,pattern", GPU_CASES)
def test_gpu_channel_matches_reference_rmse(gpu, nx, pattern):
    r, ref = _case(gpu, nx, pattern)
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)


# The 3D step on the same channel extruded over 4 cells in z: its steady
# Newtonian flow is the 2D one, so it reproduces the Newtonian column too
# (the FENE-P columns belong to the 2D model, f = (L^2 - 2)/(L^2 - tr C)).
def test_oracle_3d_channel_matches_reference_rmse(oracle):
    r, ref = _case(oracle, 16, "1", nz=4)
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("nx", [16, 64])
def test_gpu_3d_channel_matches_reference_rmse(gpu, nx):
    r, ref = _case(gpu, nx, "1", nz=4)
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("nx", [32, 64])
def test_gpu_mixed_3d_channel_matches_reference_rmse(gpu, nx):
    """The mixed-precision step (FP32 increments on a double-FP32 state) on the
    32-cell-deep channel.  Its RMSE is stationary after ~4000 steps; its steady
    state is the FP64 one up to the FP32 rounding of the right-hand side,
    which leaves the RMSE 1.5e-8 (NX = 32) and 1.3e-7 (NX = 64) away from the
    table in units of U (u_max = 1.23).  Bound: 4e-7."""
    r, ref = _case(gpu, nx, "1", nz=32, precision=abi.F8_MIXED, steps=10000)
    assert abs(r - ref) <= 4e-7, (r, ref)
