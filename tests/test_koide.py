"""The wall-bounded step against the reference's own accuracy table.

The reference reports the steady RMSE of its 2D wall-bounded solver against
Koide's analytic Poiseuille profile for NX = 16 ... 128 (_theory.py:44-49,
koide_theory fenep_2d.f90:1385-1437; tests/golden/koide_rmse.json).  The
steady discrete solution does not depend on dt, so the numbers are a pin of
the whole step: the oracle (CPU) and the FP64 GPU path reproduce the
Newtonian column to 1e-10 relative.
"""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from fortran8_gb300 import validation
from fortran8_gb300.solver import Solver

GOLD = json.loads((Path(__file__).parent / "golden" / "koide_rmse.json").read_text())


def _case(fns, nx, pattern):
    p = GOLD["patterns"][pattern]
    g, ph, st = validation.koide_case(nx, p["beta"], p["wi"], GOLD["lp"], GOLD["re"])
    with Solver(fns, g, ph, ()) as s:
        s.load(st)
        r, steps = validation.run_to_steady(s, nx, p["beta"], p["wi"], GOLD["lp"])
    return r, GOLD["patterns"][pattern]["rmse"][GOLD["nx"].index(nx)]


@pytest.mark.parametrize("nx", [16, 32])
def test_oracle_newtonian_channel_matches_reference_rmse(oracle, nx):
    r, ref = _case(oracle, nx, "1")
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("nx", [16, 32, 64, 128])
def test_gpu_newtonian_channel_matches_reference_rmse(gpu, nx):
    r, ref = _case(gpu, nx, "1")
    assert abs(r - ref) <= 1e-10 * ref, (r, ref)
