"""The wall-bounded step against the reference's own accuracy table.

The reference reports the steady RMSE of its 2D wall-bounded solver against
Koide's analytic Poiseuille profile for NX = 16 ... 128 (_theory.py:44-49,
koide_theory fenep_2d.f90:1385-1437; tests/golden/koide_rmse.json).  The
steady discrete solution does not depend on dt, so the numbers are a pin of
the whole step.  The oracle (CPU) and the FP64 GPU path reproduce the
Newtonian column and both FENE-P columns (beta = 0.9, Wi = 1 and 10, with
the table's Lp = 10, tests/golden/make_koide.py) to 1e-10 relative.
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
