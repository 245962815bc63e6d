"""The staged projection of the FP32-mixed step (k_march_tma: row pairs of
its inputs brought into shared memory by bulk asynchronous copies on
mbarriers), which F8_STAGED_PROJECTION=1 selects when a context is created,
gives the same bits as the default direct-load kernel (k_march_df): fields, drag and
diagnostics after several steps, on the channel (y walls, Neumann rows of
Phi) and on the periodic box (wrapped rows and planes), with grids whose y
tiles and z runs do not divide evenly."""
from __future__ import annotations

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def run(gpu, w, steps):
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(configs.initial_state(w))
        st, drag = s.step(steps)
        out = s.store()
        diag = s.diagnostics()
    assert st == abi.F8_OK, st
    return drag, out, diag


@pytest.mark.parametrize("name,shape", [("c3_channel", (64, 32, 32)), ("c3_channel", (128, 64, 32)),
                                        ("c2_3d", (32, 32, 32)), ("c2_3d", (64, 64, 64))])
def test_staged_projection_matches_direct_loads_bitwise(gpu, monkeypatch, name, shape):
    w = configs.scaled(configs.WORKLOADS[name](), *shape)
    monkeypatch.setenv("F8_STAGED_PROJECTION", "1")
    d1, o1, g1 = run(gpu, w, 12)
    monkeypatch.delenv("F8_STAGED_PROJECTION", raising=False)
    d0, o0, g0 = run(gpu, w, 12)
    assert np.array_equal(d1, d0)
    for f in ("u", "v", "w", "p", "c", "ax0", "ay0", "az0"):
        assert np.array_equal(o1[f], o0[f]), f
    assert g1.ke == g0.ke and g1.div_max == g0.div_max
