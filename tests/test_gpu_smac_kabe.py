"""The z-walled channel of smac_kabe.f90 (F8_BC_WALLS_Z) on the GPU, through
the C ABI:

* FP64 against the numpy restatement of smac_kabe.f90 (oracle/smac_kabe_np.py,
  pinned to the CPU oracle in tests/test_oracle_smac_kabe.py) with a tight
  sweep tolerance: velocities within 1e-10 (relative L2), the pressure within
  1e-9 up to its additive constant; at the reference's sweep tolerance
  (1e-5) within the sweep truncation (measured 3e-6 on u; bound 1e-5);
* the boundary exchange: a z-walled run equals, bit for bit, the y-walled run
  of the same box with y and z exchanged by the caller (FP64 and FP32-mixed,
  step, store and the state adjoint of f8_grad);
* FP32-mixed against FP64: the velocity vector within 1e-6;
* the entries that do not map the exchanged axes back refuse the box.
"""
from __future__ import annotations

import numpy as np
import pytest

from fortran8_gb300 import abi
from fortran8_gb300.solver import F8Error, Solver

from .conftest import interior, rel_l2
from .kabe_cases import restatement, state, swap_state, swapped_grid, workload

pytestmark = pytest.mark.gpu


def run(fns, w, st, steps, precision=abi.F8_FP64, grid=None):
    with Solver(fns, grid or w.grid, w.phys, (), precision=precision) as s:
        s.load(st)
        status, _ = s.step(steps)
        out = s.store()
    assert status == abi.F8_OK, status
    return out


@pytest.mark.parametrize("n,uwall", [(16, 1.0), (32, 0.0)])
def test_fp64_matches_restatement(gpu, n, uwall):
    w, force = workload(n, uwall=uwall, force=0.5)
    st = state(w, force)
    out = run(gpu, w, st, 8)
    ref = restatement(w, st, 8)
    for name, key in (("u", "U"), ("v", "V"), ("w", "W")):
        assert rel_l2(interior(out[name]), interior(ref[key])) < 1e-10, name
    pa, pb = interior(out["p"]), interior(ref["P"])
    assert rel_l2(pa - pa.mean(), pb - pb.mean()) < 1e-9


def test_reference_sweep_tolerance(gpu):
    w, force = workload(16, uwall=1.0, force=0.5)
    st = state(w, force)
    out = run(gpu, w, st, 8)
    ref = restatement(w, st, 8, eps=1e-5)
    err = rel_l2(interior(out["u"]), interior(ref["U"]))
    print("u vs the reference-tolerance restatement", err)
    assert err < 1e-5


@pytest.mark.parametrize("precision", [abi.F8_FP64, abi.F8_MIXED])
def test_exchange_is_bitwise_the_y_walled_box(gpu, precision):
    w, force = workload(32, uwall=1.0, force=0.5)
    st = state(w, force)
    out_z = run(gpu, w, st, 5, precision)
    out_y = swap_state(run(gpu, w, swap_state(st), 5, precision, grid=swapped_grid(w.grid))).arrays
    for name in ("u", "v", "w", "p", "c", "ax0", "ay0", "az0", "fx", "fy", "fz"):
        assert np.array_equal(out_z[name], out_y[name]), name


def test_state_adjoint_is_exchanged(gpu):
    w, force = workload(16, uwall=1.0, force=0.5)
    st = state(w, force)
    rng = np.random.default_rng(3)
    seed = state(w, 0.0)
    for name in ("u", "v", "w", "p"):
        seed.arrays[name] = rng.standard_normal(seed.arrays[name].shape)
    res = []
    for grid, s0, sd in ((w.grid, st, seed), (swapped_grid(w.grid), swap_state(st), swap_state(seed))):
        with Solver(gpu, grid, w.phys, ()) as s:
            s.load(s0)
            status, J, dp, ds, _ = s.grad(3, 0, None, sd, True)
        assert status == abi.F8_OK
        res.append(ds)
    back = swap_state(res[1]).arrays
    for name in ("u", "v", "w", "p", "ax0", "ay0", "az0"):
        assert np.array_equal(res[0][name], back[name]), name


def test_mixed_matches_fp64(gpu):
    w, force = workload(32, uwall=1.0, force=0.5)
    st = state(w, force)
    a = run(gpu, w, st, 20, abi.F8_MIXED)
    b = run(gpu, w, st, 20, abi.F8_FP64)
    # the velocity vector as a whole: v and w are noise-level (the flow is
    # driven along x), so their own relative errors are ill-posed
    diff = sum(np.sum((interior(a[f]) - interior(b[f])) ** 2) for f in ("u", "v", "w"))
    ref = sum(np.sum(interior(b[f]) ** 2) for f in ("u", "v", "w"))
    assert np.sqrt(diff / ref) < 1e-6


def test_unmapped_entries_refuse_the_box(gpu):
    w, force = workload(16)
    with Solver(gpu, w.grid, w.phys, ()) as s:
        s.load(state(w, force))
        s.step(1)
        with pytest.raises(F8Error):
            s.slice(2, 0)
        with pytest.raises(F8Error):
            s.selection_codes()
