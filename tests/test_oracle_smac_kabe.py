"""The numpy restatement of smac_kabe.f90's z-walled channel step
(oracle/smac_kabe_np.py) against the CPU oracle's y-walled step on the same
box with y and z exchanged.  smac_kabe.f90 solves its (kx, ky) systems with
SOR sweeps along z (smac_kabe.f90:800-834, 1013-1039); with a tight sweep
tolerance they converge to the oracle's direct tridiagonal solves, and the
two steps agree to round-off: velocities within 1e-11 (relative L2), the
pressure within 1e-10 up to its additive constant (smac_kabe.f90 shifts the
correction to zero mean, the tridiagonal solve pins the mean mode).  At the
reference's tolerance (1e-5) the sweeps stop early; the difference is the
sweep truncation."""
from __future__ import annotations

import numpy as np

from fortran8_gb300.solver import Solver

from .conftest import interior, rel_l2
from .kabe_cases import restatement, state, swap_state, swapped_grid, workload


def oracle_run(oracle, w, st, steps):
    g = swapped_grid(w.grid)
    with Solver(oracle, g, w.phys, ()) as s:
        s.load(swap_state(st))
        s.step(steps)
        out = s.store()
    return swap_state(out)   # the exchange is its own inverse


def test_restatement_matches_oracle_on_the_exchanged_box(oracle):
    w, force = workload(16, uwall=1.0, force=0.5)
    st = state(w, force)
    ref = restatement(w, st, 6)
    out = oracle_run(oracle, w, st, 6).arrays
    for name, key in (("u", "U"), ("v", "V"), ("w", "W")):
        assert rel_l2(interior(out[name]), interior(ref[key])) < 1e-11, name
    pa, pb = interior(out["p"]), interior(ref["P"])
    assert rel_l2(pa - pa.mean(), pb - pb.mean()) < 1e-10


def test_reference_tolerance_is_the_sweep_truncation(oracle):
    w, force = workload(16, uwall=1.0, force=0.5)
    st = state(w, force)
    loose = restatement(w, st, 6, eps=1e-5)
    tight = restatement(w, st, 6, eps=1e-13)
    err = rel_l2(interior(loose["U"]), interior(tight["U"]))
    assert 0.0 < err < 1e-4, err
