"""The CPU oracle reports its iteration caps as the library does.

The reference continues silently when Newton or SOR reaches itrmax
(fenep.f90:556-577, 885-901); the oracle finishes the step and returns
F8_WARN_NEWTON / F8_WARN_SOR, with poisson_iters = sor_itrmax + 1 (the value of
the reference's loop counter after a DO loop that did not exit).  The GPU
library's counterpart is tests/test_gpu_caps.py.
"""
from __future__ import annotations

from dataclasses import replace

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import Solver


def run(fns, w, steps, poisson=abi.F8_POISSON_FFT):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=abi.F8_FP64, poisson=poisson) as s:
        s.load(configs.initial_state(w))
        st, _ = s.step(steps)
        diag = s.diagnostics()
    return st, diag


def test_oracle_reports_the_same_caps(oracle):
    w = configs.scaled(configs.c3_channel(), 16, 8, 8)
    wn = replace(w, phys=replace(w.phys, newton_itrmax=1))
    st, diag = run(oracle, wn, 1)
    assert st == abi.F8_WARN_NEWTON and diag.newton_unconverged > 0
    ws = replace(w, phys=replace(w.phys, sor_itrmax=2, sor_eps=1e-12))
    st, diag = run(oracle, ws, 1, poisson=abi.F8_POISSON_SOR)
    assert st == abi.F8_WARN_SOR and diag.poisson_iters == 3
