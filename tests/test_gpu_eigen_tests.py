"""The alternative SPD tests of the face candidates (f8_phys.eigen_test: the
reference's eigen_method 0, 1, 2; fenep.f90:187-212, 384-461) on the FP64 GPU
step against the CPU oracle: relative L2 <= 1e-10 on u, v, w, p, C and
<= 1e-12 on the drag, with the selection codes compared after every step
(Sylvester's test is exact arithmetic; Cardano's and the symmetric solver's
transcendentals can break a near-tie differently, counted as flips)."""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import F8Error, Solver

from .conftest import interior, rel_l2
from .test_gpu_configs import lockstep

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", [abi.F8_EIGEN_CARDANO, abi.F8_EIGEN_SYLVESTER, abi.F8_EIGEN_SYMMETRIC])
@pytest.mark.parametrize("name,shape,steps", [("c3_channel", (32, 16, 16), 20), ("c2_3d", (16, 16, 16), 20)])
def test_eigen_test_matches_oracle(gpu, oracle, method, name, shape, steps):
    w = configs.scaled(configs.WORKLOADS[name](), *shape)
    w = replace(w, phys=replace(w.phys, eigen_test=method))
    og, oo, dg, do, iters, flips = lockstep(gpu, oracle, w, steps)
    for f in ("u", "v", "w", "p", "c"):
        assert rel_l2(interior(og[f]), interior(oo[f])) <= 1e-10, f
    assert np.max(np.abs(dg - do)) <= 1e-12 * np.max(np.abs(do))
    if method == abi.F8_EIGEN_SYLVESTER:
        assert sum(flips) == 0


def test_alternative_tests_are_fp64_3d_only(gpu):
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    with pytest.raises(F8Error):
        Solver(gpu, w.grid, replace(w.phys, eigen_test=abi.F8_EIGEN_CARDANO), w.cyls, precision=abi.F8_MIXED)
