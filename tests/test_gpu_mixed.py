"""FP32-mixed step vs the FP64 oracle (and the FP64 GPU step) through the C ABI.

Gate (the benchmark's accuracy condition): drag within 1e-5 relative of the
FP64 result; velocity within 1e-5 relative L2; the projected velocity is
divergence-free to FP64 round-off thanks to the FP64 defect correction of
the FP32 Poisson solve.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from fortran8_gb300 import abi, configs
from fortran8_gb300.solver import F8Error, Solver

from .conftest import interior, rel_l2

pytestmark = pytest.mark.gpu

DRAG_TOL = 1e-5
VEL_TOL = 1e-5


def run(fns, w, steps, precision):
    with Solver(fns, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(configs.initial_state(w))
        st, drag = s.step(steps)
        return st, drag, s.store(), s.diagnostics()


def drag_rel(dm, d64, all_components=False):
    """Max deviation of the drag (x force) relative to its largest magnitude in the history.

    With all_components the scale is the largest force component: in the
    Taylor-Green box the cylinder sits at a stagnation point and its drag is
    noise-level, so a relative drag error is ill-posed there.
    """
    if all_components:
        return float(np.max(np.abs(dm - d64)) / np.max(np.abs(d64)))
    return float(np.max(np.abs(dm[..., 0] - d64[..., 0])) / np.max(np.abs(d64[..., 0])))


@pytest.mark.parametrize("name,shape,steps", [("c3_channel", (32, 16, 16), 30), ("c2_3d", (16, 16, 16), 30),
                                              ("c4_adjoint", (32, 16, 16), 20)])
def test_mixed_matches_fp64_oracle(gpu, oracle, name, shape, steps):
    w = configs.scaled(configs.WORKLOADS[name](), *shape)
    sm, dm, om, diag = run(gpu, w, steps, abi.F8_MIXED)
    so, do, oo, diag_o = run(oracle, w, steps, abi.F8_FP64)
    assert sm == abi.F8_OK
    if name != "c2_3d":
        # the drag gate applies to the channel workloads; in the Taylor-Green
        # box the cylinder sits at a stagnation point and its force is
        # noise-level, so only the fields are compared there
        assert drag_rel(dm, do) <= DRAG_TOL
    # the on-device diagnostics of the double-float state against the oracle
    for f in ("ke", "trc_mean", "trc_max"):
        a, b = getattr(diag, f), getattr(diag_o, f)
        assert abs(a - b) <= 1e-5 * abs(b), (f, a, b)
    # the pressure is compared up to its additive constant
    pm, po = interior(om["p"]), interior(oo["p"])
    assert rel_l2(pm - pm.mean(), po - po.mean()) <= 1e-4
    for f in ("u", "v", "w"):
        assert rel_l2(interior(om[f]), interior(oo[f])) <= VEL_TOL, f
    assert rel_l2(interior(om["c"]), interior(oo["c"])) <= 1e-5
    assert diag.div_max < 1e-9


def test_mixed_matches_fp64_gpu_longer(gpu):
    w = configs.scaled(configs.c3_channel(), 64, 32, 32)
    _, dm, om, _ = run(gpu, w, 200, abi.F8_MIXED)
    _, d64, o64, _ = run(gpu, w, 200, abi.F8_FP64)
    assert drag_rel(dm, d64) <= DRAG_TOL
    assert rel_l2(interior(om["u"]), interior(o64["u"])) <= VEL_TOL


def test_mixed_newtonian_no_ibm(gpu, oracle):
    w = configs.scaled(configs.c2_3d(), 16, 16, 16)
    w = replace(w, cyls=(), phys=replace(w.phys, beta=1.0))
    _, _, om, diag = run(gpu, w, 20, abi.F8_MIXED)
    _, _, oo, _ = run(oracle, w, 20, abi.F8_FP64)
    for f in ("u", "v", "w"):
        assert rel_l2(interior(om[f]), interior(oo[f])) <= VEL_TOL, f


def test_mixed_2d_rejects_sor(gpu):
    """The 2D mixed step solves its pressure with the FFT solvers only."""
    w = configs.scaled(configs.c1_2d(), 32, 32, 1)
    with pytest.raises(F8Error) as err:
        Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED, poisson=abi.F8_POISSON_SOR)
    assert err.value.status == abi.F8_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", [abi.F8_MIXED, abi.F8_FP64])
def test_nan_velocity_reported(gpu, precision):
    """A NaN in the loaded velocity ends the call with F8_ERR_NAN (the
    reference's 'NaN value' stop, fenep_2d.f90:1974) instead of running on."""
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    st0 = configs.initial_state(w)
    st0.arrays["u"][5, 6, 7] = np.nan
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=precision) as s:
        s.load(st0)
        with pytest.raises(F8Error) as exc:
            s.step(2)
        assert exc.value.status == abi.F8_ERR_NAN


@pytest.mark.parametrize("shape", [(32, 512, 64), (16, 256, 256)])
def test_mixed_cluster_plane_matches_fp64(gpu, shape):
    """Channels whose (z, y) plane is split over a thread-block cluster (2 CTAs
    for 512 x 64, 4 CTAs for 256 x 256, the 512x256x256 configuration's
    plane) against the FP64 step: fields after 10 steps (no cylinders, the
    IBM needs dX = dY)."""
    w = replace(configs.scaled(configs.c3_channel(), *shape), cyls=())
    sm, _, om, _ = run(gpu, w, 10, abi.F8_MIXED)
    s6, _, o6, _ = run(gpu, w, 10, abi.F8_FP64)
    assert sm == abi.F8_OK and s6 == abi.F8_OK
    for f in ("u", "v", "w"):
        assert rel_l2(interior(om[f]), interior(o6[f])) <= VEL_TOL, f
    pm, p6 = interior(om["p"]), interior(o6["p"])
    assert rel_l2(pm - pm.mean(), p6 - p6.mean()) <= 1e-4


def test_mixed_sor_variant_matches_fp64_sor(gpu):
    """The red-black SOR pressure variant (omega 1.8) of the mixed step against
    the FP64 step's SOR at a common tolerance: both stop at
    sqrt(sum E^2 / sum R^2) < 1e-6, so they agree to that level."""
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    w = replace(w, phys=replace(w.phys, sor_eps=1e-6, sor_itrmax=20000))
    out = {}
    for prec in (abi.F8_MIXED, abi.F8_FP64):
        with Solver(gpu, w.grid, w.phys, w.cyls, precision=prec, poisson=abi.F8_POISSON_SOR) as s:
            s.load(configs.initial_state(w))
            st, drag = s.step(3)
            dg = s.diagnostics()
            out[prec] = (st, drag, s.store(), dg)
    (sm, dm, om, gm), (s6, d6, o6, g6) = out[abi.F8_MIXED], out[abi.F8_FP64]
    assert sm == abi.F8_OK and s6 == abi.F8_OK
    assert 0 < gm.poisson_iters <= 20000 and 0 < g6.poisson_iters <= 20000
    for f in ("u", "v", "w"):
        assert rel_l2(interior(om[f]), interior(o6[f])) <= 1e-5, f
    assert drag_rel(dm, d6) <= 1e-4


def test_graph_replay_is_bit_identical(gpu):
    """The mixed step replays CUDA graphs when no stage timing is requested;
    the state and drag equal the directly launched step bit for bit."""
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    res = []
    for timing in (True, False):
        with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
            s.set_timing(timing)
            s.load(configs.initial_state(w))
            _, d1 = s.step(3)        # the first step (AB2 start) is never replayed
            _, d2 = s.step(4)        # odd and even buffer parities
            st = s.store()
            res.append((np.concatenate([d1, d2]), st, s.diagnostics().kernel_launches))
    (da, sa, la), (db, sb, lb) = res
    np.testing.assert_array_equal(da, db)
    for f in ("u", "v", "w", "p", "c"):
        np.testing.assert_array_equal(sa[f], sb[f])
    assert la == lb   # replayed kernels are counted as launches


@pytest.mark.parametrize("second", ["uniform", "varying"])
def test_reload_with_another_force_recaptures_the_graphs(gpu, second):
    """A uniform body force is a kernel argument of the replayed step graphs:
    reloading a context with another force (another uniform value, or a
    varying field) gives the same steps as a fresh context."""
    w = configs.scaled(configs.c3_channel(), 32, 16, 16)
    st_a = configs.initial_state(w)
    st_b = st_a.copy()
    if second == "uniform":
        st_b.arrays["fx"] = np.full_like(st_a.arrays["fx"], 2.0 * st_a.arrays["fx"].flat[0])
    else:
        fx = st_a.arrays["fx"].copy()
        fx[..., : fx.shape[-1] // 2] *= 1.5
        st_b.arrays["fx"] = fx
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(st_a)
        s.step(4)                 # graphs captured with the first force
        s.load(st_b)
        _, d_reload = s.step(4)
        out_reload = s.store()
    with Solver(gpu, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as s:
        s.load(st_b)
        _, d_fresh = s.step(4)
        out_fresh = s.store()
    np.testing.assert_array_equal(d_reload, d_fresh)
    for f in ("u", "v", "w", "p", "c"):
        np.testing.assert_array_equal(out_reload[f], out_fresh[f])
