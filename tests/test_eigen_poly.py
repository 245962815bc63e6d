"""The smallest-eigenvalue root of the FP32 eigen test (f8_step_mixed.cu, two_t2).

The mixed step evaluates t(r) = cos(acos(r)/3 + 2 pi/3), the smallest root of
4t^3 - 3t = r, as a degree-7 polynomial in u = sqrt(1 - r) on [0, sqrt 2].  This
test reads the coefficients from the kernel source and checks that

* they are 2x the monomial form of the polynomial interpolating t at the 8
  Chebyshev points of [0, sqrt 2] (the construction the source describes);
* the bounds the source states: the interpolant of t is within 2.7e-8 of t;
  the FP32 coefficients of 2t are within 1.1e-7 of 2t evaluated in FP64 and
  within 2.2e-7 in FP32 Horner form (on FP32 arguments);
* the endpoints are the repeated-root limits t(r=1) = -1/2 and t(r=-1) = -1.
"""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
from numpy.polynomial import chebyshev as Ch
from numpy.polynomial import polynomial as P

SRC = Path(__file__).resolve().parents[1] / "fortran8_gb300" / "csrc" / "f8_step_mixed.cu"
U_MAX = np.sqrt(2.0)


def source_coefficients() -> np.ndarray:
    """Monomial coefficients (degree 0 first) of two_t2 in the kernel source."""
    text = SRC.read_text()
    body = text[text.index("float2 two_t2(float2 u)"):]
    body = body[: body.index("\n}\n")]
    nums = [float(x) for x in re.findall(r"f2\((-?[0-9.]+(?:e-?[0-9]+)?)f\)", body)]
    assert len(nums) == 8, nums
    return np.array(nums[::-1])   # Horner order is highest degree first


def t_exact(u):
    r = 1.0 - np.asarray(u, dtype=np.float64) ** 2
    return np.cos((np.arccos(np.clip(r, -1.0, 1.0)) + 2.0 * np.pi) / 3.0)


def test_coefficients_are_the_chebyshev_interpolant():
    c = source_coefficients()
    fit = 2.0 * Ch.Chebyshev.interpolate(t_exact, 7, domain=[0.0, U_MAX]).convert(
        kind=P.Polynomial, domain=[0.0, U_MAX], window=[0.0, U_MAX]).coef
    assert np.allclose(c, fit.astype(np.float32), rtol=2e-7, atol=0.0), (c, fit)


def test_error_bounds_fp64_and_fp32():
    c = source_coefficients()
    u64 = np.linspace(0.0, U_MAX, 200001)
    interp = Ch.Chebyshev.interpolate(t_exact, 7, domain=[0.0, U_MAX])
    assert np.max(np.abs(interp(u64) - t_exact(u64))) <= 2.7e-8
    assert np.max(np.abs(P.polyval(u64, c) - 2.0 * t_exact(u64))) <= 1.1e-7
    u32 = u64.astype(np.float32)
    acc = np.full_like(u32, np.float32(c[-1]))
    for a in c[-2::-1]:
        acc = (acc * u32 + np.float32(a)).astype(np.float32)
    err = np.max(np.abs(acc.astype(np.float64) - 2.0 * t_exact(u32.astype(np.float64))))
    assert err <= 2.2e-7, err


def test_endpoints_are_the_repeated_root_limits():
    c = source_coefficients()
    assert abs(P.polyval(0.0, c) - (-1.0)) <= 1e-7            # r = 1: t = -1/2, 2t = -1
    assert abs(P.polyval(U_MAX, c) - (-2.0)) <= 1e-7          # r = -1: t = -1, 2t = -2
