"""ctypes mirror of include/f8.h.

One binding class serves both implementations of the ABI: the CUDA library
(symbols ``f8_*``) and the CPU oracle used by the tests (symbols ``f8o_*``).
The struct layouts must match include/f8.h field for field.
"""
from __future__ import annotations

import ctypes as C

F8_OK = 0
F8_ERR_ARG = 1
F8_ERR_STATE = 2
F8_ERR_NOMEM = 3
F8_ERR_CUDA = 4
F8_ERR_NAN = 5
F8_ERR_UNSUPPORTED = 6
F8_ERR_NO_DEVICE = 7
F8_ERR_TOO_LARGE = 8
F8_WARN_NEWTON = 16
F8_WARN_SOR = 17

F8_FP64 = 0
F8_MIXED = 1
F8_POISSON_FFT = 0
F8_POISSON_SOR = 1
F8_BC_PERIODIC = 0
F8_BC_WALLS = 1
F8_BC_WALLS_Z = 2
F8_IBM_CELL_VOLUME = 0
F8_IBM_ARC_VOLUME = 1
F8_EIGEN_VIETA = 0
F8_EIGEN_CARDANO = 1
F8_EIGEN_SYLVESTER = 2
F8_EIGEN_SYMMETRIC = 3

_dp = C.POINTER(C.c_double)


class Grid(C.Structure):
    _fields_ = [("dim", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("bc_y", C.c_int), ("uwall", C.c_double)]


class Phys(C.Structure):
    _fields_ = [("re", C.c_double), ("wi", C.c_double), ("beta", C.c_double),
                ("lp2", C.c_double), ("dt", C.c_double),
                ("newton_dc", C.c_double), ("newton_eps", C.c_double), ("newton_itrmax", C.c_int),
                ("sor_omega", C.c_double), ("sor_eps", C.c_double), ("sor_itrmax", C.c_int),
                ("ab2_start", C.c_int), ("ibm_volume", C.c_int), ("ibm_repeats", C.c_int),
                ("eigen_test", C.c_int)]


class Cyl(C.Structure):
    _fields_ = [("xc", C.c_double), ("yc", C.c_double), ("r", C.c_double),
                ("spin", C.c_double), ("filled", C.c_int)]


FIELD_NAMES = ("u", "v", "w", "p", "phi", "c", "ax0", "ay0", "az0",
               "tx0", "ty0", "tz0", "fx", "fy", "fz")


class Fields(C.Structure):
    _fields_ = [(n, _dp) for n in FIELD_NAMES]


class Turb(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("k_energy", "k_staggered", "lambda_", "re_lambda", "epsilon",
                                          "l_kolmogorov", "t_kolmogorov", "u_kolmogorov", "ep_energy",
                                          "trc_mean", "trc_std")]


class Diag(C.Structure):
    _fields_ = [("step", C.c_int), ("ke", C.c_double), ("cfl", C.c_double),
                ("trc_min", C.c_double), ("trc_max", C.c_double), ("trc_mean", C.c_double),
                ("div_max", C.c_double), ("newton_iters", C.c_longlong),
                ("newton_unconverged", C.c_longlong), ("poisson_iters", C.c_int),
                ("nan_found", C.c_int), ("kernel_launches", C.c_longlong), ("trc_std", C.c_double)]


# Entry points declared in include/f8.h (without prefix).
ABI_FUNCTIONS = {
    "create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(Grid), C.POINTER(Phys),
                         C.POINTER(Cyl), C.c_int, C.c_int, C.c_int]),
    "load": (C.c_int, [C.c_void_p, C.POINTER(Fields), C.c_int]),
    "step": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "store": (C.c_int, [C.c_void_p, C.POINTER(Fields)]),
    "diagnostics": (C.c_int, [C.c_void_p, C.POINTER(Diag)]),
    "markers": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), _dp]),
    "selection_codes": (C.c_int, [C.c_void_p, C.c_void_p]),
    "slice": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "turbulence": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_void_p]),
    "spectrum": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "stats_begin": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int]),
    "stats_read": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, C.POINTER(C.c_int)]),
    "strerror": (C.c_char_p, [C.c_int]),
    "destroy": (None, [C.c_void_p]),
    "default_phys": (None, [C.POINTER(Phys)]),
    "set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "timing": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_longlong)]),
    "timing_reset": (C.c_int, [C.c_void_p]),
    "kernel_timing": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_longlong)]),
    "fft_solve": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                            C.c_void_p, C.c_void_p, C.c_double, C.c_double]),
}

# Entry points of the CUDA library only (the oracle has no adjoint).
GPU_FUNCTIONS = {
    "grad": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.POINTER(Fields), _dp, _dp,
                       C.POINTER(Fields), _dp]),
}

NSTAGE = 7
STAGE_NAMES = ("eigen", "newton", "momentum", "ibm", "helmholtz", "poisson", "project")
NKERNEL = 6
KERNEL_NAMES = ("k_codes3_f", "k_update3_f", "k_momentum3_f", "k_poisson_rhs_df", "k_defect_df", "k_march_df")


def bind(lib: C.CDLL, prefix: str) -> dict:
    """Resolve every ABI entry point of ``lib`` under ``prefix`` (``f8_`` or ``f8o_``)."""
    out = {}
    for name, (res, args) in ABI_FUNCTIONS.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
        out[name] = fn
    for name, (res, args) in GPU_FUNCTIONS.items():
        fn = getattr(lib, prefix + name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
        out[name] = fn
    return out
