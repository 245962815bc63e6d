"""Host-side wrapper of the f8 C ABI for Python tooling.

``Solver`` drives any library that exports the ABI of include/f8.h: the CUDA
library (prefix ``f8_``) or, in tests only, the CPU oracle (prefix ``f8o_``).
Arrays are numpy arrays in the reference's memory layout: a halo field of the
Fortran shape (0:NX+1, 0:NY+1, 0:NZ+1) is held as a C-ordered array of shape
(NZ+2, NY+2, NX+2); the conformation tensor C(NC, 0:NX+1, ...) as
(NZ+2, NY+2, NX+2, NC); interior fields (1:NX, 1:NY, 1:NZ) as (NZ, NY, NX).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

HALO_FIELDS = ("u", "v", "w", "p", "phi")
INTERIOR_FIELDS = ("ax0", "ay0", "az0", "tx0", "ty0", "tz0", "fx", "fy", "fz")


class F8Error(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"f8 status {status}: {msg}")
        self.status = status


@dataclass
class GridSpec:
    dim: int
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    bc_y: int = abi.F8_BC_PERIODIC
    uwall: float = 0.0

    def to_c(self) -> abi.Grid:
        return abi.Grid(self.dim, self.nx, self.ny, self.nz, self.lx, self.ly, self.lz,
                        self.bc_y, self.uwall)

    @property
    def ncomp(self) -> int:
        return 6 if self.dim == 3 else 3

    @property
    def halo_shape(self):
        return (self.nz + 2, self.ny + 2, self.nx + 2)

    @property
    def interior_shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz


@dataclass
class PhysSpec:
    re: float
    wi: float
    beta: float
    lp2: float
    dt: float
    newton_dc: float = 1.0e-5
    newton_eps: float = 1.0e-6
    newton_itrmax: int = 10000
    sor_omega: float = 1.8
    sor_eps: float = 1.0e-5
    sor_itrmax: int = 10000
    ab2_start: int = 1
    ibm_volume: int = abi.F8_IBM_CELL_VOLUME
    ibm_repeats: int = 1
    eigen_test: int = abi.F8_EIGEN_VIETA

    def to_c(self) -> abi.Phys:
        return abi.Phys(self.re, self.wi, self.beta, self.lp2, self.dt, self.newton_dc,
                        self.newton_eps, self.newton_itrmax, self.sor_omega, self.sor_eps,
                        self.sor_itrmax, self.ab2_start, self.ibm_volume, self.ibm_repeats, self.eigen_test)


@dataclass
class CylSpec:
    xc: float
    yc: float
    r: float
    spin: float = 0.0
    filled: int = 1


@dataclass
class State:
    """A full solver state in the reference layouts (see module docstring)."""
    arrays: dict = field(default_factory=dict)

    def copy(self) -> "State":
        return State({k: v.copy() for k, v in self.arrays.items()})

    def __getitem__(self, k):
        return self.arrays[k]


def empty_state(g: GridSpec) -> State:
    a = {n: np.zeros(g.halo_shape) for n in HALO_FIELDS}
    a["c"] = np.zeros(g.halo_shape + (g.ncomp,))
    for n in INTERIOR_FIELDS:
        a[n] = np.zeros(g.interior_shape)
    return State(a)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fields_struct(st: State) -> abi.Fields:
    f = abi.Fields()
    for n in abi.FIELD_NAMES:
        arr = st.arrays.get(n)
        setattr(f, n, _ptr(arr) if arr is not None else None)
    return f


class Solver:
    """One solver context of an f8 ABI library."""

    def __init__(self, fns: dict, grid: GridSpec, phys: PhysSpec, cyls=(),
                 precision: int = abi.F8_FP64, poisson: int = abi.F8_POISSON_FFT):
        self._fns = fns
        self.grid = grid
        self.phys = phys
        self.cyls = list(cyls)
        self._cg = grid.to_c()
        self._cp = phys.to_c()
        n = len(self.cyls)
        self._cc = (abi.Cyl * max(n, 1))(*[abi.Cyl(c.xc, c.yc, c.r, c.spin, c.filled) for c in self.cyls])
        h = C.c_void_p()
        st = fns["create"](C.byref(h), C.byref(self._cg), C.byref(self._cp),
                           self._cc if n else None, n, precision, poisson)
        self._check(st)
        self._h = h

    def _check(self, st: int, allow_warn: bool = True) -> int:
        if st == abi.F8_OK:
            return st
        if allow_warn and st >= 16:
            return st
        raise F8Error(st, self._fns["strerror"](st).decode())

    @property
    def handle(self):
        return self._h

    def load(self, st: State, step0: int = 0) -> None:
        self._keep = st  # the library copies during the call; keep alive anyway
        f = _fields_struct(st)
        self._check(self._fns["load"](self._h, C.byref(f), step0))

    def step(self, nsteps: int = 1, want_drag: bool = True):
        """Advance; returns (status, drag array of shape (nsteps, ncyl, 3) or None)."""
        n = len(self.cyls)
        drag = np.zeros((nsteps, max(n, 1), 3)) if (want_drag and n) else None
        st = self._fns["step"](self._h, nsteps, _ptr(drag) if drag is not None else None)
        self._check(st)
        return st, (drag[:, :n] if drag is not None else None)

    def grad(self, nsteps: int, checkpoint_every: int = 0, weights=None, seed: State | None = None,
             want_dstate: bool = False):
        """f8_grad: advance nsteps and return the gradient of
        J = sum(weights * drag) + <seed, final state>.

        Returns (status, J (drag term), dparams [dWi, dbeta, dL2, dxc0, dyc0, ...],
        dstate State or None, drag history (nsteps, ncyl, 3))."""
        n = len(self.cyls)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(np.broadcast_to(np.asarray(weights, dtype=np.float64), (nsteps, n, 3)))
        jv = C.c_double()
        dp = np.zeros(3 + 2 * n)
        drag = np.zeros((nsteps, max(n, 1), 3))
        sf = _fields_struct(seed) if seed is not None else None
        out = empty_state(self.grid) if want_dstate else None
        of = _fields_struct(out) if out is not None else None
        st = self._fns["grad"](self._h, nsteps, checkpoint_every, _ptr(w) if w is not None else None,
                               C.byref(sf) if sf is not None else None, C.byref(jv), _ptr(dp),
                               C.byref(of) if of is not None else None, _ptr(drag))
        self._check(st)
        return st, jv.value, dp, out, drag[:, :n]

    def store(self, out: State | None = None) -> State:
        """Copy the state out; into ``out``'s arrays when given (e.g. page-locked
        buffers reused across calls), else into new arrays."""
        if out is None:
            out = empty_state(self.grid)
        f = _fields_struct(out)
        self._check(self._fns["store"](self._h, C.byref(f)))
        return out

    def diagnostics(self) -> abi.Diag:
        d = abi.Diag()
        self._check(self._fns["diagnostics"](self._h, C.byref(d)))
        return d

    def slice(self, axis: int = 2, variant: int = 0) -> np.ndarray:
        """Mid-plane slice records of get_data_binary, shape (points, 18) (see f8_slice)."""
        g = self.grid
        n = {2: g.nx * g.ny, 1: g.nx * g.nz, 0: g.ny * g.nz}[axis]
        out = np.zeros((n, 18))
        self._check(self._fns["slice"](self._h, axis, variant, _ptr(out)))
        return out

    def _means(self, mean):
        if mean is None:
            return (None, None, None), None
        arrs = [np.ascontiguousarray(m, dtype=np.float64) for m in mean]
        return tuple(_ptr(a) for a in arrs), arrs

    def turbulence(self, mean=None) -> abi.Turb:
        """all_time_dif statistics; mean = (U, V, W) interior mean fields or None."""
        ptrs, keep = self._means(mean)
        t = abi.Turb()
        self._check(self._fns["turbulence"](self._h, *ptrs, C.byref(t)))
        del keep
        return t

    def spectrum(self, mean=None) -> np.ndarray:
        """Shell-binned energy spectrum E[0..NX] of energy_single."""
        ptrs, keep = self._means(mean)
        e = np.zeros(self.grid.nx + 1)
        self._check(self._fns["spectrum"](self._h, *ptrs, _ptr(e)))
        del keep
        return e

    def stats_begin(self, mode: int, mean=None, max_steps: int = 0) -> None:
        """Start the running statistics of f8_stats_begin (mode 1: sums and probes,
        mode 2: squared fluctuations about mean = (U, V, W), 0: stop)."""
        ptrs, keep = self._means(mean)
        self._check(self._fns["stats_begin"](self._h, mode, *ptrs, max_steps))
        del keep

    def stats_read(self, max_steps: int = 0):
        """(sums: three interior fields, probes: (3, steps, NZ) or None, steps)."""
        g = self.grid
        sums = [np.zeros(g.interior_shape) for _ in range(3)]
        n = C.c_int()
        self._check(self._fns["stats_read"](self._h, *(_ptr(a) for a in sums), None, C.byref(n)))
        probes = None
        if max_steps:
            m = min(n.value, max_steps)
            probes = np.zeros((3, m, g.nz))
            self._check(self._fns["stats_read"](self._h, None, None, None, _ptr(probes), C.byref(n)))
        return sums, probes, n.value

    def selection_codes(self) -> np.ndarray:
        """SPD candidate choices of the last step (f8_selection_codes), shape
        (NZ, rows, NX) uint8; rows = NY + 2 with walls, else NY."""
        g = self.grid
        rows = g.ny + 2 if g.bc_y == abi.F8_BC_WALLS else g.ny
        out = np.zeros((g.nz, rows, g.nx), dtype=np.uint8)
        self._check(self._fns["selection_codes"](self._h, out.ctypes.data))
        return out

    def markers(self) -> np.ndarray:
        n = C.c_int()
        self._check(self._fns["markers"](self._h, C.byref(n), None))
        xy = np.zeros((max(n.value, 1), 2))
        self._check(self._fns["markers"](self._h, C.byref(n), _ptr(xy)))
        return xy[: n.value]

    def set_timing(self, on: bool = True) -> None:
        self._check(self._fns["set_timing"](self._h, 1 if on else 0))

    def timing(self):
        """(total ms of the f8_step calls, per-stage ms array, steps timed)."""
        tot = C.c_double()
        st = np.zeros(abi.NSTAGE)
        n = C.c_longlong()
        self._check(self._fns["timing"](self._h, C.byref(tot), _ptr(st), C.byref(n)))
        return tot.value, st, n.value

    def kernel_timing(self):
        """(per-kernel ms array over abi.KERNEL_NAMES, steps covered) of the
        mixed step's single-launch kernels (f8_kernel_timing)."""
        ms = np.zeros(abi.NKERNEL)
        n = C.c_longlong()
        self._check(self._fns["kernel_timing"](self._h, _ptr(ms), C.byref(n)))
        return ms, n.value

    def timing_reset(self) -> None:
        self._check(self._fns["timing_reset"](self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._fns["destroy"](self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
