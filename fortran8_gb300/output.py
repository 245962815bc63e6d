"""File formats of the reference's output and restart routines.

* Slices (``get_data_binary``, fenep.f90:1108-1183; fenep_mpi.f90:811-937):
  stream-access binary files ``z_########.bin`` (x-y plane k = NZ/2),
  ``y_########.bin`` (x-z plane j = NY/2) and, for the MPI program,
  ``x_########.bin`` (y-z plane i = NX/2), 18 float64 per point in the
  reference's loop order, as ``_map.py`` reads them
  (``np.fromfile(f, np.float64).reshape(-1, 18)``).  The records are computed
  on the device by ``Solver.slice``.
* Restart text ``Restart.d`` (``output`` / ``input``, fenep.f90:1186-1233):
  one list-directed line per interior cell, k outer, i inner:
  U V W P C(1:6) Ax Ay Az Tx Ty Tz.  Written with 17 significant digits so
  that a read restores every double.
* Restart binary ``Restart/########.bin`` per MPI rank (``output_binary`` /
  ``input_binary``, fenep_mpi.f90:939-992): Fortran sequential unformatted,
  one record per interior cell of the rank's z-slab (NZ / nranks planes), the
  same 16 doubles, each record framed by 4-byte little-endian length markers
  (gfortran's default).

The restart files carry the interior only; the halo values are re-applied by
``f8_load`` (the reference calls PBM after reading, fenep.f90:1209-1212).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .solver import GridSpec, State, empty_state

RESTART_COLUMNS = 16  # U V W P C1..C6 Ax Ay Az Tx Ty Tz


def write_slices(solver, directory, step: int, variant: int = 0):
    """Write the slice files of step ``step`` into ``directory``.

    variant 0: fenep.f90 (z and y slices, column 7 = KE); variant 1:
    fenep_mpi.f90 (z, y and x slices, column 7 = Q).  Returns the paths."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    axes = {"z": 2, "y": 1} if variant == 0 else {"z": 2, "y": 1, "x": 0}
    paths = []
    for name, axis in axes.items():
        p = d / f"{name}_{step:08d}.bin"
        solver.slice(axis, variant).astype("<f8").tofile(p)
        paths.append(p)
    return paths


def read_slice(path) -> np.ndarray:
    """The (points, 18) records of a slice file (the reader of ``_map.py``)."""
    return np.fromfile(path, dtype="<f8").reshape(-1, 18)


def _restart_matrix(st: State, g: GridSpec) -> np.ndarray:
    """(cells, 16) in the reference's loop order (k outer, j, i inner)."""
    if g.dim != 3:
        raise ValueError("the Restart formats are those of the 3D programs")
    it = (slice(1, -1),) * 3
    cols = [st["u"][it], st["v"][it], st["w"][it], st["p"][it]]
    cols += [st["c"][it + (m,)] for m in range(6)]
    cols += [st[n] for n in ("ax0", "ay0", "az0", "tx0", "ty0", "tz0")]
    return np.stack([c.reshape(-1) for c in cols], axis=1)


def _state_from_matrix(m: np.ndarray, g: GridSpec, like: State | None = None) -> State:
    st = empty_state(g) if like is None else like.copy()
    shp = g.interior_shape
    it = (slice(1, -1),) * 3
    for q, n in enumerate(("u", "v", "w", "p")):
        st.arrays[n][it] = m[:, q].reshape(shp)
    for c in range(6):
        st.arrays["c"][it + (c,)] = m[:, 4 + c].reshape(shp)
    for q, n in enumerate(("ax0", "ay0", "az0", "tx0", "ty0", "tz0")):
        st.arrays[n][...] = m[:, 10 + q].reshape(shp)
    return st


def write_restart_text(st: State, g: GridSpec, path) -> Path:
    """Restart.d of fenep.f90's ``output``."""
    m = _restart_matrix(st, g)
    np.savetxt(path, m, fmt="%.17E")
    return Path(path)


def read_restart_text(path, g: GridSpec, like: State | None = None) -> State:
    """State from Restart.d (fenep.f90's ``input``); fields not in the file
    (F, Phi) are taken from ``like`` or zero."""
    m = np.loadtxt(path, dtype=np.float64, ndmin=2)
    if m.shape != (g.cells, RESTART_COLUMNS):
        raise ValueError(f"Restart.d holds {m.shape}, expected ({g.cells}, {RESTART_COLUMNS})")
    return _state_from_matrix(m, g, like)


_REC = np.dtype([("head", "<i4"), ("v", "<f8", (RESTART_COLUMNS,)), ("tail", "<i4")])


def write_restart_binary(st: State, g: GridSpec, directory, nranks: int = 1):
    """Restart/########.bin of fenep_mpi.f90's ``output_binary`` for ``nranks``
    z-slabs of NZ / nranks planes."""
    if g.nz % nranks:
        raise ValueError("NZ must be a multiple of the rank count (fenep_mpi.f90:82)")
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    m = _restart_matrix(st, g)
    per = g.nx * g.ny * (g.nz // nranks)
    paths = []
    for r in range(nranks):
        rec = np.zeros(per, dtype=_REC)
        rec["head"] = rec["tail"] = RESTART_COLUMNS * 8
        rec["v"] = m[r * per:(r + 1) * per]
        p = d / f"{r:08d}.bin"
        rec.tofile(p)
        paths.append(p)
    return paths


def read_restart_binary(directory, g: GridSpec, nranks: int = 1, like: State | None = None) -> State:
    """State from the per-rank files of ``output_binary`` (fenep_mpi.f90's
    ``input_binary``)."""
    if g.nz % nranks:
        raise ValueError("NZ must be a multiple of the rank count (fenep_mpi.f90:82)")
    parts = []
    for r in range(nranks):
        rec = np.fromfile(Path(directory) / f"{r:08d}.bin", dtype=_REC)
        if rec.size != g.nx * g.ny * (g.nz // nranks) or np.any(rec["head"] != RESTART_COLUMNS * 8) \
                or np.any(rec["tail"] != RESTART_COLUMNS * 8):
            raise ValueError(f"rank file {r} is not a sequential record file of {RESTART_COLUMNS} doubles")
        parts.append(rec["v"])
    return _state_from_matrix(np.concatenate(parts), g, like)
