"""Slice output and restart formats (the reference's get_data_binary, output /
input and output_binary / input_binary), checked on the CPU oracle."""
from __future__ import annotations

import numpy as np
import pytest

from fortran8_gb300 import abi, configs, output
from fortran8_gb300.solver import Solver


def numpy_slice(st, g, axis, variant):
    """Independent restatement of get_data_binary's records (fenep.f90:1116-1149)
    from the stored arrays (C-ordered (k, j, i) halo fields, U_C = L_C = 1)."""
    U, V, W, C = st["u"], st["v"], st["w"], st["c"]
    dX, dY, dZ = g.lx / g.nx, g.ly / g.ny, g.lz / g.nz
    pts = []
    if axis == 2:
        idx = [(i, j, g.nz // 2) for j in range(1, g.ny + 1) for i in range(1, g.nx + 1)]
    elif axis == 1:
        idx = [(i, g.ny // 2, k) for k in range(1, g.nz + 1) for i in range(1, g.nx + 1)]
    else:
        idx = [(g.nx // 2, j, k) for k in range(1, g.nz + 1) for j in range(1, g.ny + 1)]
    for i, j, k in idx:
        u = lambda a, b, c: U[c, b, a]
        v = lambda a, b, c: V[c, b, a]
        w = lambda a, b, c: W[c, b, a]
        D = np.zeros((3, 3))
        D[0, 0] = (u(i, j, k) - u(i - 1, j, k)) / dX
        D[0, 1] = (u(i, j + 1, k) - u(i, j - 1, k) + u(i - 1, j + 1, k) - u(i - 1, j - 1, k)) / (4 * dY)
        D[0, 2] = (u(i, j, k + 1) - u(i, j, k - 1) + u(i - 1, j, k + 1) - u(i - 1, j, k - 1)) / (4 * dZ)
        D[1, 0] = (v(i + 1, j, k) - v(i - 1, j, k) + v(i + 1, j - 1, k) - v(i - 1, j - 1, k)) / (4 * dX)
        D[1, 1] = (v(i, j, k) - v(i, j - 1, k)) / dY
        D[1, 2] = (v(i, j, k + 1) - v(i, j, k - 1) + v(i, j - 1, k + 1) - v(i, j - 1, k - 1)) / (4 * dZ)
        D[2, 0] = (w(i + 1, j, k) - w(i - 1, j, k) + w(i + 1, j, k - 1) - w(i - 1, j, k - 1)) / (4 * dX)
        D[2, 1] = (w(i, j + 1, k) - w(i, j - 1, k) + w(i, j + 1, k - 1) - w(i, j - 1, k - 1)) / (4 * dY)
        D[2, 2] = (w(i, j, k) - w(i, j, k - 1)) / dZ
        E = np.array([(u(i - 1, j, k) + u(i, j, k)) / 2, (v(i, j - 1, k) + v(i, j, k)) / 2,
                      (w(i, j, k - 1) + w(i, j, k)) / 2])
        Om = np.array([D[2, 1] - D[1, 2], D[0, 2] - D[2, 0], D[1, 0] - D[0, 1]])
        Q = (D[1, 1] * D[2, 2] - D[2, 1] * D[1, 2] + D[0, 0] * D[1, 1] - D[1, 0] * D[0, 1]
             + D[0, 0] * D[2, 2] - D[2, 0] * D[0, 2])
        c = C[k, j, i]
        pts.append([(i - 0.5) * dX, (j - 0.5) * dY, (k - 0.5) * dZ, *E, Q if variant else (E @ E) / 2,
                    *Om, (Om @ Om) / 2, c[0] + c[3] + c[5], *c])
    return np.array(pts)


def stepped(oracle, steps=3):
    w = configs.scaled(configs.c3_channel(), 16, 8, 8)
    s = Solver(oracle, w.grid, w.phys, w.cyls)
    s.load(configs.initial_state(w))
    s.step(steps)
    return w, s


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("variant", [0, 1])
def test_oracle_slice_matches_restatement(oracle, axis, variant):
    w, s = stepped(oracle)
    with s:
        got = s.slice(axis, variant)
        ref = numpy_slice(s.store(), w.grid, axis, variant)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13)


def test_slice_files_round_trip(oracle, tmp_path):
    w, s = stepped(oracle)
    with s:
        paths = output.write_slices(s, tmp_path, 123, variant=1)
        assert [p.name for p in paths] == ["z_00000123.bin", "y_00000123.bin", "x_00000123.bin"]
        for p, axis in zip(paths, (2, 1, 0)):
            data = output.read_slice(p)
            assert p.stat().st_size == data.size * 8
            np.testing.assert_array_equal(data, s.slice(axis, 1))


def test_restart_text_resumes_bit_identically(oracle, tmp_path):
    w, s = stepped(oracle)
    with s:
        st = s.store()
        p = output.write_restart_text(st, w.grid, tmp_path / "Restart.d")
        lines = p.read_text().splitlines()
        assert len(lines) == w.grid.cells and len(lines[0].split()) == output.RESTART_COLUMNS
        back = output.read_restart_text(p, w.grid, like=st)
        for n in ("u", "v", "w", "p", "c", "ax0", "az0", "tx0", "tz0"):
            a, b = st[n], back[n]
            if a.shape == w.grid.interior_shape:
                np.testing.assert_array_equal(a, b)
            else:
                np.testing.assert_array_equal(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1])
        _, d_cont = s.step(2)
    with Solver(oracle, w.grid, w.phys, w.cyls) as r:
        r.load(back, step0=3)   # input_type > 0: no AB2 start rule
        _, d_rest = r.step(2)
    np.testing.assert_array_equal(d_cont, d_rest)


@pytest.mark.parametrize("nranks", [1, 2, 4])
def test_restart_binary_per_rank(oracle, tmp_path, nranks):
    w, s = stepped(oracle)
    with s:
        st = s.store()
    paths = output.write_restart_binary(st, w.grid, tmp_path / "Restart", nranks)
    per = w.grid.nx * w.grid.ny * (w.grid.nz // nranks)
    for p in paths:
        raw = np.fromfile(p, dtype=np.uint8)
        assert raw.size == per * (16 * 8 + 8)
        # Fortran sequential records: 4-byte length, 16 doubles, 4-byte length
        assert np.frombuffer(raw[:4].tobytes(), "<i4")[0] == 128
    back = output.read_restart_binary(tmp_path / "Restart", w.grid, nranks, like=st)
    it = (slice(1, -1),) * 3
    for n in ("u", "v", "w", "p"):
        np.testing.assert_array_equal(st[n][it], back[n][it])
    np.testing.assert_array_equal(st["tz0"], back["tz0"])
    with pytest.raises(ValueError):
        output.read_restart_binary(tmp_path / "Restart", w.grid, 2 * nranks if nranks < 4 else 3, like=st)
