"""Host-side planning of the GPU library, on the CPU: the shared-memory layout
of the wall-plane solve (the bank model of f8_common.cuh) and the plan of the
mixed gradient's kept tapes.

A small C++ program includes the library's header (host functions only, no
CUDA call) and prints the decisions for the shapes the library meets:

* wall_layout fits its shared-memory limit, covers every row of a system
  (T threads x L rows >= R), has an odd tile stride, and costs no more bank
  wavefronts than the compact layout; on the 256 x 128 x 128 channel it picks
  the 133 / 133 / 19 layout; a plane too large for one CTA gets none;
* wall_plane_cluster gives one CTA per plane for NY = 128, NZ = 128 and four
  for NY = 256, NZ = 256 (the 512 x 256 x 256 channel);
* kept_segments returns the largest R that fits, every segment when all fit,
  one when none does, and grows with the memory available.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "fortran8_gb300" / "csrc"

HARNESS = r"""
#include <cstdio>
#include "f8_common.cuh"
using namespace f8;

int main() {
    const size_t limit = 227 * 1024;
    // wall layouts: R rows of a system, T threads per system, NZ
    const int cases[][3] = {{130, 8, 128}, {66, 16, 64}, {34, 32, 32}, {65, 4, 256}, {258, 8, 128}};
    for (auto &cz : cases) {
        const int R = cz[0], T = cz[1], nz = cz[2];
        const WallLayout wl = wall_layout(R, T, nz, limit);
        const long c = wl.ps > 0 ? wl_cost(R, T, wl.ps, wl.rs, wl.L) : -1;
        const long c0 = wl_cost(R, T, R | 1, R, (R + T - 1) / T);
        std::printf("layout %d %d %d %d %d %d %ld %ld %zu\n", R, T, nz, wl.ps, wl.rs, wl.L, c, c0,
                    wl.ps > 0 ? wall_plane_smem(wl, nz) : (size_t)0);
    }
    const int cl[][2] = {{128, 128}, {256, 256}, {64, 64}, {32, 32}};
    for (auto &p : cl) {
        WallLayout wl{0, 0, 0};
        std::printf("cluster %d %d %d\n", p[0], p[1], wall_plane_cluster(p[0], p[1], limit, &wl));
    }
    // kept segments: avail, slot bytes, checkpoint bytes, K, nseg
    const double GB = 1e9;
    const double kc[][5] = {{200 * GB, 3.05 * GB, 2.88 * GB, 10, 10}, {1e15, 1.0, 1.0, 10, 10},
                            {1.0, 1.0, 1.0, 10, 10}, {25 * GB, 0.05 * GB, 0.03 * GB, 20, 20},
                            {100 * GB, 3.05 * GB, 2.88 * GB, 10, 10}, {150 * GB, 3.05 * GB, 2.88 * GB, 10, 10},
                            {50 * GB, 3.05 * GB, 2.88 * GB, 10, 1}};
    for (auto &k : kc)
        std::printf("kept %.6g %.6g %.6g %d %d %d\n", k[0], k[1], k[2], (int)k[3], (int)k[4],
                    kept_segments(k[0], k[1], k[2], (int)k[3], (int)k[4]));
    return 0;
}
"""


@pytest.fixture(scope="module")
def decisions(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = next((p for p in ("/usr/local/cuda/include",) if Path(p, "cuda_runtime.h").exists()), None)
    if cuda_inc is None:
        pytest.skip("no CUDA headers")
    d = tmp_path_factory.mktemp("plan")
    src, exe = d / "plan.cpp", d / "plan"
    src.write_text(HARNESS)
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{CSRC}", f"-I{cuda_inc}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {"layout": [], "cluster": {}, "kept": []}
    for line in out.splitlines():
        f = line.split()
        if f[0] == "layout":
            res["layout"].append([int(x) for x in f[1:]])
        elif f[0] == "cluster":
            res["cluster"][(int(f[1]), int(f[2]))] = int(f[3])
        else:
            res["kept"].append([float(x) for x in f[1:4]] + [int(x) for x in f[4:]])
    return res


def test_wall_layouts_fit_and_beat_the_compact_layout(decisions):
    for R, T, nz, ps, rs, L, cost, cost0, smem in decisions["layout"]:
        if (R, nz) == (258, 128):
            # a whole 256-row plane of 128 z does not fit one CTA: no layout
            # (the plane is then split over a cluster)
            assert ps == 0
            continue
        assert ps > 0, (R, T, nz)
        assert smem <= 227 * 1024
        assert T * L >= R and ps >= R and ps % 2 == 1 and rs >= R
        assert cost <= cost0, (R, T, nz, cost, cost0)


def test_wall_layout_of_the_channel(decisions):
    row = next(r for r in decisions["layout"] if r[:3] == [130, 8, 128])
    assert row[3:6] == [133, 133, 19]
    assert row[6] < row[7]      # fewer wavefronts than the compact 131 / 130 / 17


def test_wall_plane_clusters(decisions):
    c = decisions["cluster"]
    assert c[(128, 128)] == 1
    assert c[(256, 256)] == 4
    assert c[(64, 64)] == 1 and c[(32, 32)] == 1


def test_kept_segments(decisions):
    for avail, slot, ck, K, nseg, R in decisions["kept"]:
        assert 1 <= R <= nseg
        nck = nseg - R + 1 if R < nseg else 0
        if R > 1:
            assert R * K * slot + nck * ck <= avail
        if R < nseg:
            nck1 = nseg - R if R + 1 < nseg else 0
            assert (R + 1) * K * slot + nck1 * ck > avail
    by = {(a, n): R for a, s, c, K, n, R in decisions["kept"]}
    assert by[(1e15, 10)] == 10          # everything fits
    assert by[(1.0, 10)] == 1            # nothing fits
    assert by[(25e9, 20)] == 20          # the 400-step adjoint workload keeps every segment
    assert by[(100e9, 10)] <= by[(150e9, 10)] <= by[(200e9, 10)]
    assert by[(50e9, 1)] == 1
