// f8_common.cuh — shared device definitions of the GB300 SMAC + FENE-P + IBM step.
//
// Device memory layout (structure of arrays, x fastest):
//   halo scalar fields (U, V, W, P, Phi, Ua.., Up..): (NX+2)(NY+2)(NZ+2) values,
//     index h(i,j,k) = i + SX*(j + SY*k), i in 0..NX+1 (the reference's
//     (0:NX+1, 0:NY+1, 0:NZ+1) Fortran layout, fenep.f90:2424).
//   C: NC separate halo fields (SoA) instead of the reference's component-fastest
//     C(6, 0:NX+1, ...): a warp then reads 32 consecutive x of one component.
//   interior fields (A0, T0, F, B, Q): NX*NY*NZ values, index q(i,j,k) =
//     (i-1) + NX*((j-1) + NY*(k-1)).
//   spectra: complex (re, im interleaved) [k][j][kx], kx in 0..NX/2.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace f8 {

struct Geo {
    int nx, ny, nz;      // cells
    int sx, sy, sz;      // halo extents nx+2 ...
    int dim;             // 2 or 3
    int walls;           // y walls (1) or periodic (0)
    double dx, dy, dz;
    double dt;
    double uwall;
};

__host__ __device__ inline int hix(const Geo &g, int i, int j, int k) { return i + g.sx * (j + g.sy * k); }
__host__ __device__ inline int qix(const Geo &g, int i, int j, int k) { return (i - 1) + g.nx * ((j - 1) + g.ny * (k - 1)); }
__host__ __device__ inline int wrapx(const Geo &g, int i) { return i < 1 ? i + g.nx : (i > g.nx ? i - g.nx : i); }
__host__ __device__ inline int wrapy(const Geo &g, int j) { return j < 1 ? j + g.ny : (j > g.ny ? j - g.ny : j); }
__host__ __device__ inline int wrapz(const Geo &g, int k) { return k < 1 ? k + g.nz : (k > g.nz ? k - g.nz : k); }

// Rows of the polymer update.  Periodic in y: 1..NY.  With y walls also the
// ghost rows 0 and NY+1: the reference's wall mode updates C on every row of
// its box, the rows beyond the walls holding zero C and velocity, keeps the
// updated ghost rows through the stress and extrapolates them only at the end
// of the step (fenep_2d.f90:1097-1143, 1371-1374, 1912-1966).
__host__ __device__ inline int prow0(const Geo &g) { return g.walls ? 0 : 1; }
__host__ __device__ inline int prows(const Geo &g) { return g.walls ? g.ny + 2 : g.ny; }
// selection codes of the ghost rows (walls): [k][side][i], side 0: j = 0, 1: j = NY+1
__host__ __device__ inline int gcix(const Geo &g, int i, int j, int k) {
    return (i - 1) + g.nx * ((j == 0 ? 0 : 1) + 2 * (k - 1));
}

// Physical parameters the kernels need (copied from f8_phys).
struct Phys {
    double re, wi, beta, lp2, dt;
    double newton_dc, newton_eps;
    int newton_itrmax;
};

// Boundary-condition kinds of the halo fill kernel.
enum BcKind { BC_U = 0, BC_V = 1, BC_W = 2, BC_P = 3, BC_C = 4, BC_CODE = 5 };

// Kernel launches issued by this library in the process (reported through
// f8_diagnostics so that a caller can count the launches of a timed region).
inline std::atomic<long long> g_kernel_launches{0};
inline void count_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }

// Per-step device counters (status words read by the host after a step).
// Shared memory of the scan-Thomas wall plane kernel, whose (z, y) plane of
// one kx is split over a cluster of cl CTAs, each holding R = ceil(lj / cl)
// y rows: the rows (complex, odd row stride), the 1/den table of its systems
// (row stride >= R and = T (mod 32), T = 1024 / nz threads per system, so
// that the systems x chunks of a warp read distinct banks), the z twiddles,
// and the composed forward / backward maps of its systems (3 floats each).
__host__ __device__ inline int wall_rows_per_cta(int lj, int cl) { return (lj + cl - 1) / cl; }
__host__ __device__ inline int wall_rd_stride(int r, int t) { return r + (((t - r) % 32) + 32) % 32; }

// Halo cells of a field with one halo layer, numbered face by face.
__host__ __device__ inline long halo_count(const Geo &g) {
    return 2L * g.sy * g.sz + 2L * g.nx * g.sz + 2L * g.nx * g.ny;
}

// halo cell number t -> (i, j, k): the two x faces (all j, k), the two y
// faces (interior i, all k), the two z faces (interior i, j).  32-bit index
// arithmetic (the grid has fewer than 2^31 cells), one division per cell.
__device__ inline bool halo_cell(const Geo &g, long tl, int &i, int &j, int &k) {
    if (tl < 0 || tl >= halo_count(g)) return false;
    int t = (int)tl;
    int plane = g.sy * g.sz;
    if (t < 2 * plane) {
        const bool hi = t >= plane;
        const int r = hi ? t - plane : t;
        i = hi ? g.sx - 1 : 0;
        k = r / g.sy; j = r - k * g.sy;
        return true;
    }
    t -= 2 * plane;
    plane = g.nx * g.sz;
    if (t < 2 * plane) {
        const bool hi = t >= plane;
        const int r = hi ? t - plane : t;
        j = hi ? g.sy - 1 : 0;
        k = r / g.nx; i = 1 + r - k * g.nx;
        return true;
    }
    t -= 2 * plane;
    plane = g.nx * g.ny;
    const bool hi = t >= plane;
    const int r = hi ? t - plane : t;
    k = hi ? g.sz - 1 : 0;
    j = r / g.nx; i = 1 + r - j * g.nx;
    j += 1;
    return true;
}

__host__ __device__ inline size_t wall_plane_smem(int ny, int nz, int cl) {
    const int r = wall_rows_per_cta(ny + 2, cl);
    return (size_t)8 * (r | 1) * nz + (size_t)4 * wall_rd_stride(r, 1024 / nz) * nz + (size_t)(nz / 2) * 8
           + (size_t)24 * nz;
}

// smallest cluster (<= 8 CTAs) whose per-CTA share of the plane fits in
// `limit` bytes of shared memory, or 0
inline int wall_plane_cluster(int ny, int nz, size_t limit) {
    if (nz != 32 && nz != 64 && nz != 128 && nz != 256) return 0;
    for (int cl = 1; cl <= 8; ++cl)
        if (wall_plane_smem(ny, nz, cl) <= limit) return cl;
    return 0;
}

struct StepCounters {
    unsigned long long newton_iters;
    unsigned long long newton_unconverged;
    unsigned long long nan_cells;
};

}  // namespace f8

#define F8_CUDA_RET(call)                          \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)
