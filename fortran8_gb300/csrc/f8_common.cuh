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
    int eigen_test;      // f8_eigen_test (3D FP64 step)
};

// Boundary-condition kinds of the halo fill kernel.
enum BcKind { BC_U = 0, BC_V = 1, BC_W = 2, BC_P = 3, BC_C = 4, BC_CODE = 5 };

// Kernel launches issued by this library in the process (reported through
// f8_diagnostics so that a caller can count the launches of a timed region).
inline std::atomic<long long> g_kernel_launches{0};
inline void count_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }

// Shared memory of the scan-Thomas wall plane kernel, whose (z, y) plane of
// one kx is split over a cluster of cl CTAs, each holding R = ceil(lj / cl)
// y rows: the rows (complex, odd row stride), the 1/den table of its systems,
// the z twiddles, and the composed forward / backward maps of its systems
// (3 floats each); the strides come from wall_layout below.
__host__ __device__ inline int wall_rows_per_cta(int lj, int cl) { return (lj + cl - 1) / cl; }

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

// Shared-memory layout of the wall-plane kernel for R rows per CTA and T
// threads per (kx, kz) system: the row stride ps (float2) of the spectrum
// tile, the row stride rs (float) of the pivot table and the rows L per
// thread of the scan-parallel Thomas solve (L >= ceil(R / T)).  The thread
// (row, t) = (lane / T, lane % T) of the solve touches row * stride + t * L +
// it at step it; the layout minimises the wavefronts of those accesses: a
// 64-bit access takes one wavefront per half-warp whose 16 lanes hit distinct
// 8-byte bank pairs, a 32-bit access one per warp on 32 distinct banks.  ps
// stays odd, which keeps the z transforms' accesses (lane stride ps) free of
// conflicts.  Evaluated once per context on the host.
struct WallLayout {
    int ps, rs, L;
};

inline int wl_max_per_bank(const int *word, int n) {
    int cnt[32] = {0}, seen[32][32];
    int best = 0;
    for (int q = 0; q < n; ++q) {
        const int b = word[q] & 31;
        bool dup = false;
        for (int r = 0; r < cnt[b]; ++r) dup = dup || seen[b][r] == word[q];
        if (dup) continue;
        seen[b][cnt[b]++] = word[q];
        best = cnt[b] > best ? cnt[b] : best;
    }
    return best;
}

inline long wl_cost(int R, int T, int ps, int rs, int L) {
    long tot = 0;
    int w2[32], w1[32];
    for (int it = 0; it < L; ++it) {
        int n1 = 0;
        for (int h = 0; h < 32; h += 16) {
            int n2 = 0;
            for (int lane = h; lane < h + 16; ++lane) {
                const int row = lane / T, t = lane % T;
                const int c0 = t * L < R ? t * L : R, c1 = c0 + L < R ? c0 + L : R;
                const int jl = c0 + it;
                if (jl >= c1) continue;
                const int q = row * ps + jl;
                w2[n2++] = 2 * q;
                w2[n2++] = 2 * q + 1;
                w1[n1++] = row * rs + jl;
            }
            tot += wl_max_per_bank(w2, n2);
        }
        tot += wl_max_per_bank(w1, n1);
    }
    return tot;
}

inline size_t wall_plane_smem(const WallLayout &wl, int nz) {
    return (size_t)8 * wl.ps * nz + (size_t)4 * wl.rs * nz + (size_t)nz * 8 + (size_t)24 * nz;
}

// the layout of least cost whose shared memory fits in `limit` bytes (ps = 0:
// none fits)
inline WallLayout wall_layout(int R, int T, int nz, size_t limit) {
    const int L0 = (R + T - 1) / T;
    WallLayout best{0, 0, 0};
    long bc = -1;
    for (int L = L0; L < L0 + 12; ++L)
        for (int ps = R | 1; ps < (R | 1) + 16; ps += 2)      // ps matters modulo 16 (8-byte pairs)
            for (int rs = R; rs < R + 32; ++rs) {             // rs modulo 32
                if (wall_plane_smem(WallLayout{ps, rs, L}, nz) > limit) continue;
                const long c = wl_cost(R, T, ps, rs, L);
                if (bc < 0 || c < bc) { bc = c; best = WallLayout{ps, rs, L}; }
            }
    return best;
}

// smallest cluster (<= 8 CTAs) whose per-CTA share of the plane fits in
// `limit` bytes of shared memory with some layout (its best layout in *wl), or 0
inline int wall_plane_cluster(int ny, int nz, size_t limit, WallLayout *wl) {
    if (nz != 32 && nz != 64 && nz != 128 && nz != 256) return 0;
    for (int cl = 1; cl <= 8; ++cl) {
        const int r = wall_rows_per_cta(ny + 2, cl);
        // the most compact layout first: skip the search where even it does not fit
        if (wall_plane_smem(WallLayout{r | 1, r, 0}, nz) > limit) continue;
        *wl = wall_layout(r, 1024 / nz, nz, limit);
        if (wl->ps > 0) return cl;
    }
    return 0;
}

// Segments (the last R >= 1 of nseg segments of K steps) whose tape the first
// forward pass of a gradient keeps: the largest R whose tapes (slot_bytes per
// step) and the checkpoints of the nseg - R segments before them plus one for
// the final state (ck_bytes each) fit in avail bytes; 1 when none does.
inline int kept_segments(double avail, double slot_bytes, double ck_bytes, int K, int nseg) {
    for (int r = nseg; r > 1; --r) {
        const int nck = r < nseg ? nseg - r + 1 : 0;
        if ((double)r * K * slot_bytes + nck * ck_bytes <= avail) return r;
    }
    return 1;
}

struct StepCounters {
    unsigned long long newton_iters;
    unsigned long long newton_unconverged;
    unsigned long long nan_cells;
    unsigned long long copy_timeouts;   // bulk-copy waits that ran out (the kernel stopped early)
};

}  // namespace f8

#define F8_CUDA_RET(call)                          \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)
