// f8_fft_fused.cuh — FP32 spectral solves of the mixed-precision path with the
// whole (z, y) plane of one x-wavenumber resident in shared memory.
//
// Spectrum layout S[kx][k][j] (complex float), j contiguous, LJ values per
// (kx, k) line: LJ = NY for periodic y, NY + 2 for walls (rows 0 and NY+1 are
// the ghost rows of the wall systems, fenep_2d.f90:1222-1238).
//
//   k_xfwd_t   real rows -> S: two rows per complex FFT of length NX (the
//              same pairing as the FP64 kernels), transposed through shared
//              memory so that each kx receives RB consecutive rows.
//   k_plane_*  one CTA per kx: in-place radix-2 transforms along z (and y when
//              periodic), the spectral divide (fft_solve, fenep.f90:1400-1428)
//              or the Thomas solve along y (tdma, fenep_2d.f90:1145-1177), and
//              the inverse transforms.  Forward transforms are decimation in
//              time (bit-reversed load), inverse ones decimation in frequency
//              (bit-reversed store), so no reordering pass is needed.
//   k_xinv_t   S -> real rows through a destination functor (XOutF).
#pragma once
#include <cooperative_groups.h>
#include "f8_common.cuh"
#include "f8_fft.cuh"

namespace f8 {

__device__ inline int bitrev(int v, int lg) { return lg ? (int)(__brev((unsigned)v) >> (32 - lg)) : 0; }

// ---------------------------------------------------------------------------
// x forward, transposing.  Block b handles RB rows (RB/2 pairs) of plane k.
// The [kx][row] tile has an odd row stride (RB + 1) against bank conflicts.
template <typename TS>
__global__ void k_xfwd_t(const TS *__restrict__ src, float2 *__restrict__ S, int nx, int ny, int nz, int rb, int lj,
                         int joff, const float *__restrict__ twr, const float *__restrict__ twi) {
    extern __shared__ unsigned char smem_raw[];
    Cx<float> *sm = reinterpret_cast<Cx<float> *>(smem_raw);
    const int half = nx >> 1, nxh = half + 1;
    const int npair = rb >> 1;
    const int p = threadIdx.x / half, t = threadIdx.x % half;
    const int blocks_per_plane = (ny + rb - 1) / rb;
    const int k = blockIdx.x / blocks_per_plane;
    const int r0 = (blockIdx.x % blocks_per_plane) * rb;       // first row (0-based) of the block
    const int nrows = min(rb, ny - r0);
    const bool active = p < npair && 2 * p < nrows;
    Cx<float> *x = sm + (size_t)p * 2 * nx, *y = x + nx;
    if (active) {
        const TS *ra = src + (size_t)nx * ((size_t)(r0 + 2 * p) + (size_t)ny * k);
        const TS *rbp = ra + nx;
        for (int e = t; e < nx; e += half) { x[e].r = (float)ra[e]; x[e].i = (float)rbp[e]; }
    }
    __syncthreads();
    for (int ns = 1; ns < nx; ns *= 2) {
        if (active) stockham_stage(x, y, nx, ns, t, twr, twi, -1);
        __syncthreads();
        Cx<float> *tmp = x; x = y; y = tmp;
    }
    // unpack the two real spectra of each pair into a [kx][row] tile; the
    // result of pair p is in buffer x (the same buffer index for all pairs)
    const bool res_in_first = ((__ffs(nx) - 1) % 2) == 0;  // log2(nx) even -> back in the first buffer
    float2 *tile = reinterpret_cast<float2 *>(sm + (size_t)npair * 2 * nx);
    if (active) {
        const Cx<float> *z = sm + (size_t)p * 2 * nx + (res_in_first ? 0 : nx);
        for (int kx = t; kx < nxh; kx += half) {
            const int m = (nx - kx) % nx;
            const Cx<float> zk = z[kx], zm = z[m];
            tile[(size_t)kx * (rb + 1) + 2 * p] = make_float2((zk.r + zm.r) * 0.5f, (zk.i - zm.i) * 0.5f);
            tile[(size_t)kx * (rb + 1) + 2 * p + 1] = make_float2((zk.i + zm.i) * 0.5f, (zm.r - zk.r) * 0.5f);
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nxh * rb; q += blockDim.x) {
        const int kx = q / rb, r = q % rb;
        if (r < nrows) S[((size_t)kx * nz + k) * lj + (r0 + r + 1 + joff)] = tile[(size_t)kx * (rb + 1) + r];
    }
}

// x inverse, transposing: rows j = jlo .. jlo+nrow-1 of S (S row index
// j + joff2) become real rows j of a halo-layout field (x at 1..nx), written
// through the destination functor (XOutF).
template <typename Out>
__global__ void k_xinv_t(const float2 *__restrict__ S, Out out, int nx, int nrow, int jlo, int nz,
                         int rb, int lj, int joff2, int sx, int sy, const float *__restrict__ twr,
                         const float *__restrict__ twi) {
    extern __shared__ unsigned char smem_raw[];
    Cx<float> *sm = reinterpret_cast<Cx<float> *>(smem_raw);
    const int half = nx >> 1, nxh = half + 1;
    const int npair = rb >> 1;
    const int blocks_per_plane = (nrow + rb - 1) / rb;
    const int k = blockIdx.x / blocks_per_plane;
    const int r0 = (blockIdx.x % blocks_per_plane) * rb;
    const int nrows = min(rb, nrow - r0);
    float2 *tile = reinterpret_cast<float2 *>(sm + (size_t)npair * 2 * nx);
    for (int q = threadIdx.x; q < nxh * rb; q += blockDim.x) {
        const int kx = q / rb, r = q % rb;
        tile[(size_t)kx * (rb + 1) + r] = r < nrows ? S[((size_t)kx * nz + k) * lj + (jlo + r0 + r + joff2)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int p = threadIdx.x / half, t = threadIdx.x % half;
    const bool active = p < npair && 2 * p < nrows;
    Cx<float> *x = sm + (size_t)p * 2 * nx, *y = x + nx;
    if (active) {
        for (int e = t; e < nx; e += half) {
            float ar, ai, br, bi;
            if (e <= half) {
                const float2 A = tile[(size_t)e * (rb + 1) + 2 * p], B = tile[(size_t)e * (rb + 1) + 2 * p + 1];
                ar = A.x; ai = A.y; br = B.x; bi = B.y;
                x[e].r = ar - bi; x[e].i = ai + br;
            } else {
                const int m = nx - e;
                const float2 A = tile[(size_t)m * (rb + 1) + 2 * p], B = tile[(size_t)m * (rb + 1) + 2 * p + 1];
                ar = A.x; ai = A.y; br = B.x; bi = B.y;
                x[e].r = ar + bi; x[e].i = br - ai;
            }
        }
    }
    __syncthreads();
    for (int ns = 1; ns < nx; ns *= 2) {
        if (active) stockham_stage(x, y, nx, ns, t, twr, twi, +1);
        __syncthreads();
        Cx<float> *tmp = x; x = y; y = tmp;
    }
    if (!active) return;
    const size_t oa = 1 + (size_t)sx * ((size_t)(jlo + r0 + 2 * p) + (size_t)sy * (k + 1));
    const bool has_b = 2 * p + 1 < nrows;
    for (int e = t; e < nx; e += half) {
        out.put(oa + e, x[e].r);
        if (has_b) out.put(oa + sx + e, x[e].i);
    }
}

// ---------------------------------------------------------------------------
// In-place radix-2 stages over nlines lines of length n held in shared memory
// (element e of line l at P[l*lstride_l + e*estride]).
__device__ inline void dit_lines(float2 *P, int n, int lg, int nlines, int lstride, int estride, const float *twr,
                                 const float *twi, float sign) {
    const int half = n >> 1;
    for (int m = 1; m < n; m <<= 1) {
        const int tws = n / (2 * m);
        for (int q = threadIdx.x; q < nlines * half; q += blockDim.x) {
            // consecutive threads take consecutive addresses: along the line
            // when it is contiguous, across lines otherwise
            const int l = estride == 1 ? q / half : q % nlines;
            const int b = estride == 1 ? q % half : q / nlines;
            const int pos = b % m, grp = b / m;
            const int i0 = grp * 2 * m + pos;
            float2 *base = P + (size_t)l * lstride;
            const float wr = twr[pos * tws], wi = sign * twi[pos * tws];
            const float2 a = base[(size_t)i0 * estride], c = base[(size_t)(i0 + m) * estride];
            const float tr = c.x * wr - c.y * wi, ti = c.x * wi + c.y * wr;
            base[(size_t)i0 * estride] = make_float2(a.x + tr, a.y + ti);
            base[(size_t)(i0 + m) * estride] = make_float2(a.x - tr, a.y - ti);
        }
        __syncthreads();
    }
    (void)lg;
}

__device__ inline void dif_lines(float2 *P, int n, int nlines, int lstride, int estride, const float *twr,
                                 const float *twi, float sign) {
    const int half = n >> 1;
    for (int m = half; m >= 1; m >>= 1) {
        const int tws = n / (2 * m);
        for (int q = threadIdx.x; q < nlines * half; q += blockDim.x) {
            const int l = estride == 1 ? q / half : q % nlines;
            const int b = estride == 1 ? q % half : q / nlines;
            const int pos = b % m, grp = b / m;
            const int i0 = grp * 2 * m + pos;
            float2 *base = P + (size_t)l * lstride;
            const float wr = twr[pos * tws], wi = sign * twi[pos * tws];
            const float2 a = base[(size_t)i0 * estride], c = base[(size_t)(i0 + m) * estride];
            const float dr = a.x - c.x, di = a.y - c.y;
            base[(size_t)i0 * estride] = make_float2(a.x + c.x, a.y + c.y);
            base[(size_t)(i0 + m) * estride] = make_float2(dr * wr - di * wi, dr * wi + di * wr);
        }
        __syncthreads();
    }
}

// Periodic y and z: forward 2-D transform, divide by ntot * LHS (LHS = lhs0 +
// lhs1 (kx2 + ky2 + kz2); zero where |LHS| < 1e-16), inverse transform.
struct PlaneSpec {
    const float *kx2, *ky2, *kz2;   // modified wavenumbers (FP32 copies)
    float lhs0, lhs1, inv_ntot;
    // walls: row coefficients of the y systems (see k_plane_walls)
    float ai_base, bc;        // interior a = ai_base + kap * lam; b = c = bc
    float kap;                // dt beta / (2 Re) (Helmholtz) or -1 (Poisson: a = -(lam + 2/dy^2))
    int sys;                  // WallSys
    float nxz_inv;            // 1 / (NX NZ)
};

__global__ void k_plane_periodic(float2 *S, int ny, int nz, int lgy, int lgz, const float *twyr, const float *twyi,
                                 const float *twzr, const float *twzi, PlaneSpec ps) {
    extern __shared__ unsigned char smem_raw[];
    const int nys = ny + 1;                              // odd shared-memory row stride
    float2 *P = reinterpret_cast<float2 *>(smem_raw);    // [k][j], bit-reversed in both on load
    const int kx = blockIdx.x;
    float2 *Sp = S + (size_t)kx * nz * ny;
    for (int q = threadIdx.x; q < ny * nz; q += blockDim.x) {
        const int k = q / ny, j = q % ny;
        P[(size_t)bitrev(k, lgz) * nys + bitrev(j, lgy)] = Sp[q];
    }
    __syncthreads();
    dit_lines(P, ny, lgy, nz, nys, 1, twyr, twyi, 1.0f);     // along y (lines k)
    dit_lines(P, nz, lgz, ny, 1, nys, twzr, twzi, 1.0f);     // along z (lines j)
    const float k2x = ps.kx2[kx];
    for (int q = threadIdx.x; q < ny * nz; q += blockDim.x) {
        const int k = q / ny, j = q % ny;
        const float lhs = ps.lhs0 + ps.lhs1 * (k2x + ps.ky2[j] + ps.kz2[k]);
        const float sc = fabsf(lhs) < 1.0e-16f ? 0.0f : ps.inv_ntot / lhs;
        const float2 v = P[(size_t)k * nys + j];
        P[(size_t)k * nys + j] = make_float2(v.x * sc, v.y * sc);
    }
    __syncthreads();
    dif_lines(P, nz, ny, 1, nys, twzr, twzi, -1.0f);
    dif_lines(P, ny, nz, nys, 1, twyr, twyi, -1.0f);
    for (int q = threadIdx.x; q < ny * nz; q += blockDim.x) {
        const int k = q / ny, j = q % ny;
        Sp[q] = P[(size_t)bitrev(k, lgz) * nys + bitrev(j, lgy)];
    }
}

// Walls in y: forward z transform of rows 1..NY, Thomas solve along y of each
// kz over rows 0..NY+1 with the boundary rows of the system (homogeneous:
// the mixed path solves for increments), inverse z transform of all rows.
__global__ void k_plane_walls(float2 *S, int ny, int nz, int lgz, const float *twzr, const float *twzi, PlaneSpec ps) {
    extern __shared__ unsigned char smem_raw[];
    const int lj = ny + 2;
    const int ljs = lj | 1;                                            // odd shared-memory row stride
    float2 *P = reinterpret_cast<float2 *>(smem_raw);                 // [k][j], k bit-reversed on load
    float *Pc = reinterpret_cast<float *>(P + (size_t)ljs * nz);      // Thomas P coefficients [k][j]
    const int kx = blockIdx.x;
    float2 *Sp = S + (size_t)kx * nz * lj;
    for (int q = threadIdx.x; q < lj * nz; q += blockDim.x) {
        const int k = q / lj, j = q % lj;
        P[(size_t)bitrev(k, lgz) * ljs + j] = (j >= 1 && j <= ny) ? Sp[q] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    dit_lines(P + 1, nz, lgz, ny, 1, ljs, twzr, twzi, 1.0f);  // lines j = 1..ny, along k
    // Thomas along j for each kz (natural order after DIT)
    const float lamx = ps.kx2[kx];
    for (int kz = threadIdx.x; kz < nz; kz += blockDim.x) {
        float2 *x = P + (size_t)kz * ljs;
        float *pc = Pc + (size_t)kz * ljs;
        const float lam = lamx + ps.kz2[kz];
        float ai, bc = ps.bc;
        if (ps.sys == SYS_P) ai = -(lam + ps.ai_base);
        else ai = ps.ai_base + ps.kap * lam;
        // row 0
        float a0, b0;
        if (ps.sys == SYS_U) { a0 = 1.f; b0 = 1.f; }
        else if (ps.sys == SYS_V) { a0 = 1.f; b0 = 0.f; }
        else { a0 = 1.f; b0 = -1.f; }
        float p = -b0 / a0;
        float2 qv = make_float2(0.f, 0.f);
        pc[0] = p; x[0] = qv;
        for (int j = 1; j < lj; ++j) {
            float a, b, c;
            float2 d;
            const bool last = j == lj - 1;
            if (ps.sys == SYS_U) {
                if (last) { a = 1.f; b = 0.f; c = 1.f; d = make_float2(0.f, 0.f); }
                else { a = ai; b = bc; c = bc; d = x[j]; d.x *= ps.nxz_inv; d.y *= ps.nxz_inv; }
            } else if (ps.sys == SYS_V) {
                if (j >= ny) { a = 1.f; b = 0.f; c = 0.f; d = make_float2(0.f, 0.f); }
                else { a = ai; b = bc; c = bc; d = x[j]; d.x *= ps.nxz_inv; d.y *= ps.nxz_inv; }
            } else {
                if (last) { a = 1.f; b = 0.f; c = -1.f; d = make_float2(0.f, 0.f); }
                else { a = ai; b = bc; c = bc; d = x[j]; d.x *= ps.nxz_inv; d.y *= ps.nxz_inv; }
            }
            // true divisions, as tdma does: on the singular Neumann mode of the
            // pressure system p stays exactly 1 and the last pivot is exactly
            // zero, so the reference's guard pins that mode
            const float den = a + c * p;
            if (fabsf(den) < 1.0e-16f) {
                p = 0.f; qv = make_float2(0.f, 0.f);
            } else {
                p = -b / den;
                qv = make_float2((d.x - c * qv.x) / den, (d.y - c * qv.y) / den);
            }
            pc[j] = p; x[j] = qv;
        }
        float2 xv = x[lj - 1];
        for (int j = lj - 2; j >= 0; --j) {
            const float pj = pc[j];
            const float2 qj = x[j];
            xv = make_float2(pj * xv.x + qj.x, pj * xv.y + qj.y);
            x[j] = xv;
        }
    }
    __syncthreads();
    dif_lines(P, nz, lj, 1, ljs, twzr, twzi, -1.0f);         // all rows, along k
    for (int q = threadIdx.x; q < lj * nz; q += blockDim.x) {
        const int k = q / lj, j = q % lj;
        Sp[q] = P[(size_t)bitrev(k, lgz) * ljs + j];
    }
}

}  // namespace f8

namespace f8 {

// ---------------------------------------------------------------------------
// Warp-level radix-2 transform of one line of N = 32*V points: lane t holds
// elements t + 32 s (s < V).  Spans >= 32 are butterflies inside the lane,
// spans < 32 exchange with lane t ^ span.  tw: forward twiddles in shared
// memory, stage-major: the stage of span m reads w^(p N / (2m)), p < m, at
// tw[m - 1 + p], w = (cos, -sin)(2 pi / N), so the lanes of a stage read
// consecutive entries (no bank conflicts, where a table indexed by p N/(2m)
// has lane stride N/(2m)).  The complex arithmetic uses packed FP32x2
// operations; the cross-lane butterflies are branch-free (the lanes holding
// the first element of a pair multiply by 1).
__device__ __forceinline__ float2 cmul_p(float2 a, float2 w) {
    return __ffma2_rn(make_float2(a.x, a.x), w, __fmul2_rn(make_float2(a.y, a.y), make_float2(-w.y, w.x)));
}

template <int V>
__device__ inline void warp_dif_fwd(float2 (&v)[V], const float2 *tw, int lane) {
    constexpr int N = 32 * V;
#pragma unroll
    for (int m = N / 2; m >= 1; m >>= 1) {
        const float2 *tm = tw + (m - 1);
        if (m >= 32) {
            const int sm = m / 32;
#pragma unroll
            for (int s = 0; s < V; ++s) {
                if ((s / sm) % 2) continue;          // upper element of the pair
                const int pos = (lane + 32 * s) % (2 * m);
                const float2 w = tm[pos];
                const float2 a = v[s], b = v[s + sm];
                v[s] = __fadd2_rn(a, b);
                v[s + sm] = cmul_p(__ffma2_rn(b, make_float2(-1.0f, -1.0f), a), w);
            }
        } else {
            const bool second = lane & m;            // this lane holds the second element
            const float2 w = second ? tm[(lane % (2 * m)) - m] : make_float2(1.0f, 0.0f);
            const float sg = second ? -1.0f : 1.0f;
#pragma unroll
            for (int s = 0; s < V; ++s) {
                float2 o;
                o.x = __shfl_xor_sync(0xffffffffu, v[s].x, m);
                o.y = __shfl_xor_sync(0xffffffffu, v[s].y, m);
                // first: a + b; second: (a - b) w, with a the first element
                v[s] = cmul_p(__ffma2_rn(make_float2(sg, sg), v[s], o), w);
            }
        }
    }
}

// inverse (conjugate twiddles), decimation in time: bit-reversed in, natural out
template <int V>
__device__ inline void warp_dit_inv(float2 (&v)[V], const float2 *tw, int lane) {
    constexpr int N = 32 * V;
#pragma unroll
    for (int m = 1; m < N; m <<= 1) {
        const float2 *tm = tw + (m - 1);
        if (m >= 32) {
            const int sm = m / 32;
#pragma unroll
            for (int s = 0; s < V; ++s) {
                if ((s / sm) % 2) continue;
                const int pos = (lane + 32 * s) % (2 * m);
                const float2 w = tm[pos];
                const float2 t = cmul_p(v[s + sm], make_float2(w.x, -w.y));
                const float2 a = v[s];
                v[s] = __fadd2_rn(a, t);
                v[s + sm] = __ffma2_rn(t, make_float2(-1.0f, -1.0f), a);
            }
        } else {
            const bool second = lane & m;
            float2 w = make_float2(1.0f, 0.0f);
            if (second) {
                const float2 tv = tm[(lane % (2 * m)) - m];
                w = make_float2(tv.x, -tv.y);
            }
            const float sg = second ? -1.0f : 1.0f;
#pragma unroll
            for (int s = 0; s < V; ++s) {
                // the second element is multiplied by the twiddle before the
                // exchange: first: a + b w; second: a - b w
                const float2 p = cmul_p(v[s], w);
                float2 o;
                o.x = __shfl_xor_sync(0xffffffffu, p.x, m);
                o.y = __shfl_xor_sync(0xffffffffu, p.y, m);
                v[s] = __ffma2_rn(make_float2(sg, sg), p, o);
            }
        }
    }
}

// Pivot table of the y systems of one solve type: for each (kx, kz) the
// Thomas factors 1/den_j (0 where the pivot vanishes, the reference's guard),
// computed on the host in FP64.  The back-substitution multipliers are
// P_j = -b_j / den_j with b_j the super-diagonal of row j.
struct WallTables {
    const float *rden;   // [kx][kz][j]
    float bc;            // interior off-diagonal b = c
    float c_last;        // c of the last row (1 U, -1 P); V: rows >= ny are identities
    float b_first;       // b of row 0 (1 U, -1 P, 0 V)
    float nxz_inv;
    int sys;
    WallLayout wl;       // shared-memory strides and Thomas rows per thread (wall_layout)
};

// ---------------------------------------------------------------------------
// Warp-per-row-pair x passes (NX = 32 E).  Each warp transforms two real rows
// packed as one complex line with warp_dif_fwd / warp_dit_inv (lane t holds
// x = t + 32 s), unpacks / packs the two half spectra through a per-warp
// buffer, and the block exchanges RB rows with the [kx][row] tile as the
// radix-2 passes above do.  Per-warp buffer index of X[k]: k + (k >> lg E),
// which makes both the bit-reversed (lane stride E + 1) and the natural
// accesses free of bank conflicts.
template <int E> struct LgE { static constexpr int v = E == 1 ? 0 : E == 2 ? 1 : E == 4 ? 2 : E == 8 ? 3 : 4; };

__device__ __forceinline__ int zb_ix(int k, int lge) { return k + (k >> lge); }

// natural index of element s of lane t after a DIF transform (bit-reversed)
template <int E>
__device__ __forceinline__ int brev_elem(int lane, int s) {
    constexpr int LG = LgE<E>::v;
    const int bl = (int)(__brev((unsigned)lane) >> 27);
    const int bs = LG ? (int)(__brev((unsigned)s) >> (32 - LG)) : 0;
    return (bl << LG) | bs;
}

constexpr int XW_WARPS = 4;   // warps per block of the x passes
constexpr int XW_RB = 16;     // rows per block of the x passes (a constant: the tile indexing divides by it)

inline size_t xw_smem(int nx, int rb) {
    const int nh = nx / 2;
    return ((size_t)nx + (size_t)(nh + 1) * (rb + 1) + (size_t)XW_WARPS * (nx + 32)) * sizeof(float2);
}

template <int E, typename TS>
__global__ void __launch_bounds__(32 * XW_WARPS) k_xfwd_w(const TS *__restrict__ src, float2 *__restrict__ S, int ny,
                                                         int nz, int lj, int joff, const float2 *__restrict__ twx) {
    constexpr int N = 32 * E, NH = N / 2, LG = LgE<E>::v, rb = XW_RB;
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 *tws = reinterpret_cast<float2 *>(smem_raw);
    float2 *tile = tws + N;
    float2 *zb = tile + (size_t)(NH + 1) * (rb + 1) + (size_t)warp * (N + 32);
    for (int q = threadIdx.x; q < N; q += blockDim.x) tws[q] = twx[q];
    const int bpp = (ny + rb - 1) / rb;
    const int k = blockIdx.x / bpp;
    const int r0 = (blockIdx.x % bpp) * rb;
    const int nrows = min(rb, ny - r0);
    __syncthreads();
    for (int p = warp; 2 * p < nrows; p += XW_WARPS) {
        const bool has_b = 2 * p + 1 < nrows;
        const TS *ra = src + (size_t)N * ((size_t)(r0 + 2 * p) + (size_t)ny * k);
        float2 v[E];
#pragma unroll
        for (int s = 0; s < E; ++s)
            v[s] = make_float2((float)ra[lane + 32 * s], has_b ? (float)ra[N + lane + 32 * s] : 0.0f);
        warp_dif_fwd<E>(v, tws, lane);
#pragma unroll
        for (int s = 0; s < E; ++s) zb[zb_ix(brev_elem<E>(lane, s), LG)] = v[s];
        __syncwarp();
        for (int kx = lane; kx <= NH; kx += 32) {
            const float2 zk = zb[zb_ix(kx, LG)], zm = zb[zb_ix((N - kx) & (N - 1), LG)];
            tile[(size_t)kx * (rb + 1) + 2 * p] = make_float2((zk.x + zm.x) * 0.5f, (zk.y - zm.y) * 0.5f);
            tile[(size_t)kx * (rb + 1) + 2 * p + 1] = make_float2((zk.y + zm.y) * 0.5f, (zm.x - zk.x) * 0.5f);
        }
        __syncwarp();
    }
    __syncthreads();
    for (int q = threadIdx.x; q < (NH + 1) * rb; q += blockDim.x) {
        const int kx = q / rb, r = q % rb;
        if (r < nrows) S[((size_t)kx * nz + k) * lj + (r0 + r + 1 + joff)] = tile[(size_t)kx * (rb + 1) + r];
    }
}

template <int E, typename Out>
__global__ void __launch_bounds__(32 * XW_WARPS) k_xinv_w(const float2 *__restrict__ S, Out out,
                                                         int nrow, int jlo, int nz, int lj, int joff2, int sx,
                                                         int sy, const float2 *__restrict__ twx) {
    constexpr int N = 32 * E, NH = N / 2, LG = LgE<E>::v, rb = XW_RB;
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 *tws = reinterpret_cast<float2 *>(smem_raw);
    float2 *tile = tws + N;
    float2 *zb = tile + (size_t)(NH + 1) * (rb + 1) + (size_t)warp * (N + 32);
    for (int q = threadIdx.x; q < N; q += blockDim.x) tws[q] = twx[q];
    const int bpp = (nrow + rb - 1) / rb;
    const int k = blockIdx.x / bpp;
    const int r0 = (blockIdx.x % bpp) * rb;
    const int nrows = min(rb, nrow - r0);
    // gather the tile: four loads in flight per thread before their stores
    for (int q0 = threadIdx.x; q0 < (NH + 1) * rb; q0 += 4 * blockDim.x) {
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * blockDim.x;
            const int kx = q / rb, r = q % rb;
            v[u] = (q < (NH + 1) * rb && r < nrows) ? S[((size_t)kx * nz + k) * lj + (jlo + r0 + r + joff2)]
                                                   : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * blockDim.x;
            if (q < (NH + 1) * rb) tile[(size_t)(q / rb) * (rb + 1) + q % rb] = v[u];
        }
    }
    __syncthreads();
    for (int p = warp; 2 * p < nrows; p += XW_WARPS) {
        const bool has_b = 2 * p + 1 < nrows;
        // Z = A + i B over the full line from the two half spectra
        for (int e = lane; e < N; e += 32) {
            const int m = e <= NH ? e : N - e;
            const float2 A = tile[(size_t)m * (rb + 1) + 2 * p], B = tile[(size_t)m * (rb + 1) + 2 * p + 1];
            zb[zb_ix(e, LG)] = e <= NH ? make_float2(A.x - B.y, A.y + B.x) : make_float2(A.x + B.y, B.x - A.y);
        }
        __syncwarp();
        float2 v[E];
#pragma unroll
        for (int s = 0; s < E; ++s) v[s] = zb[zb_ix(brev_elem<E>(lane, s), LG)];
        __syncwarp();
        warp_dit_inv<E>(v, tws, lane);
        const size_t oa = 1 + (size_t)sx * ((size_t)(jlo + r0 + 2 * p) + (size_t)sy * (k + 1));
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int e = lane + 32 * s;
            out.put(oa + e, v[s].x);
            if (has_b) out.put(oa + sx + e, v[s].y);
        }
    }
}

// Wall plane with the Thomas solves split over T = 1024 / NZ threads per
// (kx, kz) system and, for planes larger than one CTA's shared memory, over a
// thread-block cluster of cl CTAs holding consecutive bands of y rows.  Both
// sweeps are first-order affine recurrences,
//   forward   q_j = alpha_j q_{j-1} + beta_j,  alpha_j = -c_j / den_j,
//                                              beta_j  = d_j / den_j,
//   backward  x_j = P_j x_{j+1} + q_j,          P_j = -b_j / den_j,
// so each thread composes the maps of its chunk of rows, the T threads of a
// system scan the composed maps with shuffles, the CTAs of the cluster
// exchange their composed maps through distributed shared memory, and each
// thread then replays its chunk from its incoming value.  The coefficients
// are those of the sequential Thomas solve of k_plane_walls (tdma,
// fenep_2d.f90:1145-1177); the 1/den table of the CTA's rows is staged in
// shared memory, its rows in the bit-reversed kz order of the spectrum rows.
// The cluster barriers are hardware barriers; no thread waits on a flag.
template <int V>
__global__ void __launch_bounds__(1024, 1) k_plane_walls_c(float2 *S, int ny, int cl, const float2 *twz,
                                                           WallTables wt) {
    constexpr int NZ = 32 * V;
    constexpr int LG = V == 1 ? 5 : (V == 2 ? 6 : (V == 4 ? 7 : 8));
    constexpr int T = 1024 / NZ;
    namespace cg = cooperative_groups;
    extern __shared__ unsigned char smem_raw[];
    const int lj = ny + 2;
    const int R = wall_rows_per_cta(lj, cl);
    const int rank = cl > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int kx = blockIdx.x / cl;
    const int jlo = rank * R;
    const int nr = max(0, min(R, lj - jlo));   // rows held by this CTA
    const int ps = wt.wl.ps;
    const int rs = wt.wl.rs;
    float2 *P = reinterpret_cast<float2 *>(smem_raw);                 // [k][jl]
    float *Rs = reinterpret_cast<float *>(P + (size_t)ps * NZ);       // [row][jl], row = bitrev(kz)
    float2 *tws = reinterpret_cast<float2 *>(Rs + (size_t)rs * NZ);   // NZ stage-major twiddles
    float *mapF = reinterpret_cast<float *>(tws + NZ);                // [3][NZ]: A, Bx, By
    float *mapB = mapF + 3 * NZ;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float2 *Sp = S + (size_t)kx * NZ * lj;
    const float *Rg = wt.rden + (size_t)kx * NZ * lj;
    for (int q = threadIdx.x; q < NZ; q += blockDim.x) tws[q] = twz[q];
    for (int k = warp; k < NZ; k += nwarp) {
        float *rrow = Rs + (size_t)(__brev((unsigned)k) >> (32 - LG)) * rs;
        for (int jl0 = lane; jl0 < nr; jl0 += 128) {   // four loads of each array in flight per lane
            float2 pv[4];
            float rv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int jl = jl0 + 32 * u, j = jlo + jl;
                const size_t q = (size_t)k * lj + j;
                pv[u] = (jl < nr && j >= 1 && j <= ny) ? Sp[q] : make_float2(0.f, 0.f);
                rv[u] = jl < nr ? Rg[q] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int jl = jl0 + 32 * u;
                if (jl < nr) { P[(size_t)k * ps + jl] = pv[u]; rrow[jl] = rv[u]; }
            }
        }
    }
    __syncthreads();
    for (int jl = warp; jl < nr; jl += nwarp) {
        const int j = jlo + jl;
        if (j < 1 || j > ny) continue;   // ghost rows are zero
        float2 v[V];
#pragma unroll
        for (int s = 0; s < V; ++s) v[s] = P[(size_t)(lane + 32 * s) * ps + jl];
        warp_dif_fwd<V>(v, tws, lane);
#pragma unroll
        for (int s = 0; s < V; ++s) P[(size_t)(lane + 32 * s) * ps + jl] = v[s];
    }
    __syncthreads();
    {
        const int row = threadIdx.x / T, t = threadIdx.x % T;
        float2 *x = P + (size_t)row * ps;
        const float *rd = Rs + (size_t)row * rs;
        const int L = wt.wl.L;
        const int c0 = min(nr, t * L), c1 = min(nr, c0 + L);
        const bool sysv = wt.sys == SYS_V;
        auto fwd_coef = [&](int jl, float &al, float2 &be) {
            const int j = jlo + jl;
            const bool ident = sysv ? (j >= ny) : (j == lj - 1);
            const float c = ident ? (sysv ? 0.f : wt.c_last) : wt.bc;
            const float r = j == 0 ? 0.0f : rd[jl];
            const float2 d = ident ? make_float2(0.f, 0.f) : x[jl];
            al = -c * r;
            const float dr = wt.nxz_inv * r;
            be = make_float2(d.x * dr, d.y * dr);
        };
        auto pmul = [&](int jl) {
            const int j = jlo + jl;
            const bool zero_b = (j == lj - 1) || (sysv && j >= ny);
            const float b = j == 0 ? wt.b_first : (zero_b ? 0.0f : wt.bc);
            return -b * rd[jl];
        };
        // forward: compose the chunk's maps (row 0: q_0 = 0)
        float A = 1.0f;
        float2 B = make_float2(0.f, 0.f);
        for (int jl = c0; jl < c1; ++jl) {
            float al;
            float2 be;
            fwd_coef(jl, al, be);
            B = make_float2(fmaf(al, B.x, be.x), fmaf(al, B.y, be.y));
            A *= al;
        }
#pragma unroll
        for (int o = 1; o < T; o <<= 1) {
            const float Ap = __shfl_up_sync(0xffffffffu, A, o, T);
            const float Bx = __shfl_up_sync(0xffffffffu, B.x, o, T), By = __shfl_up_sync(0xffffffffu, B.y, o, T);
            if (t >= o) { B = make_float2(fmaf(A, Bx, B.x), fmaf(A, By, B.y)); A *= Ap; }
        }
        if (t == T - 1) { mapF[row] = A; mapF[NZ + row] = B.x; mapF[2 * NZ + row] = B.y; }
        float Ae = __shfl_up_sync(0xffffffffu, A, 1, T);
        float2 Be;
        Be.x = __shfl_up_sync(0xffffffffu, B.x, 1, T);
        Be.y = __shfl_up_sync(0xffffffffu, B.y, 1, T);
        if (t == 0) { Ae = 1.0f; Be = make_float2(0.f, 0.f); }
        float2 qin = make_float2(0.f, 0.f);
        if (cl > 1) {
            cg::this_cluster().sync();
            for (int rr = 0; rr < rank; ++rr) {
                const float *m = cg::this_cluster().map_shared_rank(mapF, rr);
                const float a = m[row];
                qin = make_float2(fmaf(a, qin.x, m[NZ + row]), fmaf(a, qin.y, m[2 * NZ + row]));
            }
        }
        float2 q = make_float2(fmaf(Ae, qin.x, Be.x), fmaf(Ae, qin.y, Be.y));
        for (int jl = c0; jl < c1; ++jl) {
            float al;
            float2 be;
            fwd_coef(jl, al, be);
            q = make_float2(fmaf(al, q.x, be.x), fmaf(al, q.y, be.y));
            x[jl] = q;
        }
        // backward: x_j = P_j x_{j+1} + q_j (b and so P of the last row are 0)
        A = 1.0f;
        B = make_float2(0.f, 0.f);
        for (int jl = c1 - 1; jl >= c0; --jl) {
            const float pj = pmul(jl);
            const float2 qj = x[jl];
            B = make_float2(fmaf(pj, B.x, qj.x), fmaf(pj, B.y, qj.y));
            A *= pj;
        }
#pragma unroll
        for (int o = 1; o < T; o <<= 1) {
            const float An = __shfl_down_sync(0xffffffffu, A, o, T);
            const float Bx = __shfl_down_sync(0xffffffffu, B.x, o, T), By = __shfl_down_sync(0xffffffffu, B.y, o, T);
            if (t + o < T) { B = make_float2(fmaf(A, Bx, B.x), fmaf(A, By, B.y)); A *= An; }
        }
        if (t == 0) { mapB[row] = A; mapB[NZ + row] = B.x; mapB[2 * NZ + row] = B.y; }
        Ae = __shfl_down_sync(0xffffffffu, A, 1, T);
        Be.x = __shfl_down_sync(0xffffffffu, B.x, 1, T);
        Be.y = __shfl_down_sync(0xffffffffu, B.y, 1, T);
        if (t == T - 1) { Ae = 1.0f; Be = make_float2(0.f, 0.f); }
        float2 xin = make_float2(0.f, 0.f);
        if (cl > 1) {
            cg::this_cluster().sync();
            for (int rr = cl - 1; rr > rank; --rr) {
                const float *m = cg::this_cluster().map_shared_rank(mapB, rr);
                const float a = m[row];
                xin = make_float2(fmaf(a, xin.x, m[NZ + row]), fmaf(a, xin.y, m[2 * NZ + row]));
            }
        }
        float2 xv = make_float2(fmaf(Ae, xin.x, Be.x), fmaf(Ae, xin.y, Be.y));
        for (int jl = c1 - 1; jl >= c0; --jl) {
            const float pj = pmul(jl);
            const float2 qj = x[jl];
            xv = make_float2(fmaf(pj, xv.x, qj.x), fmaf(pj, xv.y, qj.y));
            x[jl] = xv;
        }
    }
    // the other CTAs' reads of this CTA's maps are complete past this barrier
    if (cl > 1) cg::this_cluster().sync();
    else __syncthreads();
    for (int jl = warp; jl < nr; jl += nwarp) {
        float2 v[V];
#pragma unroll
        for (int s = 0; s < V; ++s) v[s] = P[(size_t)(lane + 32 * s) * ps + jl];
        warp_dit_inv<V>(v, tws, lane);
#pragma unroll
        for (int s = 0; s < V; ++s) P[(size_t)(lane + 32 * s) * ps + jl] = v[s];
    }
    __syncthreads();
    for (int k = warp; k < NZ; k += nwarp)
        for (int jl = lane; jl < nr; jl += 32) Sp[(size_t)k * lj + jlo + jl] = P[(size_t)k * ps + jl];
}

}  // namespace f8
