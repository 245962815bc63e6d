// f8_fft.cuh — batched radix-2 Stockham FFT kernels and the wall-normal
// tridiagonal solve, templated on the real type.
//
// Replaces FFTW (fft_solve, fenep.f90:1400-1428; fenep_2d.f90:841-867) and the
// Thomas solver tdma (fenep_2d.f90:1145-1177).  Every butterfly is written in
// the same order as the CPU oracle's Stockham loop, so the FP64 instantiation
// compiled without FMA contraction reproduces the oracle bit for bit.
//
// Spectral layout: complex values interleaved (re, im), [k][j][kx] with
// kx = 0..NX/2 (NXH = NX/2+1 values per row).
#pragma once
#include "f8_common.cuh"
#include "f8_df64.cuh"

namespace f8 {

template <typename T>
struct Cx { T r, i; };

// One Stockham pass set over a line held in shared memory.  x and y are two
// buffers of n complex values; t is the butterfly index (0..n/2-1) owned by the
// calling thread; nthr threads cooperate on several lines: the caller passes
// line-local pointers.  Returns the buffer that holds the result.
//   tw: forward twiddles exp(-2 pi i t/n), t < n/2 (re, im arrays)
template <typename T>
__device__ inline void stockham_stage(const Cx<T> *x, Cx<T> *y, int n, int ns, int j, const T *twr, const T *twi,
                                      int sign) {
    const int half = n >> 1;
    const int kk = j % ns;
    const int stride = n / (2 * ns);
    T wr = twr[kk * stride];
    T wi = sign < 0 ? twi[kk * stride] : -twi[kk * stride];
    Cx<T> a = x[j], b = x[j + half];
    T tr = b.r * wr - b.i * wi;
    T ti = b.r * wi + b.i * wr;
    int o = (j / ns) * 2 * ns + kk;
    y[o].r = a.r + tr; y[o].i = a.i + ti;
    y[o + ns].r = a.r - tr; y[o + ns].i = a.i - ti;
}

// ---------------------------------------------------------------------------
// x direction, real <-> half spectrum, two rows per complex transform.
//
// Forward: rows (j0 + jj, j0 + jj + 1) of plane k of the interior-ordered
// source src (row length n, nrow_src rows per plane) become spectral rows
// jj, jj+1 of H (nrow_h rows per plane).  One CTA handles ppc row pairs with
// n/2 threads each.
template <typename T, typename TS>
__global__ void k_fft_x_fwd(const TS *__restrict__ src, T *__restrict__ H, int n, int nrow_src, int j0, int nrow_h,
                            int npairs_per_plane, int nplanes, const T *__restrict__ twr, const T *__restrict__ twi) {
    extern __shared__ unsigned char smem_raw[];
    Cx<T> *sm = reinterpret_cast<Cx<T> *>(smem_raw);
    const int half = n >> 1;
    const int tpp = half > 0 ? half : 1;
    const int ppc = blockDim.x / tpp;
    const int p = threadIdx.x / tpp, t = threadIdx.x % tpp;
    const long pair = (long)blockIdx.x * ppc + p;
    const bool active = pair < (long)npairs_per_plane * nplanes;
    Cx<T> *x = sm + (size_t)p * 2 * n, *y = x + n;
    int k = 0, jj = 0;
    if (active) {
        k = (int)(pair / npairs_per_plane);
        jj = 2 * (int)(pair % npairs_per_plane);
        const TS *ra = src + (size_t)n * ((size_t)(j0 + jj - 1) + (size_t)nrow_src * k);
        const TS *rb = ra + n;
        for (int e = t; e < n; e += tpp) { x[e].r = T(ra[e]); x[e].i = T(rb[e]); }
    }
    __syncthreads();
    for (int ns = 1; ns < n; ns *= 2) {
        if (active && t < half) stockham_stage(x, y, n, ns, t, twr, twi, -1);
        __syncthreads();
        Cx<T> *tmp = x; x = y; y = tmp;
    }
    if (!active) return;
    const int nxh = half + 1;
    T *ha = H + 2 * ((size_t)nxh * ((size_t)jj + (size_t)nrow_h * k));
    T *hb = ha + 2 * nxh;
    for (int kx = t; kx < nxh; kx += tpp) {
        int m = (n - kx) % n;
        Cx<T> zk = x[kx], zm = x[m];
        ha[2 * kx] = (zk.r + zm.r) * T(0.5);
        ha[2 * kx + 1] = (zk.i - zm.i) * T(0.5);
        hb[2 * kx] = (zk.i + zm.i) * T(0.5);
        hb[2 * kx + 1] = (zm.r - zk.r) * T(0.5);
    }
}

// Destinations of an inverse x pass.  XOutD: an FP64 field, optionally the
// sum base + value (FP64 path and stand-alone solve).  XOutF: the FP32 /
// double-float fields of the mixed path (modes below).
struct XOutD {
    double *dst;
    const double *base;
    __device__ __forceinline__ void put(size_t o, double v) const { dst[o] = base ? base[o] + v : v; }
};

struct XOutF {
    float *hi, *lo;
    int mode;
    // mode 0: hi = v.  mode 2: (hi, lo) = hi + v exactly (two-sum), the
    // correction of an FP32 field to a df64 pair
    __device__ __forceinline__ void put(size_t o, float v) const {
        if (mode == 0) {
            hi[o] = v;
        } else {
            float s, e;
            two_sum(hi[o], v, s, e);
            hi[o] = s;
            lo[o] = e;
        }
    }
};

// Inverse: spectral rows jj, jj+1 (nrow_h per plane) -> real rows jdst0 + jj,
// jdst0 + jj + 1 of a halo-layout field (x written at 1..n) through the
// destination functor.
template <typename T, typename Out>
__global__ void k_fft_x_inv(const T *__restrict__ H, Out out, int n, int nrow_h, int npairs_per_plane,
                            int nplanes, int jdst0, int sx, int sy, const T *__restrict__ twr, const T *__restrict__ twi,
                            int plain = 0) {
    extern __shared__ unsigned char smem_raw[];
    Cx<T> *sm = reinterpret_cast<Cx<T> *>(smem_raw);
    const int half = n >> 1;
    const int tpp = half > 0 ? half : 1;
    const int ppc = blockDim.x / tpp;
    const int p = threadIdx.x / tpp, t = threadIdx.x % tpp;
    const long pair = (long)blockIdx.x * ppc + p;
    const bool active = pair < (long)npairs_per_plane * nplanes;
    Cx<T> *x = sm + (size_t)p * 2 * n, *y = x + n;
    int k = 0, jj = 0;
    const int nxh = half + 1;
    if (active) {
        k = (int)(pair / npairs_per_plane);
        jj = 2 * (int)(pair % npairs_per_plane);
        const T *ha = H + 2 * ((size_t)nxh * ((size_t)jj + (size_t)nrow_h * k));
        const T *hb = ha + 2 * nxh;
        for (int e = t; e < n; e += tpp) {
            if (e <= half) {
                T ar = ha[2 * e], ai = ha[2 * e + 1], br = hb[2 * e], bi = hb[2 * e + 1];
                x[e].r = ar - bi; x[e].i = ai + br;
            } else {
                int m = n - e;
                T ar = ha[2 * m], ai = ha[2 * m + 1], br = hb[2 * m], bi = hb[2 * m + 1];
                x[e].r = ar + bi; x[e].i = br - ai;
            }
        }
    }
    __syncthreads();
    for (int ns = 1; ns < n; ns *= 2) {
        if (active && t < half) stockham_stage(x, y, n, ns, t, twr, twi, +1);
        __syncthreads();
        Cx<T> *tmp = x; x = y; y = tmp;
    }
    if (!active) return;
    // halo layout (x at 1..n) or, with plain, a dense [k][j][x] array of
    // row length n and sy rows per plane
    const size_t oa = plain ? (size_t)n * ((size_t)(jdst0 + jj) + (size_t)sy * k)
                            : 1 + (size_t)sx * ((size_t)(jdst0 + jj) + (size_t)sy * (k + 1));
    const size_t ob = oa + (plain ? n : sx);
    for (int e = t; e < n; e += tpp) { out.put(oa + e, x[e].r); out.put(ob + e, x[e].i); }
}

// ---------------------------------------------------------------------------
// Strided complex transforms along y or z of the half spectrum.  A CTA owns tx
// consecutive kx columns of one line set and keeps [n][tx] complex values in
// shared memory (so global reads are row segments of tx complex values).
//   line element e of column c: H[base + e*lstride + c]  (complex units)
//   base = set*sstride + kx0
// mode 0: single transform with sign; mode 1: forward, spectral divide,
// inverse (periodic solve, fenep.f90:1408-1426); the divide needs the
// modified-wavenumber tables and the line index of the other axes.
struct DivideSpec {
    const double *kx2, *ky2, *kz2;  // tables (FP64)
    double lhs0, lhs1, ntot;        // LHS = lhs0 + lhs1*((kx2+ky2)+kz2); Q/ntot/LHS
    int line_is_z;                  // 1: line along z (set = j); 0: along y (set = k)
};

template <typename T>
__global__ void k_fft_lines(T *__restrict__ H, int n, int lstride, int ncols, int sstride, int tx,
                            const T *__restrict__ twr, const T *__restrict__ twi, int sign, int mode, DivideSpec dv) {
    extern __shared__ unsigned char smem_raw[];
    Cx<T> *bufA = reinterpret_cast<Cx<T> *>(smem_raw);
    Cx<T> *bufB = bufA + (size_t)n * tx;
    const int set = blockIdx.y;
    const int kx0 = blockIdx.x * tx;
    const int ncol = min(tx, ncols - kx0);
    Cx<T> *Hc = reinterpret_cast<Cx<T> *>(H);
    const size_t base = (size_t)set * sstride + kx0;
    // load: element (e, c) -> buf[c*n + e]
    for (int q = threadIdx.x; q < n * tx; q += blockDim.x) {
        int e = q / tx, c = q % tx;
        if (c < ncol) bufA[(size_t)c * n + e] = Hc[base + (size_t)e * lstride + c];
    }
    __syncthreads();
    const int half = n >> 1;
    const int nbfly = half * tx;
    int passes = mode == 1 ? 2 : 1;
    Cx<T> *x = bufA, *y = bufB;
    for (int ps = 0; ps < passes; ++ps) {
        const int sg = mode == 1 ? (ps == 0 ? -1 : +1) : sign;
        for (int ns = 1; ns < n; ns *= 2) {
            for (int q = threadIdx.x; q < nbfly; q += blockDim.x) {
                int c = q / half, j = q % half;
                if (c < ncol) stockham_stage(x + (size_t)c * n, y + (size_t)c * n, n, ns, j, twr, twi, sg);
            }
            __syncthreads();
            Cx<T> *tmp = x; x = y; y = tmp;
        }
        if (mode == 1 && ps == 0) {
            for (int q = threadIdx.x; q < n * tx; q += blockDim.x) {
                int c = q / n, e = q % n;
                if (c >= ncol) continue;
                int kx = kx0 + c;
                // element e of the line: along z -> kz = e, ky = set; along y -> ky = e, kz = set
                int jy = dv.line_is_z ? set : e;
                int kz = dv.line_is_z ? e : set;
                double lhs = dv.lhs0 + dv.lhs1 * (dv.kx2[kx] + dv.ky2[jy] + dv.kz2[kz]);
                Cx<T> v = x[(size_t)c * n + e];
                T qr = v.r / T(dv.ntot), qi = v.i / T(dv.ntot);
                if (fabs(lhs) < 1.0e-16) { v.r = T(0); v.i = T(0); }
                else { v.r = qr / T(lhs); v.i = qi / T(lhs); }
                x[(size_t)c * n + e] = v;
            }
            __syncthreads();
        }
    }
    for (int q = threadIdx.x; q < n * tx; q += blockDim.x) {
        int e = q / tx, c = q % tx;
        if (c < ncol) Hc[base + (size_t)e * lstride + c] = x[(size_t)c * n + e];
    }
}

// ---------------------------------------------------------------------------
// Wall-normal systems (fenep_2d.f90:1222-1238, 1262-1277, 1318-1332 with
// NA = 0, NB = NY; x and z periodic).  Input spectrum Hin has rows j = 1..NY
// (ny rows per plane), output Hout rows j = 0..NY+1 (ny+2 rows per plane).
// One thread per kx column runs the Thomas recurrence of tdma with the
// reference's near-zero-pivot guard; the real coefficient recurrence P and the
// complex right-hand side share shared memory.
enum WallSys { SYS_U = 0, SYS_V = 1, SYS_P = 2 };

struct WallSpec {
    const double *kx2, *kz2;
    double dt, beta, re, dy;
    double nxz;     // NX*NZ normalisation of the forward transforms
    double uwall;   // 2*uwall on the top ghost row of mode (0,0) for SYS_U
    int sys;
};

template <typename T>
__device__ inline void wall_coef(const WallSpec &w, int sys, int j, int ny, double lam, T &a, T &b, T &c) {
    const int n = ny + 2;
    if (sys == SYS_U) {
        if (j == 0) { a = T(1.0); b = T(1.0); c = T(0.0); }
        else if (j == n - 1) { a = T(1.0); b = T(0.0); c = T(1.0); }
        else {
            a = T(1.0 + w.dt * w.beta / w.re / 2.0 * (lam + 2.0 / (w.dy * w.dy)));
            b = T(-w.dt * w.beta / w.re / 2.0 / (w.dy * w.dy));
            c = b;
        }
    } else if (sys == SYS_V) {
        if (j == 0 || j >= ny) { a = T(1.0); b = T(0.0); c = T(0.0); }
        else {
            a = T(1.0 + w.dt * w.beta / w.re / 2.0 * (lam + 2.0 / (w.dy * w.dy)));
            b = T(-w.dt * w.beta / w.re / 2.0 / (w.dy * w.dy));
            c = b;
        }
    } else {
        if (j == 0) { a = T(1.0); b = T(-1.0); c = T(0.0); }
        else if (j == n - 1) { a = T(1.0); b = T(0.0); c = T(-1.0); }
        else {
            a = T(-(lam + 2.0 / (w.dy * w.dy)));
            b = T(1.0 / (w.dy * w.dy));
            c = b;
        }
    }
}

template <typename T>
__global__ void k_wall_tdma(const T *__restrict__ Hin, T *__restrict__ Hout, int ny, int nxh, int tx, WallSpec w) {
    extern __shared__ unsigned char smem_raw[];
    const int n = ny + 2;
    Cx<T> *q = reinterpret_cast<Cx<T> *>(smem_raw);       // [n][tx] rhs, then Q
    T *P = reinterpret_cast<T *>(q + (size_t)n * tx);       // [n][tx]
    const int kz = blockIdx.y;
    const int kx0 = blockIdx.x * tx;
    const int ncol = min(tx, nxh - kx0);
    const Cx<T> *Hi = reinterpret_cast<const Cx<T> *>(Hin);
    Cx<T> *Ho = reinterpret_cast<Cx<T> *>(Hout);
    for (int e = threadIdx.x; e < n * tx; e += blockDim.x) {
        int j = e / tx, c = e % tx;
        if (c >= ncol) continue;
        Cx<T> v;
        if (j >= 1 && j <= ny && !(w.sys == SYS_V && j == ny)) {
            Cx<T> h = Hi[(size_t)nxh * ((size_t)(j - 1) + (size_t)ny * kz) + kx0 + c];
            v.r = h.r / T(w.nxz); v.i = h.i / T(w.nxz);
        } else {
            v.r = T(0); v.i = T(0);
            if (w.sys == SYS_U && j == n - 1 && kx0 + c == 0 && kz == 0) v.r = T(2 * w.uwall);
        }
        q[(size_t)j * tx + c] = v;
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c < ncol) {
        const double lam = w.kx2[kx0 + c] + w.kz2[kz];
        T a, b, cc;
        wall_coef<T>(w, w.sys, 0, ny, lam, a, b, cc);
        Cx<T> d = q[c];
        T p = -b / a;
        Cx<T> Q; Q.r = d.r / a; Q.i = d.i / a;
        P[c] = p; q[c] = Q;
        for (int j = 1; j < n; ++j) {
            wall_coef<T>(w, w.sys, j, ny, lam, a, b, cc);
            d = q[(size_t)j * tx + c];
            T den = a + cc * p;
            if (fabs(den) < T(1.0e-16)) { p = T(0); Q.r = T(0); Q.i = T(0); }
            else {
                p = -b / den;
                Q.r = (d.r - cc * Q.r) / den;
                Q.i = (d.i - cc * Q.i) / den;
            }
            P[(size_t)j * tx + c] = p;
            q[(size_t)j * tx + c] = Q;
        }
        Cx<T> x = q[(size_t)(n - 1) * tx + c];
        for (int j = n - 2; j >= 0; --j) {
            T pj = P[(size_t)j * tx + c];
            Cx<T> qj = q[(size_t)j * tx + c];
            x.r = pj * x.r + qj.r;
            x.i = pj * x.i + qj.i;
            q[(size_t)j * tx + c] = x;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * tx; e += blockDim.x) {
        int j = e / tx, cc2 = e % tx;
        if (cc2 >= ncol) continue;
        Ho[(size_t)nxh * ((size_t)j + (size_t)n * kz) + kx0 + cc2] = q[(size_t)j * tx + cc2];
    }
}

}  // namespace f8
