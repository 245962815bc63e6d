// f8_diag.cu — on-device reductions of log_progress (fenep.f90:2266-2342) plus
// the divergence residual: kinetic energy on the cell centres, CFL from the
// maxima of U, V, W over the whole halo field, trC minimum / maximum / mean /
// standard deviation (the reference's two-pass form, mean first), max |div u|
// and a NaN flag.  Deterministic: a grid of 4 blocks per SM (fixed for a
// device) accumulates grid-stride partials per thread, a block tree reduces
// them, and one block reduces the block partials in a fixed order.  Both precisions: the
// FP64 state, or the double-float state and FP32 C of the mixed path.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include "f8_common.cuh"
#include "f8_kernels.h"

namespace f8 {
namespace {

constexpr int DIAG_THREADS = 256;

struct DiagIn {
    const double *U, *V, *W;                  // FP64 state (null in mixed)
    const float *Uh, *Ul, *Vh, *Vl, *Wh, *Wl; // double-float state (mixed)
    const double *C;                          // FP64 C (SoA), or
    const float *Cf;                          // FP32 C (SoA)
    int cs, d3, mixed;
    double idx, idy, idz;
};

}  // namespace

static __device__ double slice_vel(const DiagSliceIn &in, int c, int q) {
    if (in.mixed) {
        const float *h = c == 0 ? in.Uh : (c == 1 ? in.Vh : in.Wh);
        const float *l = c == 0 ? in.Ul : (c == 1 ? in.Vl : in.Wl);
        return (double)h[q] + (double)l[q];
    }
    return (c == 0 ? in.U : (c == 1 ? in.V : in.W))[q];
}

static __device__ double slice_c(const DiagSliceIn &in, int m, int q) {
    return in.mixed ? (double)in.Cf[(size_t)m * in.cs + q] : in.C[(size_t)m * in.cs + q];
}

namespace {

__device__ inline double vel(const DiagIn &in, int c, int q) {
    if (in.mixed) {
        const float *h = c == 0 ? in.Uh : (c == 1 ? in.Vh : in.Wh);
        const float *l = c == 0 ? in.Ul : (c == 1 ? in.Vl : in.Wl);
        return (double)h[q] + (double)l[q];
    }
    return (c == 0 ? in.U : (c == 1 ? in.V : in.W))[q];
}

__device__ inline double ccomp(const DiagIn &in, int m, int q) {
    return in.mixed ? (double)in.Cf[(size_t)m * in.cs + q] : in.C[(size_t)m * in.cs + q];
}

__device__ inline double trace_at(const DiagIn &in, int q) {
    return in.d3 ? ccomp(in, 0, q) + ccomp(in, 3, q) + ccomp(in, 5, q) : ccomp(in, 0, q) + ccomp(in, 2, q);
}

// block reductions over DIAG_THREADS threads (fixed tree order)
template <typename Op>
__device__ inline double block_reduce(double v, double *sh, Op op) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = DIAG_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = op(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

struct Add { __device__ double operator()(double a, double b) const { return a + b; } };
struct Max { __device__ double operator()(double a, double b) const { return a > b ? a : b; } };
struct Min { __device__ double operator()(double a, double b) const { return a < b ? a : b; } };

enum { P_KE, P_TSUM, P_TMIN, P_TMAX, P_DIV, P_UMAX, P_VMAX, P_WMAX, P_NAN, P_N };

// pass 1: partials per block
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_pass1(DiagIn in, Geo g, double *part) {
    __shared__ double sh[DIAG_THREADS];
    const long ni = (long)g.nx * g.ny * g.nz;
    double ke = 0.0, tsum = 0.0, tmin = DBL_MAX, tmax = -DBL_MAX, dmax = 0.0, nan = 0.0;
    for (long t = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; t < ni; t += (long)gridDim.x * DIAG_THREADS) {
        const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
        const int h = hix(g, i, j, k);
        const double u0 = vel(in, 0, h), u1 = vel(in, 0, h - 1);
        const double v0 = vel(in, 1, h), v1 = vel(in, 1, h - g.sx);
        const double ur = (u0 + u1) / 2.0, vr = (v0 + v1) / 2.0;
        double wr = 0.0, dv = (u0 - u1) * in.idx + (v0 - v1) * in.idy;
        if (in.d3) {
            const double w0 = vel(in, 2, h), w1 = vel(in, 2, h - g.sx * g.sy);
            wr = (w0 + w1) / 2.0;
            dv += (w0 - w1) * in.idz;
        }
        ke += ur * ur + vr * vr + wr * wr;
        const double tr = trace_at(in, h);
        tsum += tr;
        tmin = tr < tmin ? tr : tmin;
        tmax = tr > tmax ? tr : tmax;
        dmax = fabs(dv) > dmax ? fabs(dv) : dmax;
        if (isnan(ur) || isnan(vr) || isnan(wr)) nan = 1.0;
    }
    double umax = -DBL_MAX, vmax = -DBL_MAX, wmax = -DBL_MAX;
    for (long q = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; q < in.cs; q += (long)gridDim.x * DIAG_THREADS) {
        umax = fmax(umax, vel(in, 0, (int)q));
        vmax = fmax(vmax, vel(in, 1, (int)q));
        if (in.d3) wmax = fmax(wmax, vel(in, 2, (int)q));
    }
    double *p = part + (size_t)blockIdx.x * P_N;
    const double r[P_N] = {block_reduce(ke, sh, Add()),   block_reduce(tsum, sh, Add()),
                           block_reduce(tmin, sh, Min()), block_reduce(tmax, sh, Max()),
                           block_reduce(dmax, sh, Max()), block_reduce(umax, sh, Max()),
                           block_reduce(vmax, sh, Max()), block_reduce(wmax, sh, Max()),
                           block_reduce(nan, sh, Max())};
    if (threadIdx.x == 0)
        for (int m = 0; m < P_N; ++m) p[m] = r[m];
}

// pass 2: sum of (trC - mean)^2 per block, mean = out[P_TSUM] / N
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_pass2(DiagIn in, Geo g, const double *out, double *part) {
    __shared__ double sh[DIAG_THREADS];
    const long ni = (long)g.nx * g.ny * g.nz;
    const double mean = out[P_TSUM] / (double)ni;
    double s = 0.0;
    for (long t = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; t < ni; t += (long)gridDim.x * DIAG_THREADS) {
        const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
        const double d = trace_at(in, hix(g, i, j, k)) - mean;
        s += d * d;
    }
    const double r = block_reduce(s, sh, Add());
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// final: one block reduces the block partials (stride np per block) in order
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_final(const double *part, int nb, int np, int nv, double *out) {
    __shared__ double sh[DIAG_THREADS];
    for (int m = 0; m < nv; ++m) {
        const bool mx = m == P_TMAX || m == P_DIV || m == P_UMAX || m == P_VMAX || m == P_WMAX || m == P_NAN;
        const bool mn = m == P_TMIN;
        double v = mn ? DBL_MAX : (mx ? -DBL_MAX : 0.0);
        for (int b = threadIdx.x; b < nb; b += DIAG_THREADS) {
            const double x = part[(size_t)b * np + m];
            v = mn ? fmin(v, x) : (mx ? fmax(v, x) : v + x);
        }
        const double r = mn ? block_reduce(v, sh, Min()) : (mx ? block_reduce(v, sh, Max()) : block_reduce(v, sh, Add()));
        if (threadIdx.x == 0) out[m] = r;
    }
}

}  // namespace

cudaError_t device_diagnostics(Dev &d, bool mixed, double *part, double *out, DiagValues *res, cudaStream_t s) {
    const Geo &g = d.g;
    DiagIn in{};
    in.cs = d.cs;
    in.d3 = g.dim == 3;
    in.mixed = mixed ? 1 : 0;
    in.idx = 1.0 / g.dx; in.idy = 1.0 / g.dy; in.idz = 1.0 / g.dz;
    if (mixed) {
        in.Uh = d.Uf; in.Ul = d.Ul; in.Vh = d.Vf; in.Vl = d.Vl; in.Wh = d.Wf; in.Wl = d.Wl;
        in.Cf = d.Cf;
    } else {
        in.U = d.U; in.V = d.V; in.W = d.W;
        in.C = d.C;
    }
    const int nb = diag_blocks();
    k_diag_pass1<<<nb, DIAG_THREADS, 0, s>>>(in, g, part); count_launch();
    k_diag_final<<<1, DIAG_THREADS, 0, s>>>(part, nb, P_N, P_N, out); count_launch();
    k_diag_pass2<<<nb, DIAG_THREADS, 0, s>>>(in, g, out, part); count_launch();
    k_diag_final<<<1, DIAG_THREADS, 0, s>>>(part, nb, 1, 1, out + P_N); count_launch();
    double h[P_N + 1];
    F8_CUDA_RET(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
    F8_CUDA_RET(cudaStreamSynchronize(s));
    const double N = (double)g.nx * g.ny * g.nz;
    res->ke = h[P_KE] / 2.0 / N;
    double cfl = std::max(h[P_UMAX] * g.dt / g.dx, h[P_VMAX] * g.dt / g.dy);
    if (g.dim == 3) cfl = std::max(cfl, h[P_WMAX] * g.dt / g.dz);
    res->cfl = cfl * 6.0;
    res->trc_min = h[P_TMIN];
    res->trc_max = h[P_TMAX];
    res->trc_mean = h[P_TSUM] / N;
    res->trc_std = std::sqrt(h[P_N] / N);
    res->div_max = h[P_DIV];
    res->nan_found = h[P_NAN] > 0.0 ? 1 : 0;
    return cudaGetLastError();
}

int device_sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 152;
        }
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

size_t diag_partials() { return (size_t)diag_blocks() * P_N; }

}  // namespace f8

// ---------------------------------------------------------------------------
// Slice output of get_data_binary (fenep.f90:1108-1183, fenep_mpi.f90:811-937):
// per point of the mid-plane slice, 18 doubles x, y, z, E (3), KE or Q,
// Omega (3), |Omega|^2/2, trC, C (6), with the velocity gradient D of the
// reference's staggered differences.  The reference's nondimensional scales
// U_C = L_C = 1 (fenep.f90:28-29) are used, so dX_C = dX.
namespace f8 {
namespace {

__global__ void k_slice(DiagSliceIn in, Geo g, int axis, int variant, double *out) {
    const int n1 = axis == 0 ? g.ny : g.nx;          // inner loop length
    const int n2 = axis == 2 ? g.ny : g.nz;          // outer loop length
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2) return;
    const int a = t % n1, b = t / n1;
    int i, j, k;
    if (axis == 2) { k = g.nz / 2; j = 1 + b; i = 1 + a; }
    else if (axis == 1) { j = g.ny / 2; k = 1 + b; i = 1 + a; }
    else { i = g.nx / 2; k = 1 + b; j = 1 + a; }
    auto U = [&](int ii, int jj, int kk) { return slice_vel(in, 0, hix(g, ii, jj, kk)); };
    auto V = [&](int ii, int jj, int kk) { return slice_vel(in, 1, hix(g, ii, jj, kk)); };
    auto W = [&](int ii, int jj, int kk) { return slice_vel(in, 2, hix(g, ii, jj, kk)); };
    const double dX = g.dx, dY = g.dy, dZ = g.dz;
    double D[3][3];
    D[0][0] = (U(i, j, k) - U(i - 1, j, k)) / dX;
    D[0][1] = (U(i, j + 1, k) - U(i, j - 1, k) + U(i - 1, j + 1, k) - U(i - 1, j - 1, k)) / (4 * dY);
    D[0][2] = (U(i, j, k + 1) - U(i, j, k - 1) + U(i - 1, j, k + 1) - U(i - 1, j, k - 1)) / (4 * dZ);
    D[1][0] = (V(i + 1, j, k) - V(i - 1, j, k) + V(i + 1, j - 1, k) - V(i - 1, j - 1, k)) / (4 * dX);
    D[1][1] = (V(i, j, k) - V(i, j - 1, k)) / dY;
    D[1][2] = (V(i, j, k + 1) - V(i, j, k - 1) + V(i, j - 1, k + 1) - V(i, j - 1, k - 1)) / (4 * dZ);
    D[2][0] = (W(i + 1, j, k) - W(i - 1, j, k) + W(i + 1, j, k - 1) - W(i - 1, j, k - 1)) / (4 * dX);
    D[2][1] = (W(i, j + 1, k) - W(i, j - 1, k) + W(i, j + 1, k - 1) - W(i, j - 1, k - 1)) / (4 * dY);
    D[2][2] = (W(i, j, k) - W(i, j, k - 1)) / dZ;
    const double E0 = (U(i - 1, j, k) + U(i, j, k)) / 2, E1 = (V(i, j - 1, k) + V(i, j, k)) / 2,
                 E2 = (W(i, j, k - 1) + W(i, j, k)) / 2;
    const double O0 = D[2][1] - D[1][2], O1 = D[0][2] - D[2][0], O2 = D[1][0] - D[0][1];
    const double Q = D[1][1] * D[2][2] - D[2][1] * D[1][2] + D[0][0] * D[1][1] - D[1][0] * D[0][1]
                   + D[0][0] * D[2][2] - D[2][0] * D[0][2];
    const int h = hix(g, i, j, k);
    double c[6];
    for (int m = 0; m < 6; ++m) c[m] = slice_c(in, m, h);
    double *o = out + (size_t)t * 18;
    o[0] = (i - 0.5) * dX; o[1] = (j - 0.5) * dY; o[2] = (k - 0.5) * dZ;
    o[3] = E0; o[4] = E1; o[5] = E2;
    o[6] = variant == 1 ? Q : (E0 * E0 + E1 * E1 + E2 * E2) / 2;
    o[7] = O0; o[8] = O1; o[9] = O2;
    o[10] = (O0 * O0 + O1 * O1 + O2 * O2) / 2;
    o[11] = c[0] + c[3] + c[5];
    for (int m = 0; m < 6; ++m) o[12 + m] = c[m];
}

}  // namespace

int slice_points(const Geo &g, int axis) {
    return axis == 2 ? g.nx * g.ny : (axis == 1 ? g.nx * g.nz : g.ny * g.nz);
}

cudaError_t device_slice(Dev &d, bool mixed, int axis, int variant, double *dev_out, cudaStream_t s) {
    DiagSliceIn in{};
    in.cs = d.cs;
    in.mixed = mixed ? 1 : 0;
    if (mixed) {
        in.Uh = d.Uf; in.Ul = d.Ul; in.Vh = d.Vf; in.Vl = d.Vl; in.Wh = d.Wf; in.Wl = d.Wl;
        in.Cf = d.Cf;
    } else {
        in.U = d.U; in.V = d.V; in.W = d.W;
        in.C = d.C;
    }
    const int n = slice_points(d.g, axis);
    k_slice<<<(n + 127) / 128, 128, 0, s>>>(in, d.g, axis, variant, dev_out); count_launch();
    return cudaGetLastError();
}

}  // namespace f8

// ---------------------------------------------------------------------------
// Turbulence statistics of all_time_dif (fenep_mpi.f90:2200-2348) and the
// energy spectrum of energy_single / fft_energy_dif (fenep.f90:1606-1672,
// fenep_mpi.f90:2567-2667), with U_C = L_C = 1 and nu = 1/Re.  The velocity
// fluctuation U - <U> (the mean is optional) has the periodic boundary values
// the reference gives it (PBM), i.e. neighbours wrap in every direction.
#include "f8_fft.cuh"

namespace f8 {
namespace {

struct TurbIn {
    DiagSliceIn st;
    const double *mean[3];   // interior mean fields, or null
    int d3;
};

__device__ inline double fluct(const TurbIn &in, const Geo &g, int c, int i, int j, int k) {
    i = wrapx(g, i); j = wrapy(g, j); k = wrapz(g, k);
    double v = slice_vel(in.st, c, hix(g, i, j, k));
    if (in.mean[c]) v -= in.mean[c][qix(g, i, j, k)];
    return v;
}

enum { T_U2, T_V2, T_W2, T_GU, T_GV, T_GW, T_S2, T_KS, T_EP, T_N };

__global__ void __launch_bounds__(DIAG_THREADS) k_turb_pass(TurbIn in, Geo g, double dep, double lp2, double *part) {
    __shared__ double sh[DIAG_THREADS];
    const long ni = (long)g.nx * g.ny * g.nz;
    double a[T_N] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double dX = g.dx, dY = g.dy, dZ = g.dz;
    for (long t = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; t < ni; t += (long)gridDim.x * DIAG_THREADS) {
        const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
        auto U = [&](int ii, int jj, int kk) { return fluct(in, g, 0, ii, jj, kk); };
        auto V = [&](int ii, int jj, int kk) { return fluct(in, g, 1, ii, jj, kk); };
        auto W = [&](int ii, int jj, int kk) { return fluct(in, g, 2, ii, jj, kk); };
        const double ur = (U(i, j, k) + U(i - 1, j, k)) / 2.0, vr = (V(i, j, k) + V(i, j - 1, k)) / 2.0,
                     wr = (W(i, j, k) + W(i, j, k - 1)) / 2.0;
        a[T_U2] += ur * ur; a[T_V2] += vr * vr; a[T_W2] += wr * wr;
        const double gu = (U(i, j, k) - U(i - 1, j, k)) / dX, gv = (V(i, j, k) - V(i, j - 1, k)) / dY,
                     gw = (W(i, j, k) - W(i, j, k - 1)) / dZ;
        a[T_GU] += gu * gu; a[T_GV] += gv * gv; a[T_GW] += gw * gw;
        double D[3][3];
        D[0][0] = gu;
        D[0][1] = (U(i, j + 1, k) - U(i, j - 1, k) + U(i - 1, j + 1, k) - U(i - 1, j - 1, k)) / (4 * dY);
        D[0][2] = (U(i, j, k + 1) - U(i, j, k - 1) + U(i - 1, j, k + 1) - U(i - 1, j, k - 1)) / (4 * dZ);
        D[1][0] = (V(i + 1, j, k) - V(i - 1, j, k) + V(i + 1, j - 1, k) - V(i - 1, j - 1, k)) / (4 * dX);
        D[1][1] = gv;
        D[1][2] = (V(i, j, k + 1) - V(i, j, k - 1) + V(i, j - 1, k + 1) - V(i, j - 1, k - 1)) / (4 * dZ);
        D[2][0] = (W(i + 1, j, k) - W(i - 1, j, k) + W(i + 1, j, k - 1) - W(i - 1, j, k - 1)) / (4 * dX);
        D[2][1] = (W(i, j + 1, k) - W(i, j - 1, k) + W(i, j + 1, k - 1) - W(i, j - 1, k - 1)) / (4 * dY);
        D[2][2] = gw;
        double s2 = 0.0;
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) {
                const double sv = D[p][q] + D[q][p];
                s2 += sv * sv;
            }
        a[T_S2] += s2;
        const int h = hix(g, i, j, k);
        const double us = slice_vel(in.st, 0, h), vs = slice_vel(in.st, 1, h), ws = slice_vel(in.st, 2, h);
        a[T_KS] += us * us + vs * vs + ws * ws;
        // elastic energy 0.5 (1-beta)/(Re Wi) (L^2-3) log f(C)
        const double tr = slice_c(in.st, 0, h) + slice_c(in.st, 3, h) + slice_c(in.st, 5, h);
        a[T_EP] += dep * log((lp2 - 3.0) / (lp2 - tr));
    }
    double r[T_N];
    for (int m = 0; m < T_N; ++m) r[m] = block_reduce(a[m], sh, Add());
    if (threadIdx.x == 0)
        for (int m = 0; m < T_N; ++m) part[(size_t)blockIdx.x * T_N + m] = r[m];
}

__global__ void k_sum_parts(const double *part, int nb, int np, int nv, double *out) {
    __shared__ double sh[DIAG_THREADS];
    for (int m = 0; m < nv; ++m) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nb; b += DIAG_THREADS) v += part[(size_t)b * np + m];
        const double r = block_reduce(v, sh, Add());
        if (threadIdx.x == 0) out[m] = r;
    }
}

// interior fluctuation of component c, packed (x fastest) for the transform
__global__ void k_pack_fluct(TurbIn in, Geo g, int c, double *dst) {
    const long ni = (long)g.nx * g.ny * g.nz;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni) return;
    const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
    dst[t] = fluct(in, g, c, i, j, k);
}

// shell binning of |u_hat|^2 / N^2 (spectrum [k][j][kx] complex): nint(|k|)
// with the half-spectrum weights of energy_single (1/2 at kx = 0 and NX/2,
// 1 elsewhere); per-block histograms accumulated over the components
__global__ void __launch_bounds__(DIAG_THREADS) k_spec_bin(const double *H, Geo g, int nbins, double inv_n2,
                                                           double *hist, int accumulate) {
    extern __shared__ double hs[];
    for (int b = threadIdx.x; b < nbins; b += DIAG_THREADS) hs[b] = 0.0;
    __syncthreads();
    const int nxh = g.nx / 2 + 1;
    const long nm = (long)nxh * g.ny * g.nz;
    // each block owns a contiguous range of modes and bins them in order
    const long per = (nm + gridDim.x - 1) / gridDim.x;
    const long m0 = (long)blockIdx.x * per, m1 = min(nm, m0 + per);
    if (threadIdx.x == 0) {
        for (long m = m0; m < m1; ++m) {
            const int ii = (int)(m % nxh), jj = (int)((m / nxh) % g.ny), kk = (int)(m / ((long)nxh * g.ny));
            const double kx = ii, ky = jj <= g.ny / 2 ? jj : jj - g.ny, kz = kk <= g.nz / 2 ? kk : kk - g.nz;
            const int idx = min(nbins - 1, (int)lround(sqrt(kx * kx + ky * ky + kz * kz)));
            const double re = H[2 * m], im = H[2 * m + 1];
            const double e = (re * re + im * im) * inv_n2;
            hs[idx] += (ii == 0 || ii == g.nx / 2) ? e / 2.0 : e / 2.0 * 2.0;
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += DIAG_THREADS)
        hist[(size_t)blockIdx.x * nbins + b] = (accumulate ? hist[(size_t)blockIdx.x * nbins + b] : 0.0) + hs[b];
}

__global__ void k_hist_final(const double *hist, int nb, int nbins, double *out) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int q = 0; q < nb; ++q) v += hist[(size_t)q * nbins + b];
        out[b] = v;
    }
}

}  // namespace

size_t turb_partials(int nx) { return (size_t)diag_blocks() * std::max<int>(T_N, nx + 1); }

cudaError_t device_turbulence(Dev &d, bool mixed, const double *const mean[3], double *part, double *out,
                              TurbValues *res, cudaStream_t s) {
    const Geo &g = d.g;
    TurbIn in{};
    in.st.cs = d.cs;
    in.st.mixed = mixed ? 1 : 0;
    if (mixed) {
        in.st.Uh = d.Uf; in.st.Ul = d.Ul; in.st.Vh = d.Vf; in.st.Vl = d.Vl; in.st.Wh = d.Wf; in.st.Wl = d.Wl;
        in.st.Cf = d.Cf;
    } else {
        in.st.U = d.U; in.st.V = d.V; in.st.W = d.W;
        in.st.C = d.C;
    }
    for (int c = 0; c < 3; ++c) in.mean[c] = mean ? mean[c] : nullptr;
    in.d3 = 1;
    const double dep = 0.5 * (1.0 - d.ph.beta) / d.ph.re / d.ph.wi * (d.ph.lp2 - 3.0);
    const int nb = diag_blocks();
    k_turb_pass<<<nb, DIAG_THREADS, 0, s>>>(in, g, dep, d.ph.lp2, part); count_launch();
    k_sum_parts<<<1, DIAG_THREADS, 0, s>>>(part, nb, T_N, T_N, out); count_launch();
    double h[T_N];
    F8_CUDA_RET(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
    F8_CUDA_RET(cudaStreamSynchronize(s));
    const double N = (double)g.nx * g.ny * g.nz, nu = 1.0 / d.ph.re;
    const double urms = h[T_U2] / N, vrms = h[T_V2] / N, wrms = h[T_W2] / N;
    const double ugrad = h[T_GU] / N, vgrad = h[T_GV] / N, wgrad = h[T_GW] / N;
    const double all_rms = (urms + vrms + wrms) / 3.0, all_grad = (ugrad + vgrad + wgrad) / 3.0;
    res->epsilon = nu / 2.0 * h[T_S2] / N;
    res->l_kolmogorov = std::pow(nu * nu * nu / res->epsilon, 0.25);
    res->t_kolmogorov = std::pow(nu / res->epsilon, 0.5);
    res->u_kolmogorov = std::pow(nu * res->epsilon, 0.25);
    res->lambda = std::sqrt(all_rms / all_grad);
    res->re_lambda = std::sqrt(all_rms) * res->lambda / nu;
    res->k_energy = (urms + vrms + wrms) / 2.0;
    res->k_staggered = h[T_KS] / (2.0 * N);
    res->ep_energy = h[T_EP] / N;
    return cudaGetLastError();
}

cudaError_t device_spectrum(Dev &d, bool mixed, const double *const mean[3], SpecWork &w, double *energy_dev,
                            cudaStream_t s) {
    const Geo &g = d.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxh = nx / 2 + 1;
    TurbIn in{};
    in.st.cs = d.cs;
    in.st.mixed = mixed ? 1 : 0;
    if (mixed) {
        in.st.Uh = d.Uf; in.st.Ul = d.Ul; in.st.Vh = d.Vf; in.st.Vl = d.Vl; in.st.Wh = d.Wf; in.st.Wl = d.Wl;
    } else {
        in.st.U = d.U; in.st.V = d.V; in.st.W = d.W;
    }
    for (int c = 0; c < 3; ++c) in.mean[c] = mean ? mean[c] : nullptr;
    const long ni = (long)nx * ny * nz;
    const int nbins = nx + 1;
    const double inv_n2 = 1.0 / ((double)ni * (double)ni);
    for (int c = 0; c < 3; ++c) {
        k_pack_fluct<<<(unsigned)((ni + 255) / 256), 256, 0, s>>>(in, g, c, w.pack); count_launch();
        {
            const int tpp = std::max(nx / 2, 1), ppc = std::max(1, 256 / tpp);
            const int npp = ny / 2, total = npp * nz;
            const size_t smem = (size_t)ppc * 2 * nx * sizeof(Cx<double>);
            k_fft_x_fwd<double, double><<<(total + ppc - 1) / ppc, ppc * tpp, smem, s>>>(w.pack, w.H, nx, ny, 1, ny, npp, nz,
                                                                                         w.twr[0], w.twi[0]); count_launch();
        }
        DivideSpec none{};
        {
            const int tx = std::max(1, std::min(32, 2048 / ny));
            const size_t smem = (size_t)2 * ny * tx * sizeof(Cx<double>);
            k_fft_lines<double><<<dim3((nxh + tx - 1) / tx, nz), 256, smem, s>>>(w.H, ny, nxh, nxh, nxh * ny, tx, w.twr[1],
                                                                                  w.twi[1], -1, 0, none); count_launch();
        }
        {
            const int tx = std::max(1, std::min(32, 2048 / nz));
            const size_t smem = (size_t)2 * nz * tx * sizeof(Cx<double>);
            k_fft_lines<double><<<dim3((nxh + tx - 1) / tx, ny), 256, smem, s>>>(w.H, nz, nxh * ny, nxh, nxh, tx, w.twr[2],
                                                                                  w.twi[2], -1, 0, none); count_launch();
        }
        k_spec_bin<<<diag_blocks(), DIAG_THREADS, (size_t)nbins * sizeof(double), s>>>(w.H, g, nbins, inv_n2, w.hist,
                                                                                    c > 0 ? 1 : 0); count_launch();
    }
    k_hist_final<<<(nbins + 255) / 256, 256, 0, s>>>(w.hist, diag_blocks(), nbins, energy_dev); count_launch();
    return cudaGetLastError();
}

cudaError_t spectrum_kernel_attrs() {
    const int big = 200 * 1024;
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_x_fwd<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_lines<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_spec_bin, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    return cudaSuccess;
}

}  // namespace f8

// ---------------------------------------------------------------------------
// Running statistics after each step (fenep_mpi.f90:2934-2941, 3054-3056):
// mode 1 sums U, V, W and records the centre-line probes U_step(k, n) =
// (U(NX/2, NY/2, k) + U(NX/2-1, NY/2, k))/2 (V over j, W over k alike);
// mode 2 sums the squared fluctuations about given mean fields.
namespace f8 {
namespace {

__global__ void k_stats_accum(DiagSliceIn st, Geo g, int mode, const double *mean, double *sums, double *probes,
                              int n, int max_steps) {
    const long ni = (long)g.nx * g.ny * g.nz;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni) return;
    const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
    const int h = hix(g, i, j, k);
    for (int c = 0; c < 3; ++c) {
        const double v = slice_vel(st, c, h);
        if (mode == 1) {
            sums[(size_t)c * ni + t] += v;
        } else {
            const double d = v - mean[(size_t)c * ni + t];
            sums[(size_t)c * ni + t] += d * d;
        }
    }
    if (mode == 1 && i == g.nx / 2 && j == g.ny / 2 && n < max_steps) {
        const int off[3] = {1, g.sx, g.sx * g.sy};
        for (int c = 0; c < 3; ++c)
            probes[((size_t)c * max_steps + n) * g.nz + (k - 1)] =
                (slice_vel(st, c, h) + slice_vel(st, c, h - off[c])) / 2.0;
    }
}

}  // namespace

cudaError_t device_stats_accum(Dev &d, bool mixed, int mode, const double *mean, double *sums, double *probes, int n,
                               int max_steps, cudaStream_t s) {
    DiagSliceIn st{};
    st.cs = d.cs;
    st.mixed = mixed ? 1 : 0;
    if (mixed) {
        st.Uh = d.Uf; st.Ul = d.Ul; st.Vh = d.Vf; st.Vl = d.Vl; st.Wh = d.Wf; st.Wl = d.Wl;
    } else {
        st.U = d.U; st.V = d.V; st.W = d.W;
    }
    const long ni = (long)d.ni;
    k_stats_accum<<<(unsigned)((ni + 255) / 256), 256, 0, s>>>(st, d.g, mode, mean, sums, probes, n, max_steps);
    count_launch();
    return cudaGetLastError();
}

}  // namespace f8
