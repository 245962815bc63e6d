// f8_diag.cu — on-device reductions of log_progress (fenep.f90:2266-2342) plus
// the divergence residual: kinetic energy on the cell centres, CFL from the
// maxima of U, V, W over the whole halo field, trC minimum / maximum / mean /
// standard deviation (the reference's two-pass form, mean first), max |div u|
// and a NaN flag.  Deterministic: a fixed grid of DIAG_BLOCKS blocks
// accumulates grid-stride partials per thread, a block tree reduces them, and
// one block reduces the block partials in a fixed order.  Both precisions: the
// FP64 state, or the double-float state and FP32 C of the mixed path.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include "f8_common.cuh"
#include "f8_kernels.h"

namespace f8 {
namespace {

constexpr int DIAG_BLOCKS = 592;   // 4 x 148-152 SMs
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
    for (long t = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; t < ni; t += (long)DIAG_BLOCKS * DIAG_THREADS) {
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
    for (long q = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; q < in.cs; q += (long)DIAG_BLOCKS * DIAG_THREADS) {
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
    for (long t = (long)blockIdx.x * DIAG_THREADS + threadIdx.x; t < ni; t += (long)DIAG_BLOCKS * DIAG_THREADS) {
        const int i = 1 + (int)(t % g.nx), j = 1 + (int)((t / g.nx) % g.ny), k = 1 + (int)(t / ((long)g.nx * g.ny));
        const double d = trace_at(in, hix(g, i, j, k)) - mean;
        s += d * d;
    }
    const double r = block_reduce(s, sh, Add());
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// final: one block reduces the block partials (stride np per block) in order
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_final(const double *part, int np, int nv, double *out) {
    __shared__ double sh[DIAG_THREADS];
    for (int m = 0; m < nv; ++m) {
        const bool mx = m == P_TMAX || m == P_DIV || m == P_UMAX || m == P_VMAX || m == P_WMAX || m == P_NAN;
        const bool mn = m == P_TMIN;
        double v = mn ? DBL_MAX : (mx ? -DBL_MAX : 0.0);
        for (int b = threadIdx.x; b < DIAG_BLOCKS; b += DIAG_THREADS) {
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
    k_diag_pass1<<<DIAG_BLOCKS, DIAG_THREADS, 0, s>>>(in, g, part); count_launch();
    k_diag_final<<<1, DIAG_THREADS, 0, s>>>(part, P_N, P_N, out); count_launch();
    k_diag_pass2<<<DIAG_BLOCKS, DIAG_THREADS, 0, s>>>(in, g, out, part); count_launch();
    k_diag_final<<<1, DIAG_THREADS, 0, s>>>(part, 1, 1, out + P_N); count_launch();
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

size_t diag_partials() { return (size_t)DIAG_BLOCKS * P_N; }

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
