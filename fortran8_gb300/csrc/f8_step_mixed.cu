// f8_step_mixed.cu — FP32-bulk step with a double-float state (F8_MIXED).
//
// Same discretisation as the FP64 step (fenep.f90 numerics; cited per kernel
// in f8_step_fp64.cu), with the precision split:
//   df64 (hi + lo FP32 pairs, 48-bit significand, FP32 pipes only): the state
//         U, V, W, P and the pressure correction Phi; the Poisson right-hand
//         side div(U^n + dU)/dt and its defect; the projection and the
//         pressure update.
//   FP64: marker velocities, marker forces and drag; the Peterlin factor when
//         L^2 - tr C < 1% of L^2.
//   FP32: C, f(C), the AB2/trapezoid history, stress / convection / viscous
//         stencils (on the hi parts), the pressure gradient, the eigen test
//         and Newton solve of the polymer update, and every spectral
//         transform and tridiagonal solve.
// The predictor is solved in increment form: (1 - dt beta/(2Re) L) dU =
// dt (R + f), with R = -grad P + (3A - A0)/2 + B + (T + T0)/2 + F.  This is
// algebraically the reference's (1 - dt beta/(2Re) L) U* = Q (fenep.f90:
// 1469-1479, 2229-2233) with U* = U^n + dU, but FP32 rounding touches only the
// O(dt) increment.  The Poisson equation is solved in FP32 and corrected once
// with a df64 residual (iterative refinement), so that the projected velocity
// is divergence-free to the df64 rounding level.
#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include "../../include/f8.h"
#include "f8_common.cuh"
#include "f8_df64.cuh"
#include "f8_fft.cuh"
#include "f8_fft_fused.cuh"
#include "f8_kernels.h"
#include "f8_tma.cuh"

namespace f8 {
namespace {


// Grid constants of the mixed kernels, computed once on the host in FP64 so
// that no kernel divides in FP64 (FP64 division is slow on this part).
struct MixConst {
    float gx1, gx4, gy1, gy4, gz1, gz4;   // -dt/dX, -dt/(4dX), ... (velocity gradient)
    float sx, sy, sz;                      // dt/(2dX) ... (upwind weights of Cstar)
    float ix, iy, iz;                      // 1/dX ...
    float ix2, iy2, iz2;                   // 1/dX^2 ...
    df di[3], di2[3];                      // 1/dX, 1/dX^2 ... as df64 constants
    df dtd[3];                             // dt/dX ...
    df idt;                                // 1/dt
    float pcf;                             // dt beta / (2 Re)
    float dtwi, lp2f, epsf;                // dt/Wi, L^2, Newton tolerance (FP32)
    float eps2f;                           // Newton tolerance squared
    float cpet;                            // (dt/Wi) (L^2 - 3), the scale of f'(tr C)
};

MixConst make_const(const Geo &g, const Phys &ph) {
    MixConst c{};
    c.gx1 = (float)(-ph.dt / g.dx); c.gx4 = (float)(-ph.dt / (4 * g.dx));
    c.gy1 = (float)(-ph.dt / g.dy); c.gy4 = (float)(-ph.dt / (4 * g.dy));
    c.gz1 = (float)(-ph.dt / g.dz); c.gz4 = (float)(-ph.dt / (4 * g.dz));
    c.sx = (float)(ph.dt / (2 * g.dx)); c.sy = (float)(ph.dt / (2 * g.dy)); c.sz = (float)(ph.dt / (2 * g.dz));
    c.ix = (float)(1.0 / g.dx); c.iy = (float)(1.0 / g.dy); c.iz = (float)(1.0 / g.dz);
    c.ix2 = (float)(1.0 / (g.dx * g.dx)); c.iy2 = (float)(1.0 / (g.dy * g.dy)); c.iz2 = (float)(1.0 / (g.dz * g.dz));
    const double dd[3] = {g.dx, g.dy, g.dz};
    for (int q = 0; q < 3; ++q) {
        c.di[q] = df_from_d(1.0 / dd[q]);
        c.di2[q] = df_from_d(1.0 / (dd[q] * dd[q]));
        c.dtd[q] = df_from_d(ph.dt / dd[q]);
    }
    c.idt = df_from_d(1.0 / ph.dt);
    c.pcf = (float)(ph.dt * ph.beta / ph.re / 2.0);
    c.dtwi = (float)(ph.dt / ph.wi);
    c.lp2f = (float)ph.lp2;
    c.epsf = (float)ph.newton_eps;
    c.eps2f = (float)(ph.newton_eps * ph.newton_eps);
    c.cpet = (float)(ph.dt / ph.wi * (ph.lp2 - 3.0));
    return c;
}

// Peterlin factor (fenep.f90:510-515) from FP32 components: FP32 normally, FP64
// when the denominator L^2 - tr C is within 1% of L^2 of the limit.
__device__ inline float peterlin_f(float x0, float x3, float x5, float lp2f, double lp2) {
    const float tr = x0 + x3 + x5;
    const float den = lp2f - tr;
    const bool near = !(den > 0.01f * lp2f);
    float f = (lp2f - 3.0f) / den;
    // the FP64 branch is entered only by warps that hold a cell near the
    // limit (a warp-uniform test, so that it is a branch, not a predicated
    // FP64 sequence that every warp issues)
    if (__any_sync(__activemask(), near) && near) {
        const double trd = (double)x0 + (double)x3 + (double)x5;
        f = (float)((lp2 - 3.0) / (lp2 - trd));
    }
    return f;
}

// The 2D model's Peterlin factor (L^2 - 2)/(L^2 - tr C), tr C = c11 + c22
// (fenep_2d.f90), FP64 near the limit as peterlin_f
__device__ inline float peterlin2_f(float x0, float x2, float lp2f, double lp2) {
    const float tr = x0 + x2;
    const float den = lp2f - tr;
    const bool near = !(den > 0.01f * lp2f);
    float f = (lp2f - 2.0f) / den;
    if (__any_sync(__activemask(), near) && near) {
        const double trd = (double)x0 + (double)x2;
        f = (float)((lp2 - 2.0) / (lp2 - trd));
    }
    return f;
}

// f of NC stored components: 6 (3D: xx xy xz yy yz zz) or 3 (2D: xx xy yy)
template <int NC>
__device__ inline float peterlin_nc(const float (&x)[NC], float lp2f, double lp2) {
    if constexpr (NC == 6) return peterlin_f(x[0], x[3], x[5], lp2f, lp2);
    else return peterlin2_f(x[0], x[2], lp2f, lp2);
}

// C halo (C_PBM / linear extrapolation at walls) and f on the halo cells
template <int NC>
__global__ void k_bc_c_pet_f(float *C, float *fpet, Geo g, int cs, double lp2) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, j, k;
    if (!halo_cell(g, t, i, j, k)) return;
    const int h = hix(g, i, j, k);
    const int ii = wrapx(g, i), kk = wrapz(g, k);
    // the source cells: a periodic image, or the two rows of the wall
    // extrapolation (weights 2 and -1)
    int s1, s2 = -1;
    if (j >= 1 && j <= g.ny) s1 = hix(g, ii, j, kk);
    else if (!g.walls) s1 = hix(g, ii, wrapy(g, j), kk);
    else if (j == 0) { s1 = hix(g, ii, 1, kk); s2 = hix(g, ii, 2, kk); }
    else { s1 = hix(g, ii, g.ny, kk); s2 = hix(g, ii, g.ny - 1, kk); }
    // every component's sources before the first store
    float x[NC];
#pragma unroll
    for (int m = 0; m < NC; ++m) {
        const float *A = C + (size_t)m * cs;
        x[m] = s2 < 0 ? A[s1] : 2.0f * A[s1] - A[s2];
    }
#pragma unroll
    for (int m = 0; m < NC; ++m) C[(size_t)m * cs + h] = x[m];
    fpet[h] = peterlin_nc<NC>(x, (float)lp2, lp2);
}

// After the polymer update of a wall channel: the x and z halo cells of every
// row (ghost rows included) as periodic copies, with their Peterlin factor;
// the updated ghost rows are kept (extrapolated at the end of the step).
template <int NC>
__global__ void k_bc_c_pet_xz_f(float *C, float *fpet, Geo g, int cs, double lp2) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, j, k;
    if (!halo_cell(g, t, i, j, k)) return;
    if ((j == 0 || j == g.sy - 1) && i >= 1 && i <= g.nx && k >= 1 && k <= g.nz) return;   // updated ghost cell
    const int h = hix(g, i, j, k), src = hix(g, wrapx(g, i), j, wrapz(g, k));
    float x[NC];
#pragma unroll
    for (int m = 0; m < NC; ++m) x[m] = C[(size_t)m * cs + src];
#pragma unroll
    for (int m = 0; m < NC; ++m) C[(size_t)m * cs + h] = x[m];
    fpet[h] = peterlin_nc<NC>(x, (float)lp2, lp2);
}

// The wall extrapolation of the C ghost rows (C_kabe, fenep_2d.f90:1131-1143)
// and their Peterlin factor, every x and z (the x/z halo copies of rows 1, 2,
// NY-1, NY are already in place).
template <int NC>
__global__ void k_extrap_ghost_f(float *C, float *fpet, Geo g, int cs, double lp2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * g.sx * g.sz) return;
    const int side = t / (g.sx * g.sz), r = t % (g.sx * g.sz);
    const int i = r % g.sx, k = r / g.sx;
    const int j = side ? g.ny + 1 : 0, j1 = side ? g.ny : 1, j2 = side ? g.ny - 1 : 2;
    const int h = hix(g, i, j, k), h1 = hix(g, i, j1, k), h2 = hix(g, i, j2, k);
    float x[NC];
#pragma unroll
    for (int m = 0; m < NC; ++m) {
        const float *A = C + (size_t)m * cs;
        x[m] = 2.0f * A[h1] - A[h2];
    }
#pragma unroll
    for (int m = 0; m < NC; ++m) C[(size_t)m * cs + h] = x[m];
    fpet[h] = peterlin_nc<NC>(x, (float)lp2, lp2);
}

// halo values (PBM / wall rules, fenep_2d.f90:1098-1129) of a df64 field;
// uw2 = 2 * upper wall speed (0 for the increments)
__device__ inline df halo_df(const Geo &g, const float *H, const float *L, int kind, int i, int j, int k, df uw2) {
    const int ii = wrapx(g, i), kk = wrapz(g, k);
    auto at = [&](int a, int b, int c) {
        const int q = hix(g, a, b, c);
        return df{H[q], L ? L[q] : 0.0f};
    };
    if (j >= 1 && j <= g.ny) {
        if (g.walls && kind == BC_V && j == g.ny) return df{0.0f, 0.0f};
        return at(ii, j, kk);
    }
    if (!g.walls) return at(ii, wrapy(g, j), kk);
    const bool lo = j == 0;
    switch (kind) {
    case BC_U: return lo ? df_neg(at(ii, 1, kk)) : df_sub(uw2, at(ii, g.ny, kk));
    case BC_W: return df_neg(at(ii, lo ? 1 : g.ny, kk));
    case BC_V: return df{0.0f, 0.0f};
    default:   return at(ii, lo ? 1 : g.ny, kk);
    }
}

// Boundary values of up to four df64 (lo != null) or FP32 (lo == null)
// fields, and V = 0 on the upper wall face when a field of kind BC_V is given.
struct BcSet {
    float *hi[4], *lo[4];
    int kind[4];
    int n;
    df uw2;
};

__global__ void k_bc_set(BcSet b, Geo g) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, j, k;
    if (halo_cell(g, t, i, j, k)) {
        const int h = hix(g, i, j, k);
        // every field's source value before the first store
        df v[4];
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (f < b.n) v[f] = halo_df(g, b.hi[f], b.lo[f], b.kind[f], i, j, k, b.uw2);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (f < b.n) {
                b.hi[f][h] = v[f].hi;
                if (b.lo[f]) b.lo[f][h] = v[f].lo;
            }
        return;
    }
    if (g.walls) {  // V on the upper wall face
        t -= halo_count(g);
        if (t >= 0 && t < (long)g.nx * g.nz) {
            i = 1 + (int)(t % g.nx); k = 1 + (int)(t / g.nx);
            const int h = hix(g, i, g.ny, k);
#pragma unroll
            for (int f = 0; f < 4; ++f)
                if (f < b.n && b.kind[f] == BC_V) {
                    b.hi[f][h] = 0.0f;
                    if (b.lo[f]) b.lo[f][h] = 0.0f;
                }
        }
    }
}

// FP64 <-> df64 pairs (load / store)
__global__ void k_split_df(const double *src, float *hi, float *lo, int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const df v = df_from_d(src[q]);
    hi[q] = v.hi;
    lo[q] = v.lo;
}

__global__ void k_join_df(const float *hi, const float *lo, double *dst, int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    dst[q] = (double)hi[q] + (double)lo[q];
}

template <int NC>
__global__ void k_pet_all_f(const float *C, float *fpet, int cs, double lp2) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cs) return;
    if constexpr (NC == 6) fpet[h] = peterlin_f(C[h], C[3 * (size_t)cs + h], C[5 * (size_t)cs + h], (float)lp2, lp2);
    else fpet[h] = peterlin2_f(C[h], C[2 * (size_t)cs + h], (float)lp2, lp2);
}

// ---------------------------------------------------------------------------
// Polymer (3D).  Eigen test: the smallest eigenvalue of each symmetric 3x3
// candidate face in the shifted (traceless) trigonometric form, which is the
// same root as the reference's Vieta formula (fenep.f90:425-444) but free of
// the cancellation in p = a1 - a2^2/3 that FP32 would suffer near C = I.
// Equal roots (discriminant q^2 - p^3 >= 0, i.e. |r| >= 1 below) give the
// reference's -100 sentinel.  The two faces of candidate l (fenep.f90:179-184)
// are c0 - v and c0 + v with v = dp/2, dm/2, (dm + dp)/4 for l = 1, 2, 3
// (dm = c0 - c_{-1}, dp = c_{+1} - c0), so they share the mean and deviatoric
// part of c0 and are evaluated as one packed FP32x2 pair.
//
// With B the deviatoric part, p = |B|^2 / 6, q = det(B) / 2 and
// r = q / p^(3/2), the smallest eigenvalue is m + 2 sqrt(p) t(r),
// t(r) = cos(acos(r)/3 + 2 pi/3), the smallest root of 4t^3 - 3t = r.  t has a
// square-root branch point at r = 1 (two equal smallest roots) and is
// analytic at r = -1, so as a function of u = sqrt(1 - r) on [0, sqrt 2] it is
// analytic: t(u) is interpolated at the 8 Chebyshev points of [0, sqrt 2]
// (fitted offline in double precision, |error| <= 2.7e-8), and 2t(u) is
// evaluated from the FP32 coefficients of twice that polynomial in FP32 Horner
// form (|error| <= 2.2e-7).  This replaces the arccos and cosine of the
// trigonometric formula.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fms2(float2 a, float2 b, float2 c) {   // a * b - c
    return __ffma2_rn(a, b, make_float2(-c.x, -c.y));
}

// 2 t(u), u = sqrt(1 - r)
__device__ __forceinline__ float2 two_t2(float2 u) {
    float2 p = f2(-1.993398037e-04f);
    p = fma2(p, u, f2(1.522336388e-03f));
    p = fma2(p, u, f2(-5.673570558e-03f));
    p = fma2(p, u, f2(1.511769835e-02f));
    p = fma2(p, u, f2(-3.736452013e-02f));
    p = fma2(p, u, f2(1.110385135e-01f));
    p = fma2(p, u, f2(-8.164918423e-01f));
    return fma2(p, u, f2(-1.0f));
}

// smallest eigenvalues of the pair of symmetric matrices m + B (B traceless,
// components b00 b11 b22 b01 b02 b12 as FP32x2 pairs)
__device__ __forceinline__ float2 lam_min2(float2 m, float2 b00, float2 b11, float2 b22, float2 b01, float2 b02,
                                           float2 b12) {
    float2 sd = mul2(b00, b00);
    sd = fma2(b11, b11, sd);
    sd = fma2(b22, b22, sd);
    float2 so = mul2(b01, b01);
    so = fma2(b02, b02, so);
    so = fma2(b12, b12, so);
    const float2 p2 = mul2(fma2(so, f2(2.0f), sd), f2(1.0f / 6.0f));
    // q = det(B) / 2 by cofactors of the first row
    const float2 a00 = fms2(b11, b22, mul2(b12, b12));
    const float2 a01 = fms2(b01, b22, mul2(b12, b02));
    const float2 a02 = fms2(b01, b12, mul2(b11, b02));
    const float2 q = mul2(fma2(b02, a02, fms2(b00, a00, mul2(b01, a01))), f2(0.5f));
    const float2 rs = make_float2(rsqrtf(p2.x), rsqrtf(p2.y));
    const float2 r = mul2(mul2(q, rs), mul2(rs, rs));
    // w = 1 - r; 0 < w < 2 is |r| < 1.  p = 0 (an isotropic face) gives
    // r = NaN, which fails the test: equal roots, the sentinel.
    const float2 w = add2(f2(1.0f), make_float2(-r.x, -r.y));
    const bool okx = w.x > 0.0f && w.x < 2.0f, oky = w.y > 0.0f && w.y < 2.0f;
    const float2 u = make_float2(okx ? w.x * rsqrtf(w.x) : 0.0f, oky ? w.y * rsqrtf(w.y) : 0.0f);
    const float2 lam = fma2(mul2(p2, rs), two_t2(u), m);
    return make_float2(okx ? lam.x : -100.0f, oky ? lam.y : -100.0f);
}

// candidate faces (fenep.f90:179-184) as weights (w0, w1, w2) of
// (C_{m-1}, C_m, C_{m+1}); candidate c = 1, 2, 3, and 4 for the cell value
// (the Cstar stencil coefficients below).  The plus face of c is
// (p0, 1 - p0 - p2, p2) with (p0, p2) = (0, -1/2), (1/2, 0), (1/4, -1/4),
// (0, 0); the minus face is its mirror (-p0, 1 + p0 + p2, -p2).  The weights
// are exact in FP32 and are formed with selects: the candidate differs from
// thread to thread, and a constant-memory table read with per-thread indices
// is serialised.
struct FaceW {
    float p0, p1, p2, n0, n1, n2;
};
__device__ __forceinline__ FaceW face_w(int c) {
    const float p0 = c == 2 ? 0.5f : (c == 3 ? 0.25f : 0.0f);
    const float p2 = c == 1 ? -0.5f : (c == 3 ? -0.25f : 0.0f);
    return FaceW{p0, 1.0f - p0 - p2, p2, -p0, 1.0f + p0 + p2, -p2};
}

// candidate choice of one direction (maxloc over the three candidates' least
// eigenvalues and 0, first maximum, NaN ignored), returns the code 0..3
__device__ __forceinline__ int select_dir_f(const float (&c0)[6], float m0, float e00, float e11, float e22,
                                            const float (&dm)[6], const float (&dp)[6]) {
    float ml[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
        float v[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) v[m] = l == 0 ? 0.5f * dp[m] : (l == 1 ? 0.5f * dm[m] : 0.25f * (dm[m] + dp[m]));
        const float mv = (v[0] + v[3] + v[5]) * (1.0f / 3.0f);
        const float2 pm = make_float2(-1.0f, 1.0f);
        const float2 lam = lam_min2(fma2(f2(mv), pm, f2(m0)), fma2(f2(v[0] - mv), pm, f2(e00)),
                                    fma2(f2(v[3] - mv), pm, f2(e11)), fma2(f2(v[5] - mv), pm, f2(e22)),
                                    fma2(f2(v[1]), pm, f2(c0[1])), fma2(f2(v[2]), pm, f2(c0[2])),
                                    fma2(f2(v[4]), pm, f2(c0[4])));
        ml[l] = fminf(lam.x, lam.y);   // NaN-ignoring minimum
    }
    float best = 0.0f;
    int idx = 4;
    bool found = false;
#pragma unroll
    for (int l = 0; l < 3; ++l) {
        if (isnan(ml[l])) continue;
        if (!found || ml[l] > best) { best = ml[l]; idx = l + 1; found = true; }
    }
    if (!found || 0.0f > best) idx = 4;
    return idx - 1;
}

// selection codes of the ghost rows of a wall channel (the rows beyond them
// hold zero C): the reference's wall mode updates C there too
// (fenep_2d.f90:138-226, 1131-1143)
__global__ void k_codes_ghost3_f(const float *__restrict__ C, uint8_t *__restrict__ codes_g, Geo g, int cs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int side = blockIdx.y, k = blockIdx.z + 1;
    if (i > g.nx) return;
    const int j = side ? g.ny + 1 : 0;
    const int h = hix(g, i, j, k);
    float c0[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) c0[m] = C[(size_t)m * cs + h];
    const float m0 = (c0[0] + c0[3] + c0[5]) * (1.0f / 3.0f);
    const float e00 = c0[0] - m0, e11 = c0[3] - m0, e22 = c0[5] - m0;
    int code = 0;
    for (int d = 0; d < 3; ++d) {
        float dm[6], dp[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const float *Cm = C + (size_t)m * cs;
            float cmv, cpv;
            if (d == 1) {
                cmv = j - 1 < 0 ? 0.0f : Cm[hix(g, i, j - 1, k)];
                cpv = j + 1 > g.ny + 1 ? 0.0f : Cm[hix(g, i, j + 1, k)];
            } else {
                const int od = d == 0 ? 1 : g.sx * g.sy;
                cmv = Cm[h - od];
                cpv = Cm[h + od];
            }
            dm[m] = c0[m] - cmv;
            dp[m] = cpv - c0[m];
        }
        code |= select_dir_f(c0, m0, e00, e11, e22, dm, dp) << (2 * d);
    }
    codes_g[gcix(g, i, j, k)] = (uint8_t)code;
}

__global__ void __launch_bounds__(256) k_codes3_f(const float *__restrict__ C, uint8_t *__restrict__ codes, Geo g, int cs,
                                                  int *__restrict__ fixcnt) {
    if ((blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y) == 0) *fixcnt = 0;   // queue of k_update3_f
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const int h = hix(g, i, j, k);
    float c0[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) c0[m] = C[(size_t)m * cs + h];
    const float m0 = (c0[0] + c0[3] + c0[5]) * (1.0f / 3.0f);
    const float e00 = c0[0] - m0, e11 = c0[3] - m0, e22 = c0[5] - m0;
    int code = 0;
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        const int od = d == 0 ? 1 : (d == 1 ? g.sx : g.sx * g.sy);
        float dm[6], dp[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            dm[m] = c0[m] - C[(size_t)m * cs + h - od];
            dp[m] = C[(size_t)m * cs + h + od] - c0[m];
        }
        // lane x of each pair: c0 - v (the face on the minus side), lane y: c0 + v
        code |= select_dir_f(c0, m0, e00, e11, e22, dm, dp) << (2 * d);
    }
    codes[qix(g, i, j, k)] = (uint8_t)code;
}

// Cstar + implicit Newton solve of A C + C A^T = Cx + dt/Wi I with
// A = A0 + (1 + f(C) dt/Wi)/2 I (fenep.f90:518-605) in FP32.  The Jacobian is
// J = B + c x e^T with B = a I + M(A0), a = 1 + f dt/Wi, c = (dt/Wi) f'(tr C),
// e = (1,0,0,1,0,1) and M the linear Lyapunov part (rows of Lyapunov_func,
// fenep.f90:598-603).  |M|/a = O(dt |grad u|) is small, so the fast solve
// replaces B^{-1} by its three-term Neumann series (1/a)(I - M/a + (M/a)^2)
// and the rank-one term by Sherman-Morrison with B^{-1} x ~ x/a.  This is a
// Newton iteration with an approximate Jacobian: it converges to the same root
// as the reference (stopping rule: the relative step test, fenep.f90:575) at
// the rate ~(|M|/a)^3 per iteration.  Cells that have not converged after
// NEWTON_FAST_MAX iterations are queued and re-solved from the start by the
// exact elimination in k_newton_fix_f.
constexpr int NEWTON_FAST_MAX = 12;

struct Lyap9 { float a00, a01, a02, a10, a11, a12, a20, a21, a22; };

__device__ inline void lyap_M(const Lyap9 &A, const float (&v)[6], float (&o)[6]) {
    o[0] = 2.0f * (A.a00 * v[0] + A.a01 * v[1] + A.a02 * v[2]);
    o[1] = A.a10 * v[0] + (A.a11 + A.a00) * v[1] + A.a12 * v[2] + A.a01 * v[3] + A.a02 * v[4];
    o[2] = A.a20 * v[0] + A.a21 * v[1] + (A.a22 + A.a00) * v[2] + A.a01 * v[4] + A.a02 * v[5];
    o[3] = 2.0f * (A.a10 * v[1] + A.a11 * v[3] + A.a12 * v[4]);
    o[4] = A.a10 * v[2] + A.a20 * v[1] + A.a21 * v[3] + (A.a22 + A.a11) * v[4] + A.a12 * v[5];
    o[5] = 2.0f * (A.a20 * v[2] + A.a21 * v[4] + A.a22 * v[5]);
}

// relative step test of fenep.f90:575; false on NaN so that the loop ends
__device__ inline bool step_small(const float (&x)[6], float sr, float epsf) {
    float sx = 0.0f;
#pragma unroll
    for (int m = 0; m < 6; ++m) sx += x[m] * x[m];
    return !(sqrtf(sr / sx) >= epsf);
}

// The relative step test of fenep.f90:575, |dx| / |x| < eps, without the
// square root: leaves when |dx|^2 <= eps^2 |x|^2 or on NaN
__device__ inline bool step_small_sq(const float (&x)[6], float sr, float eps2) {
    float sx = 0.0f;
#pragma unroll
    for (int m = 0; m < 6; ++m) sx = fmaf(x[m], x[m], sx);
    return !(sr > eps2 * sx);
}

// returns the iterations taken; > maxit when not converged.  The reciprocals
// are hardware approximations (2 ulp): the iteration corrects them, and the
// converged root satisfies the residual built with them.
__device__ inline int newton_fast_f(float (&x)[6], const float (&b)[6], const Lyap9 &A, const MixConst &mc,
                                    double lp2, int maxit) {
    const float dtwi = mc.dtwi, lp2f = mc.lp2f;
    int itr;
#pragma unroll 1
    for (itr = 1; itr <= maxit; ++itr) {
        const float tr = x[0] + x[3] + x[5];
        const float den = lp2f - tr;
        float f = __fdividef(lp2f - 3.0f, den);
        if (__any_sync(__activemask(), !(den > 0.01f * lp2f)) && !(den > 0.01f * lp2f))
            f = peterlin_f(x[0], x[3], x[5], lp2f, lp2);
        const float a = fmaf(f, dtwi, 1.0f);
        const float ia = __fdividef(1.0f, a);
        const float cc = __fdividef(mc.cpet, den * den);
        float r[6], y[6], t[6];
        lyap_M(A, x, r);
#pragma unroll
        for (int m = 0; m < 6; ++m) { r[m] = (r[m] + a * x[m] - b[m]) * ia; y[m] = r[m]; }
#pragma unroll
        for (int q = 0; q < 2; ++q) {        // y = (1/a)(I - M/a + (M/a)^2) residual
            lyap_M(A, y, t);
#pragma unroll
            for (int m = 0; m < 6; ++m) y[m] = fmaf(-ia, t[m], r[m]);
        }
        const float g = __fdividef(cc * (y[0] + y[3] + y[5]), fmaf(cc * tr, ia, 1.0f)) * ia;
        float sr = 0.0f;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const float d = fmaf(-g, x[m], y[m]);
            x[m] -= d;
            sr = fmaf(d, d, sr);
        }
        if (step_small_sq(x, sr, mc.eps2f)) break;
    }
    return itr;
}

// The exact Newton step: J assembled analytically and eliminated without
// pivoting (J is dominated by its diagonal a >= 1), fully unrolled.
__device__ inline int newton_exact_f(float (&x)[6], const float (&b)[6], const Lyap9 &A, float dtwi, float lp2f,
                                     double lp2, float epsf, int itrmax) {
    int itr;
#pragma unroll 1
    for (itr = 1; itr <= itrmax; ++itr) {
        const float f = peterlin_f(x[0], x[3], x[5], lp2f, lp2);
        const float a = 1.0f + f * dtwi;
        const float den = lp2f - (x[0] + x[3] + x[5]);
        const float cc = dtwi * (lp2f - 3.0f) / (den * den);
        float J[6][7];
        float r[6];
        lyap_M(A, x, r);
        const float Mx[6][6] = {
            {2 * A.a00, 2 * A.a01, 2 * A.a02, 0, 0, 0},
            {A.a10, A.a11 + A.a00, A.a12, A.a01, A.a02, 0},
            {A.a20, A.a21, A.a22 + A.a00, 0, A.a01, A.a02},
            {0, 2 * A.a10, 0, 2 * A.a11, 2 * A.a12, 0},
            {0, A.a20, A.a10, A.a21, A.a22 + A.a11, A.a12},
            {0, 0, 2 * A.a20, 0, 2 * A.a21, 2 * A.a22}};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            J[q][6] = r[q] + a * x[q] - b[q];
            const float cr = cc * x[q];
#pragma unroll
            for (int w = 0; w < 6; ++w)
                J[q][w] = Mx[q][w] + ((w == 0 || w == 3 || w == 5) ? cr : 0.0f) + (w == q ? a : 0.0f);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float inv = 1.0f / J[k][k];
#pragma unroll
            for (int q = k + 1; q < 7; ++q) J[k][q] *= inv;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                if (q == k) continue;
                const float fr = J[q][k];
#pragma unroll
                for (int w = k + 1; w < 7; ++w) J[q][w] -= fr * J[k][w];
            }
        }
        float sr = 0.0f;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            x[m] -= J[m][6];
            sr += J[m][6] * J[m][6];
        }
        if (step_small(x, sr, epsf)) break;
    }
    return itr;
}

// A = transpose of the velocity gradient (fenep.f90:541-550) at cell h
__device__ inline Lyap9 vel_grad_f(const float *__restrict__ U, const float *__restrict__ V,
                                   const float *__restrict__ W, int h, int ox, int oy, int oz, const MixConst &mc) {
    Lyap9 A;
    A.a00 = mc.gx1 * (U[h] - U[h - ox]);
    A.a10 = mc.gx4 * (-V[h - ox - oy] + V[h + ox - oy] - V[h - ox] + V[h + ox]);
    A.a20 = mc.gx4 * (-W[h - ox - oz] + W[h + ox - oz] - W[h - ox] + W[h + ox]);
    A.a01 = mc.gy4 * (-U[h - ox - oy] - U[h - oy] + U[h - ox + oy] + U[h + oy]);
    A.a11 = mc.gy1 * (V[h] - V[h - oy]);
    A.a21 = mc.gy4 * (-W[h - oy - oz] + W[h + oy - oz] - W[h - oy] + W[h + oy]);
    A.a02 = mc.gz4 * (-U[h - ox - oz] - U[h - oz] + U[h - ox + oz] + U[h + oz]);
    A.a12 = mc.gz4 * (-V[h - oy - oz] - V[h - oz] + V[h - oy + oz] + V[h + oz]);
    A.a22 = mc.gz1 * (W[h] - W[h - oz]);
    return A;
}

// Upwind Cstar coefficients of one direction on the points p-2 .. p+2
// (fenep.f90:155-196): the minus face takes s_pm * (candidate is of this cell)
// + s_nm * (candidate cm of the minus neighbour), the plus face s_np * (is) +
// s_pp * (candidate cp of the plus neighbour).  A wall ghost neighbour
// contributes its cell value (gm / gp).
__device__ inline void dir_coef(float s_pm, float s_pp, float s_nm, float s_np, int is, int cm, int cp, bool gm,
                                bool gp, float &km2, float &km1, float &k0, float &kp1, float &kp2) {
    const FaceW ws = face_w(is), wm = face_w(cm), wp = face_w(cp);
    km2 = gm ? 0.0f : s_nm * wm.n0;
    km1 = s_pm * ws.p0 + s_np * ws.n0 + (gm ? s_nm : s_nm * wm.n1);
    k0 += s_pm * ws.p1 + s_np * ws.n1 + (gm ? 0.0f : s_nm * wm.n2) + (gp ? 0.0f : s_pp * wp.p0);
    kp1 = s_pm * ws.p2 + s_np * ws.n2 + (gp ? s_pp : s_pp * wp.p1);
    kp2 = gp ? 0.0f : s_pp * wp.p2;
}

__global__ void __launch_bounds__(128) k_update3_f(const float *__restrict__ C, float *__restrict__ Cn,
                                                   float *__restrict__ fpet, const uint8_t *__restrict__ codes,
                                                   const float *__restrict__ U, const float *__restrict__ V,
                                                   const float *__restrict__ W, Geo g, Phys ph, MixConst mc, int cs,
                                                   int *__restrict__ fixlist, int *__restrict__ fixcnt,
                                                   StepCounters *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j <= g.ny;
    unsigned long long my_itr = 0, my_unconv = 0;
    if (active) {
        const int h = hix(g, i, j, k);
        const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
        const int cself = codes[qix(g, i, j, k)];
        const int im = wrapx(g, i - 1), ip = wrapx(g, i + 1), km = wrapz(g, k - 1), kp = wrapz(g, k + 1);
        int jm = j - 1, jp = j + 1;
        bool gym = false, gyp = false;
        if (!g.walls) { jm = wrapy(g, jm); jp = wrapy(g, jp); }
        else { gym = jm == 0; gyp = jp == g.ny + 1; }
        // stencil points p-2 and p+2 through the periodic neighbours (their
        // p+1 / p-1 are halo copies of this cell); at a wall ghost the point
        // is unused (coefficient 0) and is aliased to p -/+ 1
        const int hxm2 = hix(g, im, j, k) - ox, hxp2 = hix(g, ip, j, k) + ox;
        const int hym2 = gym ? h - oy : hix(g, i, jm, k) - oy, hyp2 = gyp ? h + oy : hix(g, i, jp, k) + oy;
        const int hzm2 = hix(g, i, j, km) - oz, hzp2 = hix(g, i, j, kp) + oz;
        float kx[5], ky[5], kz[5];
        {
            const float u1 = U[h - ox], u2 = U[h];
            const float v1 = V[h - oy], v2 = V[h];
            const float w1 = W[h - oz], w2 = W[h];
            const int cxm = codes[qix(g, im, j, k)] & 3, cxp = codes[qix(g, ip, j, k)] & 3;
            const int czm = (codes[qix(g, i, j, km)] >> 4) & 3, czp = (codes[qix(g, i, j, kp)] >> 4) & 3;
            const int cym = gym ? 3 : (codes[qix(g, i, jm, k)] >> 2) & 3;
            const int cyp = gyp ? 3 : (codes[qix(g, i, jp, k)] >> 2) & 3;
            float k0 = 0.0f;
            // s3 s1 s4 s2 of fenep.f90:166-177 per direction
            dir_coef(1.0f / 6 + (u1 - fabsf(u1)) * mc.sx, (-u2 + fabsf(u2)) * mc.sx, (u1 + fabsf(u1)) * mc.sx,
                     1.0f / 6 + (-u2 - fabsf(u2)) * mc.sx, (cself & 3) + 1, cxm + 1, cxp + 1, false, false,
                     kx[0], kx[1], k0, kx[3], kx[4]);
            dir_coef(1.0f / 6 + (v1 - fabsf(v1)) * mc.sy, (-v2 + fabsf(v2)) * mc.sy, (v1 + fabsf(v1)) * mc.sy,
                     1.0f / 6 + (-v2 - fabsf(v2)) * mc.sy, ((cself >> 2) & 3) + 1, cym + 1, cyp + 1, gym, gyp,
                     ky[0], ky[1], k0, ky[3], ky[4]);
            dir_coef(1.0f / 6 + (w1 - fabsf(w1)) * mc.sz, (-w2 + fabsf(w2)) * mc.sz, (w1 + fabsf(w1)) * mc.sz,
                     1.0f / 6 + (-w2 - fabsf(w2)) * mc.sz, ((cself >> 4) & 3) + 1, czm + 1, czp + 1, false, false,
                     kz[0], kz[1], k0, kz[3], kz[4]);
            kx[2] = k0;
        }
        const float dtwi = mc.dtwi;
        float b[6], x[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const float *Cm = C + (size_t)m * cs;
            const float c0 = Cm[h];
            float acc = kx[2] * c0;
            acc = fmaf(kx[0], Cm[hxm2], acc); acc = fmaf(kx[1], Cm[h - ox], acc);
            acc = fmaf(kx[3], Cm[h + ox], acc); acc = fmaf(kx[4], Cm[hxp2], acc);
            acc = fmaf(ky[0], Cm[hym2], acc); acc = fmaf(ky[1], Cm[h - oy], acc);
            acc = fmaf(ky[3], Cm[h + oy], acc); acc = fmaf(ky[4], Cm[hyp2], acc);
            acc = fmaf(kz[0], Cm[hzm2], acc); acc = fmaf(kz[1], Cm[h - oz], acc);
            acc = fmaf(kz[3], Cm[h + oz], acc); acc = fmaf(kz[4], Cm[hzp2], acc);
            b[m] = acc + ((m == 0 || m == 3 || m == 5) ? dtwi : 0.0f);
            x[m] = c0;
        }
        const Lyap9 A = vel_grad_f(U, V, W, h, ox, oy, oz, mc);
        const int fast_max = min(NEWTON_FAST_MAX, ph.newton_itrmax);
        const int itr = newton_fast_f(x, b, A, mc, ph.lp2, fast_max);
        if (itr <= fast_max || fast_max == ph.newton_itrmax) {
            my_itr = (unsigned long long)itr;
            my_unconv = itr > ph.newton_itrmax ? 1ull : 0ull;
#pragma unroll
            for (int m = 0; m < 6; ++m) Cn[(size_t)m * cs + h] = x[m];
            fpet[h] = peterlin_f(x[0], x[3], x[5], mc.lp2f, ph.lp2);
        } else {
            // keep Cstar for the exact solve
            my_itr = (unsigned long long)fast_max;
#pragma unroll
            for (int m = 0; m < 6; ++m) Cn[(size_t)m * cs + h] = b[m];
            fixlist[atomicAdd(fixcnt, 1)] = h;
        }
    }
    unsigned long long a = my_itr, b2 = my_unconv;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b2 += __shfl_down_sync(0xffffffffu, b2, o);
    }
    if (((threadIdx.x + blockDim.x * threadIdx.y) & 31) == 0) {
        if (a) atomicAdd(&cnt->newton_iters, a);
        if (b2) atomicAdd(&cnt->newton_unconverged, b2);
    }
}

// Exact Newton re-solve of the cells queued by k_update3_f (Cstar in Cn)
__global__ void __launch_bounds__(128) k_newton_fix_f(const float *__restrict__ C, float *__restrict__ Cn,
                                                      float *__restrict__ fpet, const float *__restrict__ U,
                                                      const float *__restrict__ V, const float *__restrict__ W,
                                                      Geo g, Phys ph, MixConst mc, int cs,
                                                      const int *__restrict__ fixlist,
                                                      const int *__restrict__ fixcnt, StepCounters *cnt) {
    const int n = *fixcnt;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int h = fixlist[t];
        float b[6], x[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) { b[m] = Cn[(size_t)m * cs + h]; x[m] = C[(size_t)m * cs + h]; }
        const Lyap9 A = vel_grad_f(U, V, W, h, 1, g.sx, g.sx * g.sy, mc);
        const int itr = newton_exact_f(x, b, A, mc.dtwi, mc.lp2f, ph.lp2, mc.epsf, ph.newton_itrmax);
        atomicAdd(&cnt->newton_iters, (unsigned long long)itr);
        if (itr > ph.newton_itrmax) atomicAdd(&cnt->newton_unconverged, 1ull);
#pragma unroll
        for (int m = 0; m < 6; ++m) Cn[(size_t)m * cs + h] = x[m];
        fpet[h] = peterlin_f(x[0], x[3], x[5], mc.lp2f, ph.lp2);
    }
}

// Polymer update of the ghost rows of a wall channel (the reference's wall
// mode, fenep_2d.f90:1912-1929): Cstar with the rows beyond the ghost rows
// holding zero C and velocity, then the exact FP32 Newton of k_newton_fix_f.
__global__ void __launch_bounds__(128) k_update_ghost3_f(const float *__restrict__ C, float *__restrict__ Cn,
                                                         float *__restrict__ fpet, const uint8_t *__restrict__ codes,
                                                         const uint8_t *__restrict__ codes_g,
                                                         const float *__restrict__ U, const float *__restrict__ V,
                                                         const float *__restrict__ W, Geo g, Phys ph, MixConst mc,
                                                         int cs, StepCounters *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int side = blockIdx.y, k = blockIdx.z + 1;
    unsigned long long my_itr = 0, my_unconv = 0;
    if (i <= g.nx) {
    const int j = side ? g.ny + 1 : 0;
    const int h = hix(g, i, j, k);
    const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
    auto vrow = [&](const float *A, int ii, int jj, int kk) {
        return (jj < 0 || jj > g.ny + 1) ? 0.0f : A[hix(g, ii, jj, kk)];
    };
    const int im = wrapx(g, i - 1), ip = wrapx(g, i + 1), km = wrapz(g, k - 1), kp = wrapz(g, k + 1);
    const int cself = codes_g[gcix(g, i, j, k)];
    const int cxm = codes_g[gcix(g, im, j, k)] & 3, cxp = codes_g[gcix(g, ip, j, k)] & 3;
    const int czm = (codes_g[gcix(g, i, j, km)] >> 4) & 3, czp = (codes_g[gcix(g, i, j, kp)] >> 4) & 3;
    // the interior neighbour's y code (its face towards this row); the cell
    // beyond is outside (coefficient zero)
    const int cyin = (codes[qix(g, i, side ? g.ny : 1, k)] >> 2) & 3;
    const bool lower = side == 0;
    float kx[5], ky[5], kz[5];
    {
        const float u1 = U[h - ox], u2 = U[h];
        const float v1 = vrow(V, i, j - 1, k), v2 = V[h];
        const float w1 = W[h - oz], w2 = W[h];
        float k0 = 0.0f;
        dir_coef(1.0f / 6 + (u1 - fabsf(u1)) * mc.sx, (-u2 + fabsf(u2)) * mc.sx, (u1 + fabsf(u1)) * mc.sx,
                 1.0f / 6 + (-u2 - fabsf(u2)) * mc.sx, (cself & 3) + 1, cxm + 1, cxp + 1, false, false,
                 kx[0], kx[1], k0, kx[3], kx[4]);
        dir_coef(1.0f / 6 + (v1 - fabsf(v1)) * mc.sy, (-v2 + fabsf(v2)) * mc.sy, (v1 + fabsf(v1)) * mc.sy,
                 1.0f / 6 + (-v2 - fabsf(v2)) * mc.sy, ((cself >> 2) & 3) + 1, lower ? 4 : cyin + 1,
                 lower ? cyin + 1 : 4, lower, !lower, ky[0], ky[1], k0, ky[3], ky[4]);
        dir_coef(1.0f / 6 + (w1 - fabsf(w1)) * mc.sz, (-w2 + fabsf(w2)) * mc.sz, (w1 + fabsf(w1)) * mc.sz,
                 1.0f / 6 + (-w2 - fabsf(w2)) * mc.sz, ((cself >> 4) & 3) + 1, czm + 1, czp + 1, false, false,
                 kz[0], kz[1], k0, kz[3], kz[4]);
        kx[2] = k0;
    }
    const int hxm2 = hix(g, im, j, k) - ox, hxp2 = hix(g, ip, j, k) + ox;
    const int hzm2 = hix(g, i, j, km) - oz, hzp2 = hix(g, i, j, kp) + oz;
    float b[6], x[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        const float *Cm = C + (size_t)m * cs;
        const float c0 = Cm[h];
        float acc = kx[2] * c0;
        acc = fmaf(kx[0], Cm[hxm2], acc); acc = fmaf(kx[1], Cm[h - ox], acc);
        acc = fmaf(kx[3], Cm[h + ox], acc); acc = fmaf(kx[4], Cm[hxp2], acc);
        acc = fmaf(ky[0], vrow(Cm, i, j - 2, k), acc); acc = fmaf(ky[1], vrow(Cm, i, j - 1, k), acc);
        acc = fmaf(ky[3], vrow(Cm, i, j + 1, k), acc); acc = fmaf(ky[4], vrow(Cm, i, j + 2, k), acc);
        acc = fmaf(kz[0], Cm[hzm2], acc); acc = fmaf(kz[1], Cm[h - oz], acc);
        acc = fmaf(kz[3], Cm[h + oz], acc); acc = fmaf(kz[4], Cm[hzp2], acc);
        b[m] = acc + ((m == 0 || m == 3 || m == 5) ? mc.dtwi : 0.0f);
        x[m] = c0;
    }
    // velocity gradient with zero velocity beyond the ghost row
    Lyap9 A;
    A.a00 = mc.gx1 * (U[h] - U[h - ox]);
    A.a10 = mc.gx4 * (-vrow(V, i - 1, j - 1, k) + vrow(V, i + 1, j - 1, k) - V[h - ox] + V[h + ox]);
    A.a20 = mc.gx4 * (-W[h - ox - oz] + W[h + ox - oz] - W[h - ox] + W[h + ox]);
    A.a01 = mc.gy4 * (-vrow(U, i - 1, j - 1, k) - vrow(U, i, j - 1, k) + vrow(U, i - 1, j + 1, k) + vrow(U, i, j + 1, k));
    A.a11 = mc.gy1 * (V[h] - vrow(V, i, j - 1, k));
    A.a21 = mc.gy4 * (-vrow(W, i, j - 1, k - 1) + vrow(W, i, j + 1, k - 1) - vrow(W, i, j - 1, k) + vrow(W, i, j + 1, k));
    A.a02 = mc.gz4 * (-U[h - ox - oz] - U[h - oz] + U[h - ox + oz] + U[h + oz]);
    A.a12 = mc.gz4 * (-vrow(V, i, j - 1, k - 1) - V[h - oz] + vrow(V, i, j - 1, k + 1) + V[h + oz]);
    A.a22 = mc.gz1 * (W[h] - W[h - oz]);
    (void)oy;
    // the fast Newton of k_update3_f, then (rarely) the exact one from the start
    const float x0[6] = {x[0], x[1], x[2], x[3], x[4], x[5]};
    const int fast_max = min(NEWTON_FAST_MAX, ph.newton_itrmax);
    int itr = newton_fast_f(x, b, A, mc, ph.lp2, fast_max);
    if (itr > fast_max && fast_max < ph.newton_itrmax) {
#pragma unroll
        for (int m = 0; m < 6; ++m) x[m] = x0[m];
        itr = fast_max + newton_exact_f(x, b, A, mc.dtwi, mc.lp2f, ph.lp2, mc.epsf, ph.newton_itrmax);
    }
    my_itr = (unsigned long long)itr;
    my_unconv = itr > ph.newton_itrmax ? 1ull : 0ull;
#pragma unroll
    for (int m = 0; m < 6; ++m) Cn[(size_t)m * cs + h] = x[m];
    fpet[h] = peterlin_f(x[0], x[3], x[5], mc.lp2f, ph.lp2);
    }
    unsigned long long a = my_itr, b2 = my_unconv;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b2 += __shfl_down_sync(0xffffffffu, b2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&cnt->newton_iters, a);
        if (b2) atomicAdd(&cnt->newton_unconverged, b2);
    }
}

// ---------------------------------------------------------------------------
// Polymer, 2D (fenep_2d.f90:138-393) in FP32: the closed-form eigenvalues of
// the 2 x 2 candidate faces, the "last candidate >= running best" rule, Cstar
// with 1/4 weights, and the Newton iteration of the 3-unknown Lyapunov system
// with its Jacobian assembled analytically (the FP64 step differentiates by
// finite differences, which FP32 cannot resolve).

__device__ inline float face_p_f(int idx, float cm, float c0, float cp) {
    switch (idx) {
    case 1: return c0 * 1.5f - cp * 0.5f;
    case 2: return cm * 0.5f + c0 * 0.5f;
    case 3: return cm * 0.25f + c0 - cp * 0.25f;
    default: return c0;
    }
}
__device__ inline float face_n_f(int idx, float cm, float c0, float cp) {
    switch (idx) {
    case 1: return c0 * 0.5f + cp * 0.5f;
    case 2: return -cm * 0.5f + c0 * 1.5f;
    case 3: return -cm * 0.25f + c0 + cp * 0.25f;
    default: return c0;
    }
}

// smaller eigenvalue of the symmetric 2 x 2 (a0 a1; a1 a2)
__device__ inline float eig2_min_f(float a0, float a1, float a2) {
    const float d = (a0 - a2) * (a0 - a2) + 4.0f * (a1 * a1);
    return (a0 + a2 - sqrtf(d)) * 0.5f;
}

// the reference's index (0: no candidate qualified, the cell value)
__device__ inline int select2_f(const float (&cm)[3], const float (&c0)[3], const float (&cp)[3]) {
    int index = 0;
    float best = 0.0f;
#pragma unroll
    for (int l = 1; l <= 3; ++l) {
        float pt[3], nt[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            pt[m] = face_p_f(l, cm[m], c0[m], cp[m]);
            nt[m] = face_n_f(l, cm[m], c0[m], cp[m]);
        }
        const float ep = eig2_min_f(pt[0], pt[1], pt[2]), en = eig2_min_f(nt[0], nt[1], nt[2]);
        // NaN eigenvalues are skipped, as in the reference's minval
        float mv = ep;
        bool found = !isnan(ep);
        if (!isnan(en) && (!found || en < mv)) { mv = en; found = true; }
        if (found && mv >= best) { index = l; best = mv; }
    }
    return index;
}

// value of a C component at row jj of column (i, k): zero beyond the ghost
// rows of a wall channel
__device__ inline float crow_f(const float *A, const Geo &g, int i, int jj, int k) {
    return (jj < 0 || jj > g.ny + 1) ? 0.0f : A[hix(g, i, jj, k)];
}

__global__ void k_codes2_f(const float *__restrict__ C, uint8_t *__restrict__ codes, uint8_t *__restrict__ codes_g,
                           Geo g, int cs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    if (i > g.nx || j >= prow0(g) + prows(g)) return;
    const int k = 1, h = hix(g, i, j, k);
    float c0[3], cm[3], cp[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) c0[m] = C[(size_t)m * cs + h];
    int code = 0;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const float *Cm = C + (size_t)m * cs;
            if (d == 1 && g.walls) {
                cm[m] = crow_f(Cm, g, i, j - 1, k);
                cp[m] = crow_f(Cm, g, i, j + 1, k);
            } else {
                const int od = d == 0 ? 1 : g.sx;
                cm[m] = Cm[h - od];
                cp[m] = Cm[h + od];
            }
        }
        const int idx = select2_f(cm, c0, cp);   // 0..3; 0 -> the cell value (code 3)
        code |= (idx == 0 ? 3 : idx - 1) << (2 * d);
    }
    if (j >= 1 && j <= g.ny) codes[qix(g, i, j, k)] = (uint8_t)code;
    else codes_g[gcix(g, i, j, k)] = (uint8_t)code;
}

__device__ inline int code2_at(const uint8_t *codes, const uint8_t *codes_g, const Geo &g, int i, int j) {
    return (j >= 1 && j <= g.ny) ? codes[qix(g, i, j, 1)] : codes_g[gcix(g, i, j, 1)];
}

// Newton for G(x) = M x + a(x) x - b = 0, x = (c11, c12, c22), with M the 2D
// Lyapunov operator of A = (grad u)^T and a = 1 + f(x) dt/Wi (lyap_func2 of
// the FP64 step); the Jacobian is M + a I + (da/dtr) x (e1 + e3)^T.  The
// relative step test uses the larger of eps^2 and (8 ulp)^2: the 2D
// reference's eps (1e-10, fenep_2d.f90:291-293) is below FP32 resolution,
// and once the step is a few ulp of x the quadratic iteration has converged
// to FP32 rounding.  Returns the iterations taken, > itrmax when not
// converged.
__device__ __forceinline__ int newton2_f(float (&x)[3], const float (&b)[3], float a00, float a01, float a10, float a11,
                                const MixConst &mc, double lp2, int itrmax) {
    const float M[3][3] = {{2.0f * a00, 2.0f * a01, 0.0f}, {a10, a00 + a11, a01}, {0.0f, 2.0f * a10, 2.0f * a11}};
    const float ulp8 = 8.0f * FLT_EPSILON;
    const float eps2 = fmaxf(mc.eps2f, ulp8 * ulp8);
    int itr;
#pragma unroll 1
    for (itr = 1; itr <= itrmax; ++itr) {
        const float f = peterlin2_f(x[0], x[2], mc.lp2f, lp2);
        const float a = 1.0f + f * mc.dtwi;
        const float den = mc.lp2f - (x[0] + x[2]);
        const float cc = mc.dtwi * (mc.lp2f - 2.0f) / (den * den);
        float J[3][4];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            J[q][3] = M[q][0] * x[0] + M[q][1] * x[1] + M[q][2] * x[2] + a * x[q] - b[q];
#pragma unroll
            for (int w = 0; w < 3; ++w) J[q][w] = M[q][w] + (w != 1 ? cc * x[q] : 0.0f) + (w == q ? a : 0.0f);
        }
        // Gauss-Jordan without pivoting: J is dominated by its diagonal a >= 1
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float inv = 1.0f / J[k][k];
#pragma unroll
            for (int q = k + 1; q < 4; ++q) J[k][q] *= inv;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q == k) continue;
                const float fr = J[q][k];
#pragma unroll
                for (int w = k + 1; w < 4; ++w) J[q][w] -= fr * J[k][w];
            }
        }
        float sr = 0.0f, sx = 0.0f;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            x[m] -= J[m][3];
            sr = fmaf(J[m][3], J[m][3], sr);
            sx = fmaf(x[m], x[m], sx);
        }
        if (!(sr > eps2 * sx)) break;   // the relative step test, also ends on NaN
    }
    return itr;
}

__global__ void __launch_bounds__(128) k_update2_f(const float *__restrict__ C, float *__restrict__ Cn,
                                                   float *__restrict__ fpet, const uint8_t *__restrict__ codes,
                                                   const uint8_t *__restrict__ codes_g, const float *__restrict__ U,
                                                   const float *__restrict__ V, Geo g, Phys ph, MixConst mc, int cs,
                                                   StepCounters *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const int k = 1;
    const bool active = i <= g.nx && j < prow0(g) + prows(g);
    unsigned long long my_itr = 0, my_unconv = 0;
    if (active) {
        const int h = hix(g, i, j, k);
        const int cself = code2_at(codes, codes_g, g, i, j);
        const int cxm = code2_at(codes, codes_g, g, wrapx(g, i - 1), j) & 3;
        const int cxp = code2_at(codes, codes_g, g, wrapx(g, i + 1), j) & 3;
        int jm = j - 1, jp = j + 1;
        if (!g.walls) { jm = wrapy(g, jm); jp = wrapy(g, jp); }
        const int cym = jm < 0 ? 3 : (code2_at(codes, codes_g, g, i, jm) >> 2) & 3;
        const int cyp = jp > g.ny + 1 ? 3 : (code2_at(codes, codes_g, g, i, jp) >> 2) & 3;
        const int isx = (cself & 3) + 1, isy = ((cself >> 2) & 3) + 1;
        const int hxm = hix(g, wrapx(g, i - 1), j, k), hxp = hix(g, wrapx(g, i + 1), j, k);
        const int ox = 1;
        const float u1 = U[hix(g, i - 1, j, k)], u2 = U[h];
        const float v1 = crow_f(V, g, i, j - 1, k), v2 = V[h];
        // Cstar upwind coefficients with the 2D weight 1/4 (fenep_2d.f90)
        const float s1 = (-u2 + fabsf(u2)) * mc.sx, s2 = 0.25f + (-u2 - fabsf(u2)) * mc.sx;
        const float s3 = 0.25f + (u1 - fabsf(u1)) * mc.sx, s4 = (u1 + fabsf(u1)) * mc.sx;
        const float s5 = (-v2 + fabsf(v2)) * mc.sy, s6 = 0.25f + (-v2 - fabsf(v2)) * mc.sy;
        const float s7 = 0.25f + (v1 - fabsf(v1)) * mc.sy, s8 = (v1 + fabsf(v1)) * mc.sy;
        float b[3], x[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const float *Cm = C + (size_t)m * cs;
            const float c0 = Cm[h];
            const float pxm = face_p_f(isx, Cm[h - ox], c0, Cm[h + ox]);
            const float nxp = face_n_f(isx, Cm[h - ox], c0, Cm[h + ox]);
            const float pxp = face_p_f(cxp + 1, Cm[hxp - ox], Cm[hxp], Cm[hxp + ox]);
            const float nxm = face_n_f(cxm + 1, Cm[hxm - ox], Cm[hxm], Cm[hxm + ox]);
            float pym, nyp, pyp, nym;
            if (!g.walls) {
                const int hym = hix(g, i, jm, k), hyp = hix(g, i, jp, k), oy = g.sx;
                pym = face_p_f(isy, Cm[h - oy], c0, Cm[h + oy]);
                nyp = face_n_f(isy, Cm[h - oy], c0, Cm[h + oy]);
                pyp = face_p_f(cyp + 1, Cm[hyp - oy], Cm[hyp], Cm[hyp + oy]);
                nym = face_n_f(cym + 1, Cm[hym - oy], Cm[hym], Cm[hym + oy]);
            } else {
                const float ym2 = crow_f(Cm, g, i, j - 2, k), ym1 = crow_f(Cm, g, i, j - 1, k);
                const float yp1 = crow_f(Cm, g, i, j + 1, k), yp2 = crow_f(Cm, g, i, j + 2, k);
                pym = face_p_f(isy, ym1, c0, yp1);
                nyp = face_n_f(isy, ym1, c0, yp1);
                pyp = face_p_f(cyp + 1, c0, yp1, yp2);
                nym = face_n_f(cym + 1, ym2, ym1, c0);
            }
            b[m] = s3 * pxm + s1 * pxp + s4 * nxm + s2 * nxp + s7 * pym + s5 * pyp + s8 * nym + s6 * nyp;
            x[m] = c0;
        }
        b[0] += mc.dtwi;
        b[2] += mc.dtwi;
        auto u = [&](int a, int bb) { return crow_f(U, g, a, bb, k); };
        auto v = [&](int a, int bb) { return crow_f(V, g, a, bb, k); };
        // the velocity gradient of fenep_2d.f90 (A0) and its transpose A
        const float g00 = mc.gx1 * (u(i, j) - u(i - 1, j));
        const float g01 = mc.gx4 * (-v(i - 1, j - 1) + v(i + 1, j - 1) - v(i - 1, j) + v(i + 1, j));
        const float g10 = mc.gy4 * (-u(i - 1, j - 1) - u(i, j - 1) + u(i - 1, j + 1) + u(i, j + 1));
        const float g11 = mc.gy1 * (v(i, j) - v(i, j - 1));
        const int itr = newton2_f(x, b, g00, g10, g01, g11, mc, ph.lp2, ph.newton_itrmax);
        my_itr = (unsigned long long)itr;
        my_unconv = itr > ph.newton_itrmax ? 1ull : 0ull;
#pragma unroll
        for (int m = 0; m < 3; ++m) Cn[(size_t)m * cs + h] = x[m];
        fpet[h] = peterlin2_f(x[0], x[2], mc.lp2f, ph.lp2);
    }
    unsigned long long a = my_itr, b2 = my_unconv;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b2 += __shfl_down_sync(0xffffffffu, b2, o);
    }
    if (((threadIdx.x + blockDim.x * threadIdx.y) & 31) == 0) {
        if (a) atomicAdd(&cnt->newton_iters, a);
        if (b2) atomicAdd(&cnt->newton_unconverged, b2);
    }
}

// ---------------------------------------------------------------------------
// Momentum right-hand side in increment form: Q_c = dt * R_c (FP32).
struct MomArgsF {
    const float *U, *V, *W;   // hi parts of the velocity
    const float *Ph, *Pl;     // pressure (df64)
    const float *C, *fpet;
    float *A0[3], *T0[3];
    const float *F[3];        // body force, or null when uniform (value in Fu)
    float Fu[3];
    float *Q[3];
    int cs;
    int polymer, ab2_first;
    float coef_t, vis;
    float dt;                 // dt rounded on the host (a per-thread FP64 conversion used the FP64 pipe)
};

// DIM 2: the 2D stress of C = (xx, xy, yy) and no z terms (W = 0)
template <int DIM>
__device__ __forceinline__ void momentum_f(const MomArgsF &a, const Geo &g, const MixConst &mc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const int o = qix(g, i, j, k), h = hix(g, i, j, k);
    const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
    const float ix = mc.ix, iy = mc.iy, iz = mc.iz;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    if (a.polymer) {
        // polymer_stress (fenep.f90:645-691) with C0 = f(C) C - I on the fly
        const int cs = a.cs;
        const float *C = a.C, *fp = a.fpet;
        if constexpr (DIM == 3) {
            auto c0 = [&](int m, int hh) {
                const float e = (m == 1 || m == 4 || m == 6) ? 1.0f : 0.0f;
                return fp[hh] * C[(size_t)(m - 1) * cs + hh] - e;
            };
            const float sx = (c0(1, h + ox) - c0(1, h)) * ix
                           + (-c0(2, h - oy) - c0(2, h + ox - oy) + c0(2, h + oy) + c0(2, h + ox + oy)) * (0.25f * iy)
                           + (-c0(3, h - oz) - c0(3, h + ox - oz) + c0(3, h + oz) + c0(3, h + ox + oz)) * (0.25f * iz);
            const float sy = (-c0(2, h - ox) + c0(2, h + ox) - c0(2, h - ox + oy) + c0(2, h + ox + oy)) * (0.25f * ix)
                           + (c0(4, h + oy) - c0(4, h)) * iy
                           + (-c0(5, h - oz) - c0(5, h + oy - oz) + c0(5, h + oz) + c0(5, h + oy + oz)) * (0.25f * iz);
            const float sz = (-c0(3, h - ox) + c0(3, h + ox) - c0(3, h - ox + oz) + c0(3, h + ox + oz)) * (0.25f * ix)
                           + (-c0(5, h - oy) + c0(5, h + oy) - c0(5, h - oy + oz) + c0(5, h + oy + oz)) * (0.25f * iy)
                           + (c0(6, h + oz) - c0(6, h)) * iz;
            tx = a.coef_t * sx; ty = a.coef_t * sy; tz = a.coef_t * sz;
        } else {
            auto c0 = [&](int m, int hh) {
                const float e = (m == 1 || m == 3) ? 1.0f : 0.0f;
                return fp[hh] * C[(size_t)(m - 1) * cs + hh] - e;
            };
            const float sx = (c0(1, h + ox) - c0(1, h)) * ix
                           + (-c0(2, h - oy) - c0(2, h + ox - oy) + c0(2, h + oy) + c0(2, h + ox + oy)) * (0.25f * iy);
            const float sy = (-c0(2, h - ox) + c0(2, h + ox) - c0(2, h - ox + oy) + c0(2, h + ox + oy)) * (0.25f * ix)
                           + (c0(3, h + oy) - c0(3, h)) * iy;
            tx = a.coef_t * sx; ty = a.coef_t * sy;
        }
    }
    const float *U = a.U, *V = a.V, *W = a.W;
    auto u = [&](int hh) { return U[hh]; };
    auto v = [&](int hh) { return V[hh]; };
    auto w = [&](int hh) { return W[hh]; };
    // convection (fenep.f90:694-734), divergence form, and viscous
    // (fenep.f90:736-770)
    const float uc = u(h), vc = v(h);
    const float uxm = u(h - ox), uxp = u(h + ox), uym = u(h - oy), uyp = u(h + oy);
    const float vxm = v(h - ox), vxp = v(h + ox), vym = v(h - oy), vyp = v(h + oy);
    float t1 = 0.5f * (uxm + uc), t2 = 0.5f * (uc + uxp);
    float ax = (t2 * t2 - t1 * t1) * ix
             + (0.25f * (vc + v(h + ox)) * (uc + uyp) - 0.25f * (vym + v(h + ox - oy)) * (uym + uc)) * iy;
    float t3 = 0.5f * (vym + vc), t4 = 0.5f * (vc + vyp);
    float ay = (0.25f * (uc + uyp) * (vc + vxp) - 0.25f * (uxm + u(h - ox + oy)) * (vxm + vc)) * ix
             + (t4 * t4 - t3 * t3) * iy;
    float bx = (uxm - 2.0f * uc + uxp) * mc.ix2 + (uym - 2.0f * uc + uyp) * mc.iy2;
    float by = (vxm - 2.0f * vc + vxp) * mc.ix2 + (vym - 2.0f * vc + vyp) * mc.iy2;
    float az = 0.0f, bz = 0.0f;
    if constexpr (DIM == 3) {
        const float wc = w(h);
        const float uzm = u(h - oz), uzp = u(h + oz), vzm = v(h - oz), vzp = v(h + oz);
        const float wxm = w(h - ox), wxp = w(h + ox), wym = w(h - oy), wyp = w(h + oy), wzm = w(h - oz), wzp = w(h + oz);
        ax += (0.25f * (wc + w(h + ox)) * (uc + uzp) - 0.25f * (wzm + w(h + ox - oz)) * (uzm + uc)) * iz;
        ay += (0.25f * (wc + w(h + oy)) * (vc + vzp) - 0.25f * (wzm + w(h + oy - oz)) * (vzm + vc)) * iz;
        float t5 = 0.5f * (wzm + wc), t6 = 0.5f * (wc + wzp);
        az = (0.25f * (uc + uzp) * (wc + wxp) - 0.25f * (uxm + u(h - ox + oz)) * (wxm + wc)) * ix
           + (0.25f * (vc + vzp) * (wc + wyp) - 0.25f * (vym + v(h - oy + oz)) * (wym + wc)) * iy
           + (t6 * t6 - t5 * t5) * iz;
        bx += (uzm - 2.0f * uc + uzp) * mc.iz2;
        by += (vzm - 2.0f * vc + vzp) * mc.iz2;
        bz = (wxm - 2.0f * wc + wxp) * mc.ix2 + (wym - 2.0f * wc + wyp) * mc.iy2 + (wzm - 2.0f * wc + wzp) * mc.iz2;
    }
    const float A[3] = {-ax, -ay, -az};
    const float B[3] = {a.vis * bx, a.vis * by, a.vis * bz};
    const float T[3] = {tx, ty, tz};
    const int hp[3] = {h + ox, h + oy, h + oz};
    const float id[3] = {ix, iy, iz};
    const float ph0 = a.Ph[h], pl0 = a.Pl[h];
    const float dt = a.dt;
    // every load of the components before the first store (the history
    // arrays are read and written in place)
    float a0[DIM], t0[DIM], php[DIM], plp[DIM], fb[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        a0[c] = a.ab2_first ? A[c] : a.A0[c][o];
        t0[c] = a.ab2_first ? T[c] : a.T0[c][o];
        php[c] = a.Ph[hp[c]];
        plp[c] = a.Pl[hp[c]];
        fb[c] = a.F[c] ? a.F[c][o] : a.Fu[c];
    }
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        // pressure difference from the df64 pair: the hi difference is
        // correctly rounded, the lo difference carries the rest
        const float gp = -((php[c] - ph0) + (plp[c] - pl0)) * id[c];
        const float r = gp + 0.5f * (3.0f * A[c] - a0[c]) + B[c] + 0.5f * (T[c] + t0[c]) + fb[c];
        a.Q[c][o] = dt * r;
        a.A0[c][o] = A[c];
        a.T0[c][o] = T[c];
    }
}

__global__ void __launch_bounds__(256, 6) k_momentum3_f(MomArgsF a, Geo g, MixConst mc) { momentum_f<3>(a, g, mc); }
__global__ void __launch_bounds__(256, 6) k_momentum2_f(MomArgsF a, Geo g, MixConst mc) { momentum_f<2>(a, g, mc); }

// ---------------------------------------------------------------------------
// IBM (fenep_mpi.f90:1794-1929).  Ua = U + dt R at the stencil points with the
// boundary values that the reference gives Ua (PBM / wall rules).
// Ua in df64 (the velocity pair plus the FP32 increment)
__device__ inline df ua_at(const Geo &g, const float *Uh, const float *Ul, const float *Qc, int comp, int i, int j,
                           int k, df uw2) {
    const int ii = wrapx(g, i), kk = wrapz(g, k);
    auto u = [&](int q) { return df{Uh[q], Ul[q]}; };
    if (j >= 1 && j <= g.ny) {
        if (g.walls && comp == 1 && j == g.ny) return df{0.0f, 0.0f};
        return df_add_f(u(hix(g, i, j, k)), Qc[qix(g, ii, j, kk)]);
    }
    if (!g.walls) return df_add_f(u(hix(g, i, j, k)), Qc[qix(g, ii, wrapy(g, j), kk)]);
    if (comp == 1) return df{0.0f, 0.0f};
    const int jj = j == 0 ? 1 : g.ny;
    const df inner = df_add_f(u(hix(g, ii, jj, kk)), Qc[qix(g, ii, jj, kk)]);
    return (comp == 0 && j != 0) ? df_sub(uw2, inner) : df_neg(inner);
}

// U* = U^n + dU (the last Helmholtz solution) at the stencil points, with the
// boundary values the FP64 step gives Up (the increments have no halo pass:
// x and z wrap, the wall solves write the ghost rows of dU)
__device__ inline df ustar_at(const Geo &g, const float *Uh, const float *Ul, const float *D, int comp, int i, int j,
                              int k, df uw2) {
    const int ii = wrapx(g, i), kk = wrapz(g, k);
    auto us = [&](int jj) {
        const int h = hix(g, i, jj, k);
        return df_add_f(df{Uh[h], Ul[h]}, D[hix(g, ii, jj, kk)]);
    };
    if (j >= 1 && j <= g.ny) {
        if (g.walls && comp == 1 && j == g.ny) return df{0.0f, 0.0f};
        return us(j);
    }
    if (!g.walls) {
        const int jw = wrapy(g, j), h = hix(g, i, j, k);
        return df_add_f(df{Uh[h], Ul[h]}, D[hix(g, ii, jw, kk)]);
    }
    if (comp == 1) return df{0.0f, 0.0f};
    const int jj = j == 0 ? 1 : g.ny;
    const df inner = us(jj);
    return (comp == 0 && j != 0) ? df_sub(uw2, inner) : df_neg(inner);
}

struct IbmArgsF {
    const float *D[3];               // forcing iteration > 1: the increments dU of the last solve
    int mode;                        // 0: interpolate Ua = U + Q; 1: interpolate U* = U + dU
    int accumulate;                  // forcing iteration > 1: Fc += (Uc - Ub)/dt
    const float *Qb[3];              // base of the spread: Q itself (first iteration) or the
                                     // right-hand sides saved before the first spread
    const double *mu, *mv;
    const int *mcyl;
    int nm;
    const float *wx[3], *wy[3];      // per marker, 3 weights each
    const int *i0[3], *j0[3];
    float wz[3][3];                  // per component, offset k - n = -1, 0, 1
    const float *Uh[3], *Ul[3];      // velocity (df64)
    const float *Qc[3];
    double *Fc[3];
    float *Fcf[3];                   // FP32 copies of Fc, read by the spreading
    const int *off[3], *idx[3];
    const float *cw[3];              // per list entry: x weight * y weight
    const int *act[3];
    int nact[3];
    float *Q[3];
    df uw2;                          // 2 * upper wall speed
    double idt;                      // 1 / dt
    float dtf;                       // dt
};

// One marker per threadIdx.x and one z plane of its 3 x 3 x 3 stencil per
// threadIdx.y (blocks of 32 x 3): each thread sums 9 points in df64, and the
// three plane sums are added in plane order.
__global__ void __launch_bounds__(96) k_ibm_interp_f(IbmArgsF a, Geo g) {
    __shared__ df part[3][32];
    const int m = blockIdx.x * 32 + threadIdx.x;
    const int dk = threadIdx.y;
    const int n = blockIdx.y + 1;
    const int comp = blockIdx.z;
    df ub{0.0f, 0.0f};
    if (m < a.nm) {
        const int i0 = a.i0[comp][m], j0 = a.j0[comp][m];
        const float *wx = a.wx[comp] + 3 * m, *wy = a.wy[comp] + 3 * m;
        const int k = n - 1 + dk;
        const float wz = a.wz[comp][dk];
        // a stencil inside the interior columns and rows (no x wrap, no wall
        // rule) reads its 9 points at fixed offsets from one base index; the
        // values and their order of summation are those of ua_at / ustar_at
        const bool inner = i0 >= 1 && i0 + 2 <= g.nx && j0 >= 1 && j0 + 2 <= g.ny &&
                           !(g.walls && comp == 1 && j0 + 2 == g.ny);
        if (inner) {
            const int kk = wrapz(g, k);
            const int hb = hix(g, i0, j0, k);
            const float *Uh = a.Uh[comp], *Ul = a.Ul[comp];
            const float *X = a.mode ? a.D[comp] : a.Qc[comp];
            const int xb = a.mode ? hix(g, i0, j0, kk) : qix(g, i0, j0, kk);
            const int xs = a.mode ? g.sx : g.nx;
            float uh[9], ul[9], xv[9];
#pragma unroll
            for (int dj = 0; dj < 3; ++dj)
#pragma unroll
                for (int di = 0; di < 3; ++di) {
                    const int h = hb + di + g.sx * dj;
                    uh[3 * dj + di] = Uh[h];
                    ul[3 * dj + di] = Ul[h];
                    xv[3 * dj + di] = X[xb + di + xs * dj];
                }
#pragma unroll
            for (int dj = 0; dj < 3; ++dj)
#pragma unroll
                for (int di = 0; di < 3; ++di) {
                    const float w = wx[di] * wy[dj] * wz;
                    const int q = 3 * dj + di;
                    ub = df_add(ub, df_mul_f(df_add_f(df{uh[q], ul[q]}, xv[q]), w));
                }
        } else {
#pragma unroll
            for (int dj = 0; dj < 3; ++dj)
#pragma unroll
                for (int di = 0; di < 3; ++di) {
                    const float w = wx[di] * wy[dj] * wz;
                    const df uv = a.mode ? ustar_at(g, a.Uh[comp], a.Ul[comp], a.D[comp], comp, i0 + di, j0 + dj, k, a.uw2)
                                         : ua_at(g, a.Uh[comp], a.Ul[comp], a.Qc[comp], comp, i0 + di, j0 + dj, k, a.uw2);
                    ub = df_add(ub, df_mul_f(uv, w));
                }
        }
    }
    part[dk][threadIdx.x] = ub;
    __syncthreads();
    if (dk == 0 && m < a.nm) {
        const df s3 = df_add(df_add(part[0][threadIdx.x], part[1][threadIdx.x]), part[2][threadIdx.x]);
        const double uc = comp == 0 ? a.mu[m] : (comp == 1 ? a.mv[m] : 0.0);
        const size_t q = m + (size_t)a.nm * (n - 1);
        double *fc = &a.Fc[comp][q];
        const double v = (a.accumulate ? *fc : 0.0) + (uc - ((double)s3.hi + (double)s3.lo)) * a.idt;
        *fc = v;
        // one conversion per marker and plane: the spreading reads each
        // force once per list entry and plane, and a double-to-float
        // conversion there ran on the FP64 pipe
        a.Fcf[comp][q] = (float)v;
    }
}

// the spread force enters Q = dt (R + f), an FP32 field, so it is summed in FP32
__device__ inline float spread_at_f(const IbmArgsF &a, const Geo &g, int comp, int ie, int je, int ke) {
    const int col = ie + g.sx * je;
    const int b = a.off[comp][col], e = a.off[comp][col + 1];
    if (b == e) return 0.0f;
    // each list entry (marker, x y weight) is read once for the (up to) three
    // marker planes whose z stencil covers plane ke
    float acc = 0.0f;
    const int nlo = max(ke - 1, 1), nhi = min(ke + 1, g.nz);
    const float *Fc = a.Fcf[comp];
    const size_t nm = (size_t)a.nm;
    for (int q = b; q < e; ++q) {
        const int m = a.idx[comp][q];
        const float cw = a.cw[comp][q];
        for (int n = nlo; n <= nhi; ++n)
            acc = fmaf(Fc[m + nm * (n - 1)], cw * a.wz[comp][ke - n + 1], acc);
    }
    return acc;
}

// spreading with the periodic fold (ibm_PBM) over the active columns only;
// Q = dt*(R + f) for those cells
__global__ void k_ibm_spread_f(IbmArgsF a, Geo g) {
    const int comp = blockIdx.z;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y + 1;
    if (c >= a.nact[comp]) return;
    const int col = a.act[comp][c];
    const int i = col % g.nx + 1, j = col / g.nx + 1;
    int xs[2] = {i, -1}, ys[2] = {j, -1}, zs[2] = {k, -1};
    if (i == 1) xs[1] = g.nx + 1; else if (i == g.nx) xs[1] = 0;
    if (!g.walls) { if (j == 1) ys[1] = g.ny + 1; else if (j == g.ny) ys[1] = 0; }
    if (k == 1) zs[1] = g.nz + 1; else if (k == g.nz) zs[1] = 0;
    float f = 0.0f;
#pragma unroll
    for (int zz = 0; zz < 2; ++zz) {
        if (zs[zz] < 0) continue;
#pragma unroll
        for (int yy = 0; yy < 2; ++yy) {
            if (ys[yy] < 0) continue;
#pragma unroll
            for (int xx = 0; xx < 2; ++xx) {
                if (xs[xx] < 0) continue;
                f += spread_at_f(a, g, comp, xs[xx], ys[yy], zs[zz]);
            }
        }
    }
    const int o = qix(g, i, j, k);
    a.Q[comp][o] = fmaf(a.dtf, f, a.Qb[comp][o]);
}

// ---------------------------------------------------------------------------
// Pressure solve and projection on the df64 state.
// Index of the neighbour (d = -1 / +1 along axis c) of interior cell
// (i, j, k) for a field whose halo has not been filled: periodic wrap, and
// the Neumann copy (P-kind boundary value) at the walls.
__device__ __forceinline__ int nbr_p(const Geo &g, int i, int j, int k, int c, int d) {
    if (c == 0) return hix(g, wrapx(g, i + d), j, k);
    if (c == 2) return hix(g, i, j, wrapz(g, k + d));
    const int jj = g.walls ? max(1, min(g.ny, j + d)) : wrapy(g, j + d);
    return hix(g, i, jj, k);
}

// The df64 state of one field
struct DfF {
    float *hi, *lo;
    __device__ __forceinline__ df at(int q) const { return df{hi[q], lo[q]}; }
    __device__ __forceinline__ void set(int q, df v) const { hi[q] = v.hi; lo[q] = v.lo; }
};

// The three df64 kernels of the pressure stage take two cells per thread,
// (i, j, k) and (i, j, k + 1) with k odd, in the two lanes of FP32x2 pairs:
// every df64 operation runs once on the pair (the packed routines of
// f8_df64.cuh, lane-wise identical to the scalar ones), the z neighbours
// shared by the two cells are loaded once, and every load is issued before
// the first store.  For odd NZ the last thread's second lane repeats the
// first cell and is not stored.
struct Pair {
    int h, hb;    // the two cells (hb = h when there is no second cell)
    bool two;
};

__device__ __forceinline__ bool pair_of(const Geo &g, int &i, int &j, int &k, Pair &p) {
    i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    k = 2 * blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return false;
    p.two = k + 1 <= g.nz;
    p.h = hix(g, i, j, k);
    p.hb = p.two ? p.h + g.sx * g.sy : p.h;
    return true;
}

__device__ __forceinline__ df2 at2(const DfF &F, int a, int b) { return df2_pack(F.at(a), F.at(b)); }
__device__ __forceinline__ float2 at2f(const float *F, int a, int b) { return make_float2(F[a], F[b]); }
__device__ __forceinline__ df2 bcast(df a) { return df2_pack(a, a); }

// Poisson right-hand side div(U^n + dU)/dt (fenep.f90:1494-1510) in df64:
// each face difference of the state and of the FP32 increment is formed
// exactly, scaled by the df64 1/dX, and summed (x, y, z in that order).
__global__ void __launch_bounds__(256, 8) k_poisson_rhs_df(DfF U, DfF V, DfF W, const float *__restrict__ dU, const float *__restrict__ dV,
                                 const float *__restrict__ dW, float *__restrict__ Rh, float *__restrict__ Rl, Geo g,
                                 MixConst mc) {
    int i, j, k;
    Pair p;
    if (!pair_of(g, i, j, k, p)) return;
    const int h = p.h, hb = p.hb, oy = g.sx;
    // the increments have no halo pass: periodic neighbours by wrapping; at
    // the lower wall dV(j = 0) = 0 is the ghost row the wall solve wrote
    const int kb = p.two ? k + 1 : k;
    const int xa = hix(g, wrapx(g, i - 1), j, k), xb = hix(g, wrapx(g, i - 1), j, kb);
    const int ya = g.walls ? h - oy : hix(g, i, wrapy(g, j - 1), k);
    const int yb = g.walls ? hb - oy : hix(g, i, wrapy(g, j - 1), kb);
    const int za = hix(g, i, j, wrapz(g, k - 1));
    // loads: W and dW at k - 1 .. k + 1, the cells' own values and their
    // x / y neighbours
    const df2 Uc = at2(U, h, hb), Um = at2(U, h - 1, hb - 1);
    const df2 Vc = at2(V, h, hb), Vm = at2(V, h - oy, hb - oy);
    const df W0 = W.at(hix(g, i, j, k - 1)), W1 = W.at(h), W2 = W.at(hb);
    const float2 dUc = at2f(dU, h, hb), dUm = at2f(dU, xa, xb);
    const float2 dVc = at2f(dV, h, hb), dVm = at2f(dV, ya, yb);
    const float dW0 = dW[za], dW1 = dW[h], dW2 = dW[hb];
    df2 a = df2_add(df2_sub(Uc, Um), df2_diff_ff(dUc, dUm));
    df2 sum = df2_mul(a, bcast(mc.di[0]));
    a = df2_add(df2_sub(Vc, Vm), df2_diff_ff(dVc, dVm));
    sum = df2_add(sum, df2_mul(a, bcast(mc.di[1])));
    a = df2_add(df2_sub(df2_pack(W1, W2), df2_pack(W0, W1)),
                df2_diff_ff(make_float2(dW1, dW2), make_float2(dW0, dW1)));
    sum = df2_add(sum, df2_mul(a, bcast(mc.di[2])));
    sum = df2_mul(sum, bcast(mc.idt));
    const int oa = qix(g, i, j, k);
    Rh[oa] = sum.hi.x;
    Rl[oa] = sum.lo.x;
    if (p.two) {
        const int ob = oa + g.nx * g.ny;
        Rh[ob] = sum.hi.y;
        Rl[ob] = sum.lo.y;
    }
}

// defect r = rhs - L_h Phi in df64.  Phi is the first FP32 solve's result
// (no low part), so each one-sided difference is the exact difference of two
// floats; the FP32 value of r drives the correction solve.
__global__ void k_defect_df(const float *__restrict__ Phi, const float *__restrict__ Rh, const float *__restrict__ Rl,
                            float *__restrict__ r, Geo g, MixConst mc) {
    int i, j, k;
    Pair p;
    if (!pair_of(g, i, j, k, p)) return;
    const int h = p.h, hb = p.hb, kb = p.two ? k + 1 : k;
    const int oa = qix(g, i, j, k), ob = p.two ? oa + g.nx * g.ny : oa;
    const float z0 = Phi[nbr_p(g, i, j, k, 2, -1)], z1 = Phi[h], z2 = Phi[p.two ? hb : nbr_p(g, i, j, k, 2, 1)];
    const float z3 = p.two ? Phi[nbr_p(g, i, j, kb, 2, 1)] : z2;
    const float2 c0 = make_float2(z1, p.two ? z2 : z1);
    const float2 pp[3] = {make_float2(Phi[nbr_p(g, i, j, k, 0, 1)], Phi[nbr_p(g, i, j, kb, 0, 1)]),
                          make_float2(Phi[nbr_p(g, i, j, k, 1, 1)], Phi[nbr_p(g, i, j, kb, 1, 1)]),
                          make_float2(z2, p.two ? z3 : z2)};
    const float2 pm[3] = {make_float2(Phi[nbr_p(g, i, j, k, 0, -1)], Phi[nbr_p(g, i, j, kb, 0, -1)]),
                          make_float2(Phi[nbr_p(g, i, j, k, 1, -1)], Phi[nbr_p(g, i, j, kb, 1, -1)]),
                          make_float2(z0, p.two ? z1 : z0)};
    df2 res{make_float2(Rh[oa], Rh[ob]), make_float2(Rl[oa], Rl[ob])};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const df2 dp = df2_diff_ff(pp[c], c0), dm = df2_diff_ff(c0, pm[c]);
        res = df2_sub(res, df2_mul(df2_sub(dp, dm), bcast(mc.di2[c])));
    }
    r[oa] = __fadd_rn(res.hi.x, res.lo.x);
    if (p.two) r[ob] = __fadd_rn(res.hi.y, res.lo.y);
}

// projection and SMAC pressure update (fenep.f90:1562-1604):
// U^{n+1} = U^n + (dU - dt/dX (Phi_{+1} - Phi)) in df64, and
// P^{n+1} = P^n + Phi - dt beta/(2 Re) L_h Phi with the small Laplacian term
// in FP32, for the two cells (k, k + 1) of a pair, from their loaded values:
// c0 = Phi at the cells, pp / pm = Phi at their +1 / -1 neighbours along x,
// y, z; Fv = U, V, W, Dv = dU, dV, dW, Pv = P at the cells.  Shared by the
// direct-load kernel and the staged (bulk-copy) kernel, so both give the
// same bits.
__device__ __forceinline__ void march_pair_math(const df2 &c0, const df2 (&pp)[3], const df2 (&pm)[3],
                                                const df2 (&Fv)[3], const float2 (&Dv)[3], const df2 &Pv,
                                                const MixConst &mc, df2 (&nu)[3], df2 &pn) {
    const float i2[3] = {mc.ix2, mc.iy2, mc.iz2};
    // the FP32 Laplacian of Phi, per lane as the scalar expression
    float lapx = 0.0f, lapy = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const df2 dp = df2_sub(pp[c], c0);
        const df2 inc = df2_add_f(df2_mul(dp, bcast(df_neg(mc.dtd[c]))), Dv[c]);
        nu[c] = df2_add(Fv[c], inc);
        const float2 dpf = add2_rn(sub2_rn(pp[c].hi, c0.hi), sub2_rn(pp[c].lo, c0.lo));
        const float2 dmf = add2_rn(sub2_rn(c0.hi, pm[c].hi), sub2_rn(c0.lo, pm[c].lo));
        lapx = __fadd_rn(lapx, __fmul_rn(__fsub_rn(dpf.x, dmf.x), i2[c]));
        lapy = __fadd_rn(lapy, __fmul_rn(__fsub_rn(dpf.y, dmf.y), i2[c]));
    }
    pn = df2_add_f(df2_add(Pv, c0), make_float2(__fmul_rn(-mc.pcf, lapx), __fmul_rn(-mc.pcf, lapy)));
}

// NaN watch on the new U (the reference stops on a NaN velocity,
// fenep_2d.f90:1974), counted in the projection kernels instead of in a
// separate pass
__device__ __forceinline__ void count_nonfinite(float2 unew, StepCounters *cnt) {
    const unsigned act = __activemask();
    const unsigned nb = __ballot_sync(act, !isfinite(unew.x) || !isfinite(unew.y));
    if (nb && (threadIdx.x & 31) == (unsigned)(__ffs(act) - 1)) atomicAdd(&cnt->nan_cells, (unsigned long long)__popc(nb));
}

__global__ void __launch_bounds__(256, 4) k_march_df(DfF U, DfF V, DfF W, DfF P, const float *__restrict__ dU, const float *__restrict__ dV,
                           const float *__restrict__ dW, DfF Phi, Geo g, MixConst mc, StepCounters *cnt) {
    int i, j, k;
    Pair p;
    const bool in = pair_of(g, i, j, k, p);
    float2 unew = make_float2(0.0f, 0.0f);
    if (in) {
        const int h = p.h, hb = p.hb, kb = p.two ? k + 1 : k;
        const DfF F[3] = {U, V, W};
        const float *const D[3] = {dU, dV, dW};
        // Phi at z = k-1 .. k+2 and the x / y neighbours of both cells
        const df z0 = Phi.at(nbr_p(g, i, j, k, 2, -1)), z1 = Phi.at(h);
        const df z2 = Phi.at(p.two ? hb : nbr_p(g, i, j, k, 2, 1));
        const df z3 = p.two ? Phi.at(nbr_p(g, i, j, kb, 2, 1)) : z2;
        const df2 c0 = df2_pack(z1, p.two ? z2 : z1);
        const df2 pp[3] = {df2_pack(Phi.at(nbr_p(g, i, j, k, 0, 1)), Phi.at(nbr_p(g, i, j, kb, 0, 1))),
                           df2_pack(Phi.at(nbr_p(g, i, j, k, 1, 1)), Phi.at(nbr_p(g, i, j, kb, 1, 1))),
                           df2_pack(z2, p.two ? z3 : z2)};
        const df2 pm[3] = {df2_pack(Phi.at(nbr_p(g, i, j, k, 0, -1)), Phi.at(nbr_p(g, i, j, kb, 0, -1))),
                           df2_pack(Phi.at(nbr_p(g, i, j, k, 1, -1)), Phi.at(nbr_p(g, i, j, kb, 1, -1))),
                           df2_pack(z0, p.two ? z1 : z0)};
        df2 Fv[3];
        float2 Dv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            Fv[c] = at2(F[c], h, hb);
            Dv[c] = at2f(D[c], h, hb);
        }
        const df2 Pv = at2(P, h, hb);
        df2 nu[3], pn;
        march_pair_math(c0, pp, pm, Fv, Dv, Pv, mc, nu, pn);
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c].set(h, df2_x(nu[c]));
        P.set(h, df2_x(pn));
        if (p.two) {
#pragma unroll
            for (int c = 0; c < 3; ++c) F[c].set(hb, df2_y(nu[c]));
            P.set(hb, df2_y(pn));
        }
        unew = make_float2(nu[0].hi.x, p.two ? nu[0].hi.y : 0.0f);
    }
    count_nonfinite(unew, cnt);
}

// ---------------------------------------------------------------------------
// The projection with its inputs staged in shared memory by bulk copies.
//
// A work unit is a tile of two y rows [jb, jb + 2) (jb even) over a run of z
// planes; the two rows of a plane are the two lanes of the pair arithmetic
// (march_pair_math is lane-wise the scalar arithmetic, so any pairing gives
// the same bits).  A step of a unit is one plane k: the 11 point-wise arrays
// (U, V, W, P hi / lo, dU, dV, dW) on the tile's rows, and Phi (hi / lo) on
// planes k - 1, k, k + 1, each on the tile's rows and on the row pairs holding
// the rows below and above them (periodic wrap or the Neumann copy at the
// walls, as nbr_p).  Full rows are copied (x halo included), a row pair per
// bulk copy of 8 SX bytes.
//
// The CTA is persistent: it walks its units (blockIdx.x, + gridDim.x, ...)
// as one sequence of steps, and thread 0 keeps the copies of the next D steps
// in flight: D + 1 buffers of point-wise planes, each with its mbarrier, and a
// ring of D + 5 Phi planes (a step uses three; a unit's first step loads three
// planes, the others one; runs are at least D + 1 planes long, so at most one
// unit starts among any D + 1 consecutive steps).
constexpr int MT_PW = 11;   // point-wise arrays
constexpr int MT_THREADS = 256;
constexpr int MT_MAXD = 4;

struct MarchTmaArgs {
    const float *pw[MT_PW];      // U.hi, U.lo, V.hi, V.lo, W.hi, W.lo, P.hi, P.lo, dU, dV, dW
    float *out[8];               // U.hi .. P.lo (written in place)
    const float *phi[2];         // Phi hi, lo
    int zruns;                   // z runs per tile
    int depth;                   // D: steps whose copies are in flight ahead of the one computed
};

inline size_t march_tma_smem(const Geo &g, int depth) {
    return 128 + (size_t)((depth + 1) * MT_PW + (depth + 5) * 6) * 2 * g.sx * sizeof(float);
}

// units of the CTA, as a cursor over (unit, plane step)
struct MtCursor {
    int unit, s, S, k0;
    __device__ void set(const Geo &g, int zruns, int u) {
        const int ntiles = g.sy / 2, nunits = ntiles * zruns;
        for (unit = u; unit < nunits; unit += gridDim.x) {
            const int run = unit / ntiles;
            const int q0 = (int)((long)run * g.nz / zruns), q1 = (int)((long)(run + 1) * g.nz / zruns);
            S = q1 - q0;
            k0 = 1 + q0;
            s = 0;
            if (S > 0) return;
        }
        S = 0;
    }
    __device__ bool valid(const Geo &g, int zruns) const { return unit < (g.sy / 2) * zruns; }
    __device__ void next(const Geo &g, int zruns) {
        if (++s >= S) set(g, zruns, unit + gridDim.x);
    }
};

__global__ void __launch_bounds__(MT_THREADS, 1) k_march_tma(MarchTmaArgs a, Geo g, MixConst mc, StepCounters *cnt) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);          // D + 1 barriers
    __shared__ int abort_flag;
    const int D = a.depth, NB = D + 1, RING = D + 5;
    const int rowp = 2 * g.sx;                                        // floats per row pair
    float *pwb = reinterpret_cast<float *>(smem_raw + 128);           // [NB][MT_PW][rowp]
    float *phb = pwb + (size_t)NB * MT_PW * rowp;                     // [RING][2][3 pairs][rowp]
    const uint32_t pair_bytes = (uint32_t)(rowp * sizeof(float));
    const size_t plane = (size_t)g.sx * g.sy;
    const int ntiles = g.sy / 2;
    auto ynb = [&](int j, int d) { return g.walls ? max(1, min(g.ny, j + d)) : wrapy(g, j + d); };
    // row pairs of the rows below / above the computed rows of tile jb
    auto pairs_of = [&](int jb, int &jlo, int &jhi) {
        const int jc0 = max(jb, 1), jc1 = min(jb + 1, g.ny);
        jlo = ynb(jc0, -1) & ~1;
        jhi = ynb(jc1, 1) & ~1;
    };
    if (threadIdx.x == 0) {
        for (int q = 0; q < NB; ++q) mbar_init(&bar[q], 1);
        mbar_init_fence();
        abort_flag = 0;
    }
    __syncthreads();
    // producer (thread 0): cursor, groups issued, Phi planes loaded
    MtCursor pc;
    unsigned pg = 0, pphi = 0;
    auto issue = [&]() {
        const int jb = 2 * (pc.unit % ntiles);
        int jlo, jhi;
        pairs_of(jb, jlo, jhi);
        uint64_t *b = &bar[pg % NB];
        const int k = pc.k0 + pc.s;
        const int nphi = pc.s == 0 ? 3 : 1;
        mbar_expect(b, pair_bytes * (uint32_t)(MT_PW + 6 * nphi));
        float *dst = pwb + (size_t)(pg % NB) * MT_PW * rowp;
        for (int arr = 0; arr < MT_PW; ++arr)
            bulk_load(dst + (size_t)arr * rowp, a.pw[arr] + (size_t)k * plane + (size_t)jb * g.sx, pair_bytes, b);
        const int rows[3] = {jlo, jb, jhi};
        for (int kk = pc.s == 0 ? k - 1 : k + 1; kk <= k + 1; ++kk) {
            const size_t zo = (size_t)wrapz(g, kk) * plane;
            float *ps = phb + (size_t)(pphi % RING) * 6 * rowp;
            for (int arr = 0; arr < 2; ++arr)
                for (int r = 0; r < 3; ++r)
                    bulk_load(ps + (size_t)(arr * 3 + r) * rowp, a.phi[arr] + zo + (size_t)rows[r] * g.sx, pair_bytes, b);
            ++pphi;
        }
        ++pg;
        pc.next(g, a.zruns);
    };
    if (threadIdx.x == 0) {
        pc.set(g, a.zruns, blockIdx.x);
        for (int q = 0; q < D && pc.valid(g, a.zruns); ++q) issue();
    }
    // consumers: cursor, step count, Phi planes consumed through this step
    MtCursor cc;
    cc.set(g, a.zruns, blockIdx.x);
    unsigned t = 0, cphi = 0;
    for (; cc.valid(g, a.zruns); cc.next(g, a.zruns), ++t) {
        if (threadIdx.x == 0 && pc.valid(g, a.zruns)) {
            fence_async_smem();
            issue();
        }
        cphi += cc.s == 0 ? 3 : 1;
        if (!mbar_wait(&bar[t % NB], (t / NB) & 1)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) {
            // let the copies already issued finish before the CTA leaves
            if (threadIdx.x == 0) {
                for (unsigned q = t; q < pg; ++q) mbar_wait(&bar[q % NB], (q / NB) & 1, 200000000LL);
                atomicAdd(&cnt->copy_timeouts, 1ULL);
            }
            return;
        }
        const int jb = 2 * (cc.unit % ntiles);
        int jlo, jhi;
        pairs_of(jb, jlo, jhi);
        const int k = cc.k0 + cc.s;
        const float *pw = pwb + (size_t)(t % NB) * MT_PW * rowp;
        const float *sm = phb + (size_t)((cphi - 3) % RING) * 6 * rowp;   // plane k - 1
        const float *s0 = phb + (size_t)((cphi - 2) % RING) * 6 * rowp;   // plane k
        const float *sp = phb + (size_t)((cphi - 1) % RING) * 6 * rowp;   // plane k + 1
        // shared-memory row (of the six of a Phi slot) of the y neighbour of row j
        auto nrow = [&](int j, int d) {
            const int jn = ynb(j, d);
            if (jn >= jb && jn < jb + 2) return 2 + jn - jb;
            if (jn >= jlo && jn < jlo + 2) return jn - jlo;
            return 4 + jn - jhi;
        };
        const bool in0 = jb >= 1, in1 = jb + 1 <= g.ny;   // the two rows (lanes) computed
        // rows outside 1..NY are evaluated on the loaded halo values and not stored
        const int j0 = in0 ? jb : jb + 1, j1 = in1 ? jb + 1 : jb;
        const int ym0 = nrow(j0, -1) * g.sx, yp0 = nrow(j0, 1) * g.sx;
        const int ym1 = nrow(j1, -1) * g.sx, yp1 = nrow(j1, 1) * g.sx;
        for (int i = 1 + (int)threadIdx.x; i <= g.nx; i += blockDim.x) {
            const int xm = wrapx(g, i - 1), xp = wrapx(g, i + 1);
            // Phi (hi, lo) of both rows at row offset ro0 / ro1 of a slot
            auto ph2 = [&](const float *sl, int o0, int o1) {
                return df2_pack(df{sl[o0], sl[o0 + 3 * rowp]}, df{sl[o1], sl[o1 + 3 * rowp]});
            };
            const int c0o = 2 * g.sx + i, c1o = 3 * g.sx + i;   // the tile rows in a slot
            const df2 c0 = ph2(s0, c0o, c1o);
            const df2 pp[3] = {ph2(s0, 2 * g.sx + xp, 3 * g.sx + xp), ph2(s0, yp0 + i, yp1 + i), ph2(sp, c0o, c1o)};
            const df2 pm[3] = {ph2(s0, 2 * g.sx + xm, 3 * g.sx + xm), ph2(s0, ym0 + i, ym1 + i), ph2(sm, c0o, c1o)};
            auto pv = [&](int arr, int r) { return pw[(size_t)arr * rowp + r * g.sx + i]; };
            df2 Fv[3];
            float2 Dv[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                Fv[q] = df2_pack(df{pv(2 * q, 0), pv(2 * q + 1, 0)}, df{pv(2 * q, 1), pv(2 * q + 1, 1)});
                Dv[q] = make_float2(pv(8 + q, 0), pv(8 + q, 1));
            }
            const df2 Pv = df2_pack(df{pv(6, 0), pv(7, 0)}, df{pv(6, 1), pv(7, 1)});
            df2 nu[3], pn;
            march_pair_math(c0, pp, pm, Fv, Dv, Pv, mc, nu, pn);
            const size_t h0 = (size_t)hix(g, i, jb, k), h1 = h0 + g.sx;
            if (in0) {
#pragma unroll
                for (int q = 0; q < 3; ++q) { a.out[2 * q][h0] = nu[q].hi.x; a.out[2 * q + 1][h0] = nu[q].lo.x; }
                a.out[6][h0] = pn.hi.x; a.out[7][h0] = pn.lo.x;
            }
            if (in1) {
#pragma unroll
                for (int q = 0; q < 3; ++q) { a.out[2 * q][h1] = nu[q].hi.y; a.out[2 * q + 1][h1] = nu[q].lo.y; }
                a.out[6][h1] = pn.hi.y; a.out[7][h1] = pn.lo.y;
            }
            if ((in0 && !isfinite(nu[0].hi.x)) || (in1 && !isfinite(nu[0].hi.y))) atomicAdd(&cnt->nan_cells, 1ULL);
        }
        // every thread is done with this step's buffers before later copies
        // may overwrite them
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Red-black SOR variant of the pressure solve (the reference's poisson,
// fenep.f90:848-905; the GPU colours by (i+j+k) parity as the FP64 step does)
// on the FP32 pressure correction: Phi (hi part) warm-started from the
// previous step, sweeps until sqrt(sum E^2 / sum R^2) < eps with the sums in
// FP64, then the zero-mean shift (fenep_2d.f90:577-579).  The reference's
// tolerance (1e-5) is far above FP32 rounding.  Halo-free: periodic wrap and
// the Neumann copy at the walls, which is what the halo pass between the
// colour sweeps of the FP64 step provides.
__global__ void k_sor_color_f(float *Phi, float *E, const float *R, Geo g, int color, float om, float bx, float by,
                              float bz, const int *flag) {
    if (flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    if (((i + j + k) & 1) != color) return;
    const int h = hix(g, i, j, k);
    const float b0 = 2.0f * (bx + by + bz);
    const int q = qix(g, i, j, k);
    const float e = bz * Phi[nbr_p(g, i, j, k, 2, -1)] + by * Phi[nbr_p(g, i, j, k, 1, -1)]
                  + bx * Phi[nbr_p(g, i, j, k, 0, -1)] - b0 * Phi[h] + bx * Phi[nbr_p(g, i, j, k, 0, 1)]
                  + by * Phi[nbr_p(g, i, j, k, 1, 1)] + bz * Phi[nbr_p(g, i, j, k, 2, 1)] - R[q];
    E[q] = e;
    Phi[h] = Phi[h] + om * e / b0;
}

// block partials of sum(a^2) (mode 0) or of the interior sum of a halo field
// (mode 1), in FP64, fixed order
__global__ void k_sum_part_f(const float *a, int n, int mode, double *part, Geo g, const int *flag) {
    if (flag && flag[0]) return;
    __shared__ double sh[256];
    double s = 0.0;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        if (mode == 0) {
            const double v = a[q];
            s += v * v;
        } else {
            const int i = 1 + (int)(q % g.nx), j = 1 + (int)((q / g.nx) % g.ny), k = 1 + (int)(q / ((long)g.nx * g.ny));
            s += a[hix(g, i, j, k)];
        }
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// mode 0: scal[slot] = sum (er0, the reference's zero guard); mode 1: the
// convergence test against scal[0] (flag[0] = 1, flag[1] = iteration);
// mode 2: scal[slot] = sum
__global__ void k_sum_final(const double *part, int nparts, double *scal, int slot, int mode, int *flag, double eps,
                            int itr) {
    if (mode == 1 && flag[0]) return;
    __shared__ double sh[256];
    double s = 0.0;
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += part[q];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scal[slot] = (mode == 0 && sh[0] == 0.0) ? 1.0e-16 : sh[0];
        if (mode == 1) {
            flag[1] = itr;
            if (sqrt(sh[0] / scal[0]) < eps) flag[0] = 1;
        }
    }
}

__global__ void k_shift_f(float *a, Geo g, const double *scal, int slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const float mean = (float)(scal[slot] / ((double)g.nx * g.ny * g.nz));
    a[hix(g, i, j, k)] -= mean;
}

template <typename A, typename B>
__global__ void k_convert(const A *a, B *b, int n) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) b[q] = B(a[q]);
}
// C component-fastest (FP64) <-> one FP32 array per component, ncomp <= 6;
// all loads of a cell before its stores
__global__ void k_aos_to_soa_f(const double *__restrict__ aos, float *__restrict__ soa, int ncomp, int cs) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cs) return;
    float v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m)
        if (m < ncomp) v[m] = (float)aos[(size_t)ncomp * h + m];
#pragma unroll
    for (int m = 0; m < 6; ++m)
        if (m < ncomp) soa[(size_t)m * cs + h] = v[m];
}
__global__ void k_soa_to_aos_f(const float *__restrict__ soa, double *__restrict__ aos, int ncomp, int cs) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cs) return;
    double v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m)
        if (m < ncomp) v[m] = (double)soa[(size_t)m * cs + h];
#pragma unroll
    for (int m = 0; m < 6; ++m)
        if (m < ncomp) aos[(size_t)ncomp * h + m] = v[m];
}

inline dim3 cell_grid_m(const Geo &g, dim3 blk) {
    return dim3((g.nx + blk.x - 1) / blk.x, (g.ny + blk.y - 1) / blk.y, g.nz);
}

// ---------------------------------------------------------------------------
// FP32 spectral solves.  src (interior, FP32 or FP64) -> dst (FP64 halo
// interior; dst = base + result when base is given).
template <typename TS>
cudaError_t solve_periodic_mp(Dev &d, const TS *src, XOutF out, double lhs0, double lhs1, cudaStream_t s) {
    const Geo &g = d.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxh = nx / 2 + 1;
    const int tpp = std::max(nx / 2, 1), ppc = std::max(1, 256 / tpp);
    const size_t smx = (size_t)ppc * 2 * nx * sizeof(Cx<float>);
    {
        int npp = ny / 2, total = npp * nz;
        k_fft_x_fwd<float, TS><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(src, d.Hf, nx, ny, 1, ny, npp, nz, d.twxf_r, d.twxf_i); count_launch();
    }
    DivideSpec none{};
    const int txy = std::max(1, std::min(32, 4096 / ny));
    const size_t smy = (size_t)2 * ny * txy * sizeof(Cx<float>);
    if (nz == 1) {
        // 2D: the y lines transform, divide and transform back in one pass
        DivideSpec dv{d.kx2, d.ky2, d.kz2, lhs0, lhs1, (double)nx * ny * nz, 0};
        k_fft_lines<float><<<dim3((nxh + txy - 1) / txy, nz), 256, smy, s>>>(d.Hf, ny, nxh, nxh, nxh * ny, txy, d.twyf_r, d.twyf_i, -1, 1, dv); count_launch();
        int npp = ny / 2, total = npp * nz;
        k_fft_x_inv<float, XOutF><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(d.Hf, out, nx, ny, npp, nz, 1, g.sx, g.sy, d.twxf_r, d.twxf_i); count_launch();
        return cudaGetLastError();
    }
    k_fft_lines<float><<<dim3((nxh + txy - 1) / txy, nz), 256, smy, s>>>(d.Hf, ny, nxh, nxh, nxh * ny, txy, d.twyf_r, d.twyf_i, -1, 0, none); count_launch();
    {
        DivideSpec dv{d.kx2, d.ky2, d.kz2, lhs0, lhs1, (double)nx * ny * nz, 1};
        const int txz = std::max(1, std::min(32, 4096 / nz));
        const size_t smz = (size_t)2 * nz * txz * sizeof(Cx<float>);
        k_fft_lines<float><<<dim3((nxh + txz - 1) / txz, ny), 256, smz, s>>>(d.Hf, nz, nxh * ny, nxh, nxh, txz, d.twzf_r, d.twzf_i, -1, 1, dv); count_launch();
    }
    k_fft_lines<float><<<dim3((nxh + txy - 1) / txy, nz), 256, smy, s>>>(d.Hf, ny, nxh, nxh, nxh * ny, txy, d.twyf_r, d.twyf_i, +1, 0, none); count_launch();
    {
        int npp = ny / 2, total = npp * nz;
        k_fft_x_inv<float, XOutF><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(d.Hf, out, nx, ny, npp, nz, 1, g.sx, g.sy, d.twxf_r, d.twxf_i); count_launch();
    }
    return cudaGetLastError();
}

template <typename TS>
cudaError_t solve_walls_mp(Dev &d, const TS *src, XOutF out, int sys, cudaStream_t s) {
    const Geo &g = d.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxh = nx / 2 + 1, n = ny + 2;
    const int tpp = std::max(nx / 2, 1), ppc = std::max(1, 256 / tpp);
    const size_t smx = (size_t)ppc * 2 * nx * sizeof(Cx<float>);
    {
        int npp = ny / 2, total = npp * nz;
        k_fft_x_fwd<float, TS><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(src, d.Hf, nx, ny, 1, ny, npp, nz, d.twxf_r, d.twxf_i); count_launch();
    }
    DivideSpec none{};
    const int txz = std::max(1, std::min(32, 4096 / nz));
    const size_t smz = (size_t)2 * nz * txz * sizeof(Cx<float>);
    if (nz > 1) {
        k_fft_lines<float><<<dim3((nxh + txz - 1) / txz, ny), 256, smz, s>>>(d.Hf, nz, nxh * ny, nxh, nxh, txz, d.twzf_r, d.twzf_i, -1, 0, none); count_launch();
    }
    {
        WallSpec w{d.kx2, d.kz2, d.ph.dt, d.ph.beta, d.ph.re, g.dy, (double)nx * nz, 0.0, sys};
        const int tx = 32;
        const size_t sm = (size_t)n * tx * (sizeof(Cx<float>) + sizeof(float));
        k_wall_tdma<float><<<dim3((nxh + tx - 1) / tx, nz), 128, sm, s>>>(d.Hf, d.H2f, ny, nxh, tx, w); count_launch();
    }
    if (nz > 1) {
        k_fft_lines<float><<<dim3((nxh + txz - 1) / txz, n), 256, smz, s>>>(d.H2f, nz, nxh * n, nxh, nxh, txz, d.twzf_r, d.twzf_i, +1, 0, none); count_launch();
    }
    {
        int npp = n / 2, total = npp * nz;
        k_fft_x_inv<float, XOutF><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(d.H2f, out, nx, n, npp, nz, 0, g.sx, g.sy, d.twxf_r, d.twxf_i); count_launch();
    }
    return cudaGetLastError();
}


// Fused path: transposing x pass, one CTA per kx for the (z, y) plane,
// transposing inverse x pass.
inline int x_rows_per_block(int nx) { return 2 * std::max(1, std::min(8, 1024 / std::max(nx / 2, 1))); }
inline size_t x_smem(int nx, int rb) { return (size_t)(rb / 2) * 2 * nx * sizeof(float2) + (size_t)(nx / 2 + 1) * (rb + 1) * sizeof(float2); }
inline int ilog2(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

// warp-per-row-pair x passes for NX = 32 .. 512; false when NX has no instance
template <typename TS>
bool xfwd_warp(const Dev &d, const TS *src, float2 *S, int ny, int lj, int joff, cudaStream_t s) {
    const Geo &g = d.g;
    const unsigned grid = (unsigned)(((ny + XW_RB - 1) / XW_RB) * g.nz);
    const size_t sm = xw_smem(g.nx, XW_RB);
    const int thr = 32 * XW_WARPS;
    switch (g.nx) {
    case 32: k_xfwd_w<1, TS><<<grid, thr, sm, s>>>(src, S, ny, g.nz, lj, joff, d.twx2); break;
    case 64: k_xfwd_w<2, TS><<<grid, thr, sm, s>>>(src, S, ny, g.nz, lj, joff, d.twx2); break;
    case 128: k_xfwd_w<4, TS><<<grid, thr, sm, s>>>(src, S, ny, g.nz, lj, joff, d.twx2); break;
    case 256: k_xfwd_w<8, TS><<<grid, thr, sm, s>>>(src, S, ny, g.nz, lj, joff, d.twx2); break;
    case 512: k_xfwd_w<16, TS><<<grid, thr, sm, s>>>(src, S, ny, g.nz, lj, joff, d.twx2); break;
    default: return false;
    }
    count_launch();
    return true;
}

bool xinv_warp(const Dev &d, const float2 *S, XOutF out, int nrow, int jlo, int lj, int joff2, cudaStream_t s) {
    const Geo &g = d.g;
    const unsigned grid = (unsigned)(((nrow + XW_RB - 1) / XW_RB) * g.nz);
    const size_t sm = xw_smem(g.nx, XW_RB);
    const int thr = 32 * XW_WARPS;
    switch (g.nx) {
    case 32: k_xinv_w<1, XOutF><<<grid, thr, sm, s>>>(S, out, nrow, jlo, g.nz, lj, joff2, g.sx, g.sy, d.twx2); break;
    case 64: k_xinv_w<2, XOutF><<<grid, thr, sm, s>>>(S, out, nrow, jlo, g.nz, lj, joff2, g.sx, g.sy, d.twx2); break;
    case 128: k_xinv_w<4, XOutF><<<grid, thr, sm, s>>>(S, out, nrow, jlo, g.nz, lj, joff2, g.sx, g.sy, d.twx2); break;
    case 256: k_xinv_w<8, XOutF><<<grid, thr, sm, s>>>(S, out, nrow, jlo, g.nz, lj, joff2, g.sx, g.sy, d.twx2); break;
    case 512: k_xinv_w<16, XOutF><<<grid, thr, sm, s>>>(S, out, nrow, jlo, g.nz, lj, joff2, g.sx, g.sy, d.twx2); break;
    default: return false;
    }
    count_launch();
    return true;
}

template <typename TS>
cudaError_t solve_periodic_fused(Dev &d, const TS *src, XOutF out, float lhs0, float lhs1, cudaStream_t s,
                                 float *spec = nullptr) {
    const Geo &g = d.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxh = nx / 2 + 1;
    float2 *S = reinterpret_cast<float2 *>(spec ? spec : d.Hf);
    const int rb = x_rows_per_block(nx);
    const int thr = (rb / 2) * (nx / 2);
    const size_t smx = x_smem(nx, rb);
    const int bpp = (ny + rb - 1) / rb;
    if (!xfwd_warp<TS>(d, src, S, ny, ny, -1, s)) {
        k_xfwd_t<TS><<<bpp * nz, thr, smx, s>>>(src, S, nx, ny, nz, rb, ny, -1, d.twxf_r, d.twxf_i); count_launch();
    }
    PlaneSpec ps{};
    ps.kx2 = d.kx2f; ps.ky2 = d.ky2f; ps.kz2 = d.kz2f;
    ps.lhs0 = lhs0; ps.lhs1 = lhs1; ps.inv_ntot = (float)(1.0 / ((double)nx * ny * nz));
    k_plane_periodic<<<nxh, 1024, (size_t)8 * (ny + 1) * nz, s>>>(S, ny, nz, ilog2(ny), ilog2(nz), d.twyf_r, d.twyf_i,
                                                                 d.twzf_r, d.twzf_i, ps); count_launch();
    if (!xinv_warp(d, S, out, ny, 1, ny, -1, s)) {
        k_xinv_t<XOutF><<<bpp * nz, thr, smx, s>>>(S, out, nx, ny, 1, nz, rb, ny, -1, g.sx, g.sy, d.twxf_r, d.twxf_i); count_launch();
    }
    return cudaGetLastError();
}

template <typename TS>
cudaError_t solve_walls_fused(Dev &d, const TS *src, XOutF out, int sys, cudaStream_t s, float *spec = nullptr) {
    const Geo &g = d.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxh = nx / 2 + 1, lj = ny + 2;
    float2 *S = reinterpret_cast<float2 *>(spec ? spec : d.Hf);
    const int rb = x_rows_per_block(nx);
    const int thr = (rb / 2) * (nx / 2);
    const size_t smx = x_smem(nx, rb);
    if (!xfwd_warp<TS>(d, src, S, ny, lj, 0, s)) {
        k_xfwd_t<TS><<<((ny + rb - 1) / rb) * nz, thr, smx, s>>>(src, S, nx, ny, nz, rb, lj, 0, d.twxf_r, d.twxf_i); count_launch();
    }
    PlaneSpec ps{};
    ps.kx2 = d.kx2f; ps.ky2 = d.ky2f; ps.kz2 = d.kz2f;
    const double kap = d.ph.dt * d.ph.beta / d.ph.re / 2.0, idy2 = 1.0 / (g.dy * g.dy);
    ps.sys = sys;
    ps.nxz_inv = (float)(1.0 / ((double)nx * nz));
    if (sys == SYS_P) { ps.ai_base = (float)(2.0 * idy2); ps.bc = (float)idy2; ps.kap = -1.0f; }
    else { ps.ai_base = (float)(1.0 + kap * 2.0 * idy2); ps.bc = (float)(-kap * idy2); ps.kap = (float)kap; }
    const size_t smp = (size_t)12 * (lj | 1) * nz;
    if (d.plane_cl > 0 && d.wtR[0]) {
        const int t = sys == SYS_P ? 2 : (sys == SYS_V ? 1 : 0);
        const float b_first = sys == SYS_P ? -1.0f : (sys == SYS_V ? 0.0f : 1.0f);
        WallTables wt{d.wtR[t], ps.bc, sys == SYS_P ? -1.0f : 1.0f, b_first, ps.nxz_inv, sys, d.plane_wl};
        const int cl = d.plane_cl;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)(nxh * cl));
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = wall_plane_smem(d.plane_wl, nz);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cl;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaError_t e;
        if (nz == 32) e = cudaLaunchKernelEx(&cfg, k_plane_walls_c<1>, S, ny, cl, (const float2 *)d.twz2, wt);
        else if (nz == 64) e = cudaLaunchKernelEx(&cfg, k_plane_walls_c<2>, S, ny, cl, (const float2 *)d.twz2, wt);
        else if (nz == 128) e = cudaLaunchKernelEx(&cfg, k_plane_walls_c<4>, S, ny, cl, (const float2 *)d.twz2, wt);
        else e = cudaLaunchKernelEx(&cfg, k_plane_walls_c<8>, S, ny, cl, (const float2 *)d.twz2, wt);
        count_launch();
        if (e) return e;
    } else {
        k_plane_walls<<<nxh, 1024, smp, s>>>(S, ny, nz, ilog2(nz), d.twzf_r, d.twzf_i, ps); count_launch();
    }
    if (!xinv_warp(d, S, out, lj, 0, lj, 0, s)) {
        k_xinv_t<XOutF><<<((lj + rb - 1) / rb) * nz, thr, smx, s>>>(S, out, nx, lj, 0, nz, rb, lj, 0, g.sx, g.sy,
                                                                  d.twxf_r, d.twxf_i); count_launch();
    }
    return cudaGetLastError();
}

cudaError_t solve_periodic_f(Dev &d, const float *src, XOutF out, double lhs0, double lhs1, cudaStream_t s) {
    if (d.fused_planes) return solve_periodic_fused<float>(d, src, out, (float)lhs0, (float)lhs1, s);
    return solve_periodic_mp<float>(d, src, out, lhs0, lhs1, s);
}

cudaError_t solve_walls_f(Dev &d, const float *src, XOutF out, int sys, cudaStream_t s) {
    if (d.fused_planes) return solve_walls_fused<float>(d, src, out, sys, s);
    return solve_walls_mp<float>(d, src, out, sys, s);
}

cudaError_t sor_solve_m(Dev &d, const StepOpts &o, int *iters, cudaStream_t s) {
    const Geo &g = d.g;
    const dim3 blk(32, 8), grd = cell_grid_m(g, blk);
    const int nb = std::min(1024, (d.ni + 255) / 256);
    F8_CUDA_RET(cudaMemsetAsync(d.flag, 0, 2 * sizeof(int), s));
    F8_CUDA_RET(cudaMemsetAsync(d.Phil, 0, (size_t)d.cs * sizeof(float), s));
    k_sum_part_f<<<nb, 256, 0, s>>>(d.Rhf, d.ni, 0, d.red, g, nullptr); count_launch();
    k_sum_final<<<1, 256, 0, s>>>(d.red, nb, d.scal, 0, 0, d.flag, 0.0, 0); count_launch();
    const float bx = (float)(1.0 / (g.dx * g.dx)), by = (float)(1.0 / (g.dy * g.dy)), bz = (float)(1.0 / (g.dz * g.dz));
    int done = 0, it_host[2] = {0, 0};
    const int chunk = 25;
    for (int it0 = 1; it0 <= o.sor_itrmax && !done; it0 += chunk) {
        const int last = std::min(o.sor_itrmax, it0 + chunk - 1);
        for (int it = it0; it <= last; ++it) {
            for (int color = 0; color < 2; ++color) {
                k_sor_color_f<<<grd, blk, 0, s>>>(d.Phif, d.Rdf, d.Rhf, g, color, (float)o.sor_omega, bx, by, bz,
                                                  d.flag); count_launch();
            }
            k_sum_part_f<<<nb, 256, 0, s>>>(d.Rdf, d.ni, 0, d.red, g, d.flag); count_launch();
            k_sum_final<<<1, 256, 0, s>>>(d.red, nb, d.scal, 1, 1, d.flag, o.sor_eps, it); count_launch();
        }
        F8_CUDA_RET(cudaMemcpyAsync(it_host, d.flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        F8_CUDA_RET(cudaStreamSynchronize(s));
        done = it_host[0];
    }
    *iters = done ? it_host[1] : o.sor_itrmax + 1;
    k_sum_part_f<<<nb, 256, 0, s>>>(d.Phif, d.ni, 1, d.red, g, nullptr); count_launch();
    k_sum_final<<<1, 256, 0, s>>>(d.red, nb, d.scal, 2, 2, d.flag, 0.0, 0); count_launch();
    k_shift_f<<<grd, blk, 0, s>>>(d.Phif, g, d.scal, 2); count_launch();
    return cudaGetLastError();
}

}  // namespace

// FP32 solves of the mixed step for the discrete adjoint (f8_adjoint_mixed.cu):
// the periodic spectral solve with LHS = lhs0 + lhs1 k~^2, or the wall system
// sys (0 U/W Helmholtz, 1 V Helmholtz, 2 pressure).  mode 0: dst = v at the
// interior cells (and the wall ghost rows); mode 2: (dst, lo) = dst + v as an
// exact two-sum (the correction of a double-float pair).
cudaError_t mixed_solve_periodic(Dev &d, const float *src, float *dst, float *lo, int mode, double lhs0, double lhs1,
                                 cudaStream_t s) {
    return solve_periodic_f(d, src, XOutF{dst, lo, mode}, lhs0, lhs1, s);
}

cudaError_t mixed_solve_walls(Dev &d, const float *src, float *dst, float *lo, int mode, int sys, cudaStream_t s) {
    return solve_walls_f(d, src, XOutF{dst, lo, mode}, sys, s);
}

// the three Helmholtz solves of one step (dst[c] = v of component c, mode 0),
// the V and W solves forked onto the side streams with their own spectra on
// the fused spectral path, as in the forward step
cudaError_t mixed_helmholtz3(Dev &d, const float *const src[3], float *const dst[3], cudaStream_t s) {
    const Geo &g = d.g;
    const double lhs1 = d.ph.dt * d.ph.beta / d.ph.re / 2.0;
    const bool branches = d.fused_planes && d.aux[0] && d.aux[1];
    if (branches) {
        F8_CUDA_RET(cudaEventRecord(d.ev_fork, s));
        for (int b = 0; b < 2; ++b) F8_CUDA_RET(cudaStreamWaitEvent(d.aux[b], d.ev_fork, 0));
    }
    for (int c = 0; c < 3; ++c) {
        const XOutF out{dst[c], nullptr, 0};
        const int sys = c == 1 ? SYS_V : SYS_U;
        cudaError_t e;
        if (branches) {
            cudaStream_t sc = c == 0 ? s : d.aux[c - 1];
            float *spec = c == 0 ? d.Hf : d.HfB[c - 1];
            if (!g.walls) e = solve_periodic_fused<float>(d, src[c], out, 1.0f, (float)lhs1, sc, spec);
            else e = solve_walls_fused<float>(d, src[c], out, sys, sc, spec);
        } else if (!g.walls) {
            e = solve_periodic_f(d, src[c], out, 1.0, lhs1, s);
        } else {
            e = solve_walls_f(d, src[c], out, sys, s);
        }
        if (e) return e;
    }
    if (branches) {
        for (int b = 0; b < 2; ++b) {
            F8_CUDA_RET(cudaEventRecord(d.ev_join[b], d.aux[b]));
            F8_CUDA_RET(cudaStreamWaitEvent(s, d.ev_join[b], 0));
        }
    }
    return cudaGetLastError();
}

// defect rd = (rh + rl) - L_h phi of an FP32 pressure-type field in df64, the
// operator of the mixed step's Poisson solve (interior arrays rh, rl, rd)
cudaError_t mixed_defect(Dev &d, const float *phi, const float *rh, const float *rl, float *rd, cudaStream_t s) {
    const Geo &g = d.g;
    const dim3 pblk(32, 8), pgrid((g.nx + pblk.x - 1) / pblk.x, (g.ny + pblk.y - 1) / pblk.y, (g.nz + 1) / 2);
    k_defect_df<<<pgrid, pblk, 0, s>>>(phi, rh, rl, rd, g, make_const(g, d.ph)); count_launch();
    return cudaGetLastError();
}

// The staged projection (k_march_tma) needs row pairs that are contiguous,
// 16-byte aligned blocks: NX a multiple of 4, NY even, 3D; and its shared
// memory for at least one step in flight within the opt-in limit (the
// deepest of D = 1 .. 4 that fits is taken).  The z runs per y tile are
// chosen so that the units (tile, run) spread evenly over the persistent CTAs
// (one per SM), each run at least D + 1 planes.
//
// Measured on the 256 x 128 x 128 channel (GB300): 134 us against the
// direct-load kernel's 82 us.  The df64 arithmetic costs about 2.6
// instructions per byte, and the staged kernel's 8 warps per SM (one step of
// 256 cell pairs per CTA at a time, the shared memory holding D + 1 steps)
// issue too slowly to keep up with the copies, where the direct-load kernel
// keeps 32 warps per SM.  The direct-load kernel is therefore the default;
// F8_STAGED_PROJECTION=1 in the environment, read when a context is
// created, selects the staged one.
cudaError_t setup_staged_projection(Dev &d) {
    const Geo &g = d.g;
    d.march_runs = 0;
    d.march_ctas = 0;
    d.march_depth = 0;
    const char *env = std::getenv("F8_STAGED_PROJECTION");
    if (!env || env[0] != '1') return cudaSuccess;
    if (g.dim != 3 || g.nx % 4 != 0 || g.ny % 2 != 0) return cudaSuccess;
    int dev = 0, optin = 0;
    F8_CUDA_RET(cudaGetDevice(&dev));
    F8_CUDA_RET(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int depth = 0;
    for (int dd = MT_MAXD; dd >= 1 && !depth; --dd)
        if (march_tma_smem(g, dd) <= (size_t)optin) depth = dd;
    if (!depth || g.nz < depth + 1) return cudaSuccess;
    F8_CUDA_RET(cudaFuncSetAttribute(k_march_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)march_tma_smem(g, depth)));
    const int nsm = device_sm_count(), ntiles = g.sy / 2;
    int best = 1;
    double bestc = 1e30;
    for (int runs = 1; runs <= g.nz / (depth + 1); ++runs) {
        const int units = ntiles * runs;
        const int ctas = std::min(nsm, units);
        // planes on the busiest CTA (the copies stream across its units)
        const double c = (double)((units + ctas - 1) / ctas) * ((g.nz + runs - 1) / runs) + 2.0 * runs / g.nz;
        if (c < bestc) { bestc = c; best = runs; }
    }
    d.march_runs = best;
    d.march_ctas = std::min(nsm, ntiles * best);
    d.march_depth = depth;
    return cudaSuccess;
}

cudaError_t init_kernels_mixed() {
    const int big = 200 * 1024;
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_lines<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_wall_tdma<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_x_fwd<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_x_inv<float, XOutF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    int dev = 0, optin = 0;
    F8_CUDA_RET(cudaGetDevice(&dev));
    F8_CUDA_RET(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_walls, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_periodic, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_walls_c<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_walls_c<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_walls_c<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    F8_CUDA_RET(cudaFuncSetAttribute(k_plane_walls_c<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
#define F8_XW_ATTR(E)                                                                                           \
    F8_CUDA_RET(cudaFuncSetAttribute(k_xfwd_w<E, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));   \
    F8_CUDA_RET(cudaFuncSetAttribute(k_xinv_w<E, XOutF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_XW_ATTR(1) F8_XW_ATTR(2) F8_XW_ATTR(4) F8_XW_ATTR(8) F8_XW_ATTR(16)
#undef F8_XW_ATTR
    F8_CUDA_RET(cudaFuncSetAttribute(k_xfwd_t<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_xinv_t<XOutF>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    return cudaSuccess;
}

// FP64 -> FP32; with `varies`, also set *varies = 1 when some a[q] != a[0]
__global__ void k_convert_check(const double *__restrict__ a, float *__restrict__ b, int n, int *varies) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double v = a[q];
    b[q] = (float)v;
    if (v != a[0]) *varies = 1;
}

cudaError_t d2f(const double *a, float *b, int n, cudaStream_t s, int *varies) {
    if (varies) k_convert_check<<<(n + 255) / 256, 256, 0, s>>>(a, b, n, varies);
    else k_convert<double, float><<<(n + 255) / 256, 256, 0, s>>>(a, b, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t f2d(const float *a, double *b, int n, cudaStream_t s) {
    k_convert<float, double><<<(n + 255) / 256, 256, 0, s>>>(a, b, n); count_launch();
    return cudaGetLastError();
}
cudaError_t aos_to_soa_f(const double *aos, float *soa, int ncomp, int cs, cudaStream_t s) {
    k_aos_to_soa_f<<<(cs + 255) / 256, 256, 0, s>>>(aos, soa, ncomp, cs); count_launch();
    return cudaGetLastError();
}
cudaError_t soa_to_aos_f(const float *soa, double *aos, int ncomp, int cs, cudaStream_t s) {
    k_soa_to_aos_f<<<(cs + 255) / 256, 256, 0, s>>>(soa, aos, ncomp, cs); count_launch();
    return cudaGetLastError();
}

namespace {

BcSet state_bc_set(const Dev &d) {
    BcSet b{};
    b.hi[0] = d.Uf; b.lo[0] = d.Ul; b.kind[0] = BC_U;
    b.hi[1] = d.Vf; b.lo[1] = d.Vl; b.kind[1] = BC_V;
    b.hi[2] = d.Wf; b.lo[2] = d.Wl; b.kind[2] = BC_W;
    b.hi[3] = d.Pf; b.lo[3] = d.Pl; b.kind[3] = BC_P;
    b.n = 4;
    b.uw2 = df_from_d(2.0 * d.g.uwall);
    return b;
}

cudaError_t launch_bc_set(const BcSet &b, const Geo &g, cudaStream_t s) {
    const long n = halo_count(g) + (g.walls ? (long)g.nx * g.nz : 0);
    k_bc_set<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, g); count_launch();
    return cudaGetLastError();
}

__global__ void k_count_nonfinite_f(const float *a, int n, unsigned long long *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const bool bad = q < n && !isfinite(a[q]);
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(out, (unsigned long long)__popc(m));
}

}  // namespace

// the loaded FP64 state (halo values applied) -> df64 pairs, f(C)
cudaError_t bc_all_state_mixed(Dev &d, cudaStream_t s) {
    F8_CUDA_RET(bc_field(d.U, d.g, BC_U, s));
    F8_CUDA_RET(bc_field(d.V, d.g, BC_V, s));
    F8_CUDA_RET(bc_field(d.W, d.g, BC_W, s));
    F8_CUDA_RET(bc_field(d.P, d.g, BC_P, s));
    long n = halo_count(d.g);
    const unsigned nb = (unsigned)((n + 255) / 256), cb = (unsigned)((d.cs + 255) / 256);
    if (d.g.dim == 3) {
        k_bc_c_pet_f<6><<<nb, 256, 0, s>>>(d.Cf, d.fpetf, d.g, d.cs, d.ph.lp2); count_launch();
        k_pet_all_f<6><<<cb, 256, 0, s>>>(d.Cf, d.fpetf, d.cs, d.ph.lp2); count_launch();
    } else {
        k_bc_c_pet_f<3><<<nb, 256, 0, s>>>(d.Cf, d.fpetf, d.g, d.cs, d.ph.lp2); count_launch();
        k_pet_all_f<3><<<cb, 256, 0, s>>>(d.Cf, d.fpetf, d.cs, d.ph.lp2); count_launch();
    }
    const double *src[5] = {d.U, d.V, d.W, d.P, d.Phi};
    float *hi[5] = {d.Uf, d.Vf, d.Wf, d.Pf, d.Phif}, *lo[5] = {d.Ul, d.Vl, d.Wl, d.Pl, d.Phil};
    for (int q = 0; q < 5; ++q) {
        k_split_df<<<(d.cs + 255) / 256, 256, 0, s>>>(src[q], hi[q], lo[q], d.cs); count_launch();
    }
    return cudaGetLastError();
}

// df64 state -> the FP64 fields U, V, W, P, Phi (for store and diagnostics)
cudaError_t mixed_state_to_fp64(Dev &d, cudaStream_t s) {
    BcSet bphi{};   // Phi carries no halo during the step
    bphi.hi[0] = d.Phif; bphi.lo[0] = d.Phil; bphi.kind[0] = BC_P; bphi.n = 1;
    F8_CUDA_RET(launch_bc_set(bphi, d.g, s));
    double *dst[5] = {d.U, d.V, d.W, d.P, d.Phi};
    const float *hi[5] = {d.Uf, d.Vf, d.Wf, d.Pf, d.Phif}, *lo[5] = {d.Ul, d.Vl, d.Wl, d.Pl, d.Phil};
    for (int q = 0; q < 5; ++q) {
        k_join_df<<<(d.cs + 255) / 256, 256, 0, s>>>(hi[q], lo[q], dst[q], d.cs); count_launch();
    }
    return cudaGetLastError();
}

cudaError_t count_nonfinite_f(const float *a, int n, unsigned long long *out, cudaStream_t s) {
    k_count_nonfinite_f<<<(n + 255) / 256, 256, 0, s>>>(a, n, out); count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Tape of the discrete adjoint (MixTape): halo fields over the whole halo box
// with the values the forward kernels read at each position.

// Ua = U^n + dt R with the boundary values of ua_at (the IBM's explicit velocity)
__global__ void k_tape_ua(const float *__restrict__ Uh, const float *__restrict__ Ul, const float *__restrict__ Vh,
                          const float *__restrict__ Vl, const float *__restrict__ Wh, const float *__restrict__ Wl,
                          const float *__restrict__ Qu, const float *__restrict__ Qv, const float *__restrict__ Qw,
                          float *__restrict__ ou, float *__restrict__ ov, float *__restrict__ ow,
                          float *__restrict__ tu, float *__restrict__ tv, float *__restrict__ tw, Geo g, df uw2) {
    const int cs = g.sx * g.sy * g.sz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const df a = ua_at(g, Uh, Ul, Qu, 0, i, j, k, uw2);
    const df b = ua_at(g, Vh, Vl, Qv, 1, i, j, k, uw2);
    const df c = ua_at(g, Wh, Wl, Qw, 2, i, j, k, uw2);
    ou[t] = a.hi + a.lo;
    ov[t] = b.hi + b.lo;
    ow[t] = c.hi + c.lo;
    // the velocity of the start of the step (high parts; unchanged until the
    // projection)
    tu[t] = Uh[t];
    tv[t] = Vh[t];
    tw[t] = Wh[t];
}

// U* = U^n + dU: the increments have no halo pass; their readers wrap x and z
// (and y when periodic), and the wall solves write the ghost rows
struct TapeUp {
    const float *U[3], *D[3];
    float *out[3];
};
// the three Helmholtz solutions U^n + dU (blockIdx.y: component)
__global__ void k_tape_up(TapeUp a, Geo g) {
    const int cs = g.sx * g.sy * g.sz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cs) return;
    // the component's pointers by selects (an index into the parameter
    // arrays would copy them to local memory)
    const int c = blockIdx.y;
    const float *U = c == 0 ? a.U[0] : (c == 1 ? a.U[1] : a.U[2]);
    const float *D = c == 0 ? a.D[0] : (c == 1 ? a.D[1] : a.D[2]);
    float *out = c == 0 ? a.out[0] : (c == 1 ? a.out[1] : a.out[2]);
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const int jj = g.walls ? j : wrapy(g, j);
    out[t] = U[t] + D[hix(g, wrapx(g, i), jj, wrapz(g, k))];
}

// Phi (hi part) with the periodic wrap and the Neumann copy at the walls
__global__ void k_tape_phi(const float *__restrict__ Phi, float *__restrict__ out, Geo g) {
    const int cs = g.sx * g.sy * g.sz;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const int jj = g.walls ? max(1, min(g.ny, j)) : wrapy(g, j);
    out[t] = Phi[hix(g, wrapx(g, i), jj, wrapz(g, k))];
}

cudaError_t step_mixed(Dev &d, const StepOpts &o, double *drag_out_dev, int *sor_iters, cudaStream_t s) {
    const Geo &g = d.g;
    cudaError_t e;
    const MixConst mc = make_const(g, d.ph);
    auto mark = [&](int q) { if (o.ev) cudaEventRecord(o.ev[q], s); };
    // events bracketing one kernel launch (enum f8_kernel), on its stream
    auto kmark = [&](int kq, int edge) { if (o.kev) cudaEventRecord(o.kev[2 * kq + edge], s); };
    const DfF U{d.Uf, d.Ul}, V{d.Vf, d.Vl}, W{d.Wf, d.Wl}, P{d.Pf, d.Pl}, Phi{d.Phif, d.Phil};
    const MixTape *tp = o.tape;
    const size_t hbf = (size_t)d.cs * sizeof(float);
    const unsigned tnb = (unsigned)((d.cs + 255) / 256);
    if (tp && o.polymer) F8_CUDA_RET(cudaMemcpyAsync(tp->C, d.Cf, 6 * hbf, cudaMemcpyDeviceToDevice, s));
    mark(0);
    // wall channel: the ghost rows' codes and update run on a side stream
    // beside the interior kernels (they read the state and the interior codes
    // of rows 1 and NY, and write only ghost-row cells)
    const bool d3 = g.dim == 3;
    const bool gbranch = o.polymer && g.walls && d.aux[0] && d3;
    const dim3 gg((g.nx + 127) / 128, 2, g.nz);
    cudaStream_t sg = gbranch ? d.aux[0] : s;
    if (o.polymer && !d3) {
        // 2D (fenep_2d.f90:138-393): codes and update over the rows of the
        // update (with walls the ghost rows too), then the C halo
        const dim3 blk(32, 4), grd((g.nx + blk.x - 1) / blk.x, (prows(g) + blk.y - 1) / blk.y, 1);
        kmark(F8_KERNEL_CODES, 0);
        k_codes2_f<<<grd, blk, 0, s>>>(d.Cf, d.codes, d.codes_g, g, d.cs); count_launch();
        kmark(F8_KERNEL_CODES, 1);
        mark(1);
        kmark(F8_KERNEL_UPDATE, 0);
        k_update2_f<<<grd, blk, 0, s>>>(d.Cf, d.Cnf, d.fpetf, d.codes, d.codes_g, d.Uf, d.Vf, g, d.ph, mc, d.cs,
                                        d.cnt); count_launch();
        kmark(F8_KERNEL_UPDATE, 1);
        std::swap(d.Cf, d.Cnf);
        const long n = halo_count(g);
        if (g.walls) { k_bc_c_pet_xz_f<3><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch(); }
        else { k_bc_c_pet_f<3><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch(); }
        if ((e = cudaGetLastError())) return e;
    } else if (o.polymer) {
        dim3 blk(32, 4);
        if (g.walls) {
            if (gbranch) {
                F8_CUDA_RET(cudaEventRecord(d.ev_g[0], s));
                F8_CUDA_RET(cudaStreamWaitEvent(sg, d.ev_g[0], 0));
            }
            k_codes_ghost3_f<<<gg, 128, 0, sg>>>(d.Cf, d.codes_g, g, d.cs); count_launch();
        }
        kmark(F8_KERNEL_CODES, 0);
        k_codes3_f<<<cell_grid_m(g, blk), blk, 0, s>>>(d.Cf, d.codes, g, d.cs, d.fixcnt); count_launch();
        kmark(F8_KERNEL_CODES, 1);
        mark(1);
        if (g.walls) {
            if (gbranch) {
                F8_CUDA_RET(cudaEventRecord(d.ev_g[1], s));
                F8_CUDA_RET(cudaStreamWaitEvent(sg, d.ev_g[1], 0));
            }
            k_update_ghost3_f<<<gg, 128, 0, sg>>>(d.Cf, d.Cnf, d.fpetf, d.codes, d.codes_g, d.Uf, d.Vf, d.Wf, g, d.ph,
                                                  mc, d.cs, d.cnt); count_launch();
            if (gbranch) F8_CUDA_RET(cudaEventRecord(d.ev_g[2], sg));
        }
        kmark(F8_KERNEL_UPDATE, 0);
        k_update3_f<<<cell_grid_m(g, blk), blk, 0, s>>>(d.Cf, d.Cnf, d.fpetf, d.codes, d.Uf, d.Vf, d.Wf, g, d.ph, mc,
                                                        d.cs, d.fixlist, d.fixcnt, d.cnt); count_launch();
        kmark(F8_KERNEL_UPDATE, 1);
        k_newton_fix_f<<<2 * device_sm_count(), 128, 0, s>>>(d.Cf, d.Cnf, d.fpetf, d.Uf, d.Vf, d.Wf, g, d.ph, mc, d.cs, d.fixlist,
                                               d.fixcnt, d.cnt); count_launch();
        long n = halo_count(g);
        if (g.walls) {
            if (gbranch) F8_CUDA_RET(cudaStreamWaitEvent(s, d.ev_g[2], 0));
            std::swap(d.Cf, d.Cnf);
            k_bc_c_pet_xz_f<6><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch();
        } else {
            std::swap(d.Cf, d.Cnf);
            k_bc_c_pet_f<6><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch();
        }
        if (tp) F8_CUDA_RET(cudaMemcpyAsync(tp->Cn, d.Cf, 6 * hbf, cudaMemcpyDeviceToDevice, s));
        if ((e = cudaGetLastError())) return e;
    } else {
        kmark(F8_KERNEL_CODES, 0); kmark(F8_KERNEL_CODES, 1);
        mark(1);
        kmark(F8_KERNEL_UPDATE, 0); kmark(F8_KERNEL_UPDATE, 1);
    }
    mark(2);
    {
        MomArgsF a{};
        a.U = d.Uf; a.V = d.Vf; a.W = d.Wf; a.Ph = d.Pf; a.Pl = d.Pl; a.C = d.Cf; a.fpet = d.fpetf;
        for (int c = 0; c < 3; ++c) {
            a.A0[c] = d.A0f[c]; a.T0[c] = d.T0f[c]; a.Q[c] = d.Qf[c];
            a.F[c] = d.Funi[c] ? nullptr : d.Ff[c];
            a.Fu[c] = d.Fval[c];
        }
        a.cs = d.cs; a.polymer = o.polymer; a.ab2_first = o.ab2_first;
        a.coef_t = (float)((1.0 - d.ph.beta) / (d.ph.re * d.ph.wi));
        a.vis = (float)(d.ph.beta / d.ph.re);
        a.dt = (float)d.ph.dt;
        dim3 blk(32, 8);
        kmark(F8_KERNEL_MOMENTUM, 0);
        if (d3) { k_momentum3_f<<<cell_grid_m(g, blk), blk, 0, s>>>(a, g, mc); count_launch(); }
        else { k_momentum2_f<<<cell_grid_m(g, blk), blk, 0, s>>>(a, g, mc); count_launch(); }
        kmark(F8_KERNEL_MOMENTUM, 1);
        if ((e = cudaGetLastError())) return e;
    }
    if (o.polymer && g.walls) {
        // the momentum stage was the last reader of the updated ghost rows:
        // extrapolate them (C_kabe at the end of the reference's step,
        // fenep_2d.f90:1374), beside the IBM stage when a side stream exists
        const int ng = 2 * g.sx * g.sz;
        if (gbranch) {
            F8_CUDA_RET(cudaEventRecord(d.ev_g[3], s));
            F8_CUDA_RET(cudaStreamWaitEvent(sg, d.ev_g[3], 0));
        }
        if (d3) { k_extrap_ghost_f<6><<<(ng + 255) / 256, 256, 0, sg>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch(); }
        else { k_extrap_ghost_f<3><<<(ng + 255) / 256, 256, 0, sg>>>(d.Cf, d.fpetf, g, d.cs, d.ph.lp2); count_launch(); }
    }
    if (tp) {
        k_tape_ua<<<tnb, 256, 0, s>>>(d.Uf, d.Ul, d.Vf, d.Vl, d.Wf, d.Wl, d.Qf[0], d.Qf[1], d.Qf[2], tp->Ua[0],
                                      tp->Ua[1], tp->Ua[2], tp->U, tp->V, tp->W, g, df_from_d(2.0 * g.uwall));
        count_launch();
    }
    mark(3);
    // IBM direct forcing and the Helmholtz solves; with NS > 1 forcing
    // iterations (smac.f90:1607-1611) each further iteration interpolates
    // U* = U^n + dU of the last solve, adds to the marker forces, spreads them
    // onto the right-hand sides saved before the first spread and solves again
    const int repeats = o.ibm ? std::max(1, d.ibm_repeats) : 1;
    const int nvc = d3 ? 3 : 2;   // velocity components
    for (int r = 0; r < repeats; ++r) {
        if (o.ibm) {
            IbmArgsF a{};
            a.mu = d.mu; a.mv = d.mv; a.mcyl = d.mcyl; a.nm = d.nm;
            const float *Uh[3] = {d.Uf, d.Vf, d.Wf}, *Ul[3] = {d.Ul, d.Vl, d.Wl};
            // z weights of the stencil offset k - n = -1, 0, 1 (marker plane at
            // (n - 1/4) dZ; u, v at (k - 1/2) dZ, w at k dZ)
            auto roma = [](double r) {
                double ar = std::fabs(r);
                if (ar < 1.5 && ar >= 0.5) return (5.0 - 3.0 * ar - std::sqrt(-3.0 * ((1 - ar) * (1 - ar)) + 1.0)) / 6.0;
                if (ar < 0.5) return (1.0 + std::sqrt(-3.0 * (r * r) + 1.0)) / 3.0;
                return 0.0;
            };
            for (int c = 0; c < nvc; ++c) {
                a.wx[c] = d.mwx[c]; a.wy[c] = d.mwy[c]; a.i0[c] = d.mi0[c]; a.j0[c] = d.mj0[c];
                a.Uh[c] = Uh[c]; a.Ul[c] = Ul[c]; a.Qc[c] = d.Qf[c]; a.Fc[c] = d.Fc[c]; a.Fcf[c] = d.Fcf[c]; a.off[c] = d.csr_off[c];
                a.idx[c] = d.csr_idx[c]; a.cw[c] = d.csr_w[c]; a.act[c] = d.act_cols[c]; a.nact[c] = d.nact[c]; a.Q[c] = d.Qf[c];
                for (int dk = 0; dk < 3; ++dk) {
                    double zg = (dk - 1) + (c == 2 ? 0.5 : 0.0) - 0.5 + 0.25;  // (k - 1/2 [+1/2]) - (n - 1/4), k = n - 1 + dk
                    // 2D: one marker plane and no z weight (fenep_2d.f90:1726-1819)
                    a.wz[c][dk] = d3 ? (float)roma(zg) : (dk == 1 ? 1.0f : 0.0f);
                }
            }
            a.uw2 = df_from_d(2.0 * g.uwall);
            a.idt = 1.0 / g.dt;
            a.dtf = (float)g.dt;
            const bool last = r == repeats - 1;
            a.mode = r > 0 ? 1 : 0;
            a.accumulate = r > 0 ? 1 : 0;
            for (int c = 0; c < nvc; ++c) {
                a.D[c] = d.dUf[c];
                a.Qb[c] = (r > 0 && d.Qpre[c]) ? d.Qpre[c] : d.Qf[c];
            }
            if (r == 0 && repeats > 1)
                for (int c = 0; c < nvc; ++c)
                    F8_CUDA_RET(cudaMemcpyAsync(d.Qpre[c], d.Qf[c], (size_t)d.ni * sizeof(float), cudaMemcpyDeviceToDevice, s));
            dim3 gi((d.nm + 31) / 32, g.nz, nvc);
            k_ibm_interp_f<<<gi, dim3(32, 3), 0, s>>>(a, g); count_launch();
            int maxact = 0;
            for (int c = 0; c < nvc; ++c) maxact = std::max(maxact, d.nact[c]);
            if (maxact > 0) { k_ibm_spread_f<<<dim3((maxact + 127) / 128, g.nz, nvc), 128, 0, s>>>(a, g); count_launch(); }
            if (last && drag_out_dev) F8_CUDA_RET(launch_drag(d, drag_out_dev, s));
            if ((e = cudaGetLastError())) return e;
            if (tp && last)
                for (int c = 0; c < 3; ++c)
                    F8_CUDA_RET(cudaMemcpyAsync(tp->Fc[c], d.Fc[c], (size_t)d.nm * g.nz * sizeof(double),
                                                cudaMemcpyDeviceToDevice, s));
        }
        if (r == 0) mark(4);
        // Helmholtz solves for the FP32 increments dU (U* = U^n + dU).  On the
        // fused spectral path the three solves are independent branches: V and W
        // run on side streams with their own spectra, forked from and joined to
        // the step's stream (parallel branches of the captured graph), so their
        // x transforms fill the SMs that one solve's kernels leave idle.
        const double lhs1 = d.ph.dt * d.ph.beta / d.ph.re / 2.0;
        const bool branches = d.fused_planes && d.aux[0] && d.aux[1];
        if (branches) {
            F8_CUDA_RET(cudaEventRecord(d.ev_fork, s));
            for (int b = 0; b < 2; ++b) F8_CUDA_RET(cudaStreamWaitEvent(d.aux[b], d.ev_fork, 0));
        }
        for (int c = 0; c < nvc; ++c) {
            const XOutF out{d.dUf[c], nullptr, 0};
            if (branches) {
                cudaStream_t sc = c == 0 ? s : d.aux[c - 1];
                float *spec = c == 0 ? d.Hf : d.HfB[c - 1];
                if (!g.walls) e = solve_periodic_fused<float>(d, d.Qf[c], out, 1.0f, (float)lhs1, sc, spec);
                else e = solve_walls_fused<float>(d, d.Qf[c], out, c == 1 ? SYS_V : SYS_U, sc, spec);
            } else if (!g.walls) {
                e = solve_periodic_f(d, d.Qf[c], out, 1.0, lhs1, s);
            } else {
                e = solve_walls_f(d, d.Qf[c], out, c == 1 ? SYS_V : SYS_U, s);
            }
            if (e) return e;
        }
        if (branches) {
            for (int b = 0; b < 2; ++b) {
                F8_CUDA_RET(cudaEventRecord(d.ev_join[b], d.aux[b]));
                F8_CUDA_RET(cudaStreamWaitEvent(s, d.ev_join[b], 0));
            }
        }
        if (tp) {
            const TapeUp a{{d.Uf, d.Vf, d.Wf}, {d.dUf[0], d.dUf[1], d.dUf[2]}, {tp->Up[0], tp->Up[1], tp->Up[2]}};
            k_tape_up<<<dim3(tnb, 3), 256, 0, s>>>(a, g); count_launch();
        }
    }
    mark(5);
    // Poisson: FP32 solve + one df64 defect correction.  The increments and
    // Phi get no halo pass: their readers wrap / apply the Neumann rule.
    const dim3 pblk(32, 8), pgrid((g.nx + pblk.x - 1) / pblk.x, (g.ny + pblk.y - 1) / pblk.y, (g.nz + 1) / 2);
    kmark(F8_KERNEL_POISSON_RHS, 0);
    k_poisson_rhs_df<<<pgrid, pblk, 0, s>>>(U, V, W, d.dUf[0], d.dUf[1], d.dUf[2], d.Rhf, d.Rlf, g, mc);
    count_launch();
    kmark(F8_KERNEL_POISSON_RHS, 1);
    if (o.poisson == F8_POISSON_SOR) {
        kmark(F8_KERNEL_DEFECT, 0); kmark(F8_KERNEL_DEFECT, 1);
        if ((e = sor_solve_m(d, o, sor_iters, s))) return e;
    } else {
        *sor_iters = -1;
        // the first solve writes the FP32 Phi (high parts only); the
        // correction of the defect solve then sets Phi = Phi + dPhi exactly
        // as a df64 pair
        XOutF out{d.Phif, d.Phil, 0};
        if (!g.walls) e = solve_periodic_f(d, d.Rhf, out, 0.0, -1.0, s);
        else e = solve_walls_f(d, d.Rhf, out, SYS_P, s);
        if (e) return e;
        kmark(F8_KERNEL_DEFECT, 0);
        k_defect_df<<<pgrid, pblk, 0, s>>>(d.Phif, d.Rhf, d.Rlf, d.Rdf, g, mc); count_launch();
        kmark(F8_KERNEL_DEFECT, 1);
        out.mode = 2;
        if (!g.walls) e = solve_periodic_f(d, d.Rdf, out, 0.0, -1.0, s);
        else e = solve_walls_f(d, d.Rdf, out, SYS_P, s);
        if (e) return e;
    }
    if (tp) { k_tape_phi<<<tnb, 256, 0, s>>>(d.Phif, tp->Phi, g); count_launch(); }
    mark(6);
    kmark(F8_KERNEL_MARCH, 0);
    if (d.march_runs > 0) {
        MarchTmaArgs ma{};
        const float *pw[MT_PW] = {U.hi, U.lo, V.hi, V.lo, W.hi, W.lo, P.hi, P.lo, d.dUf[0], d.dUf[1], d.dUf[2]};
        float *ou[8] = {U.hi, U.lo, V.hi, V.lo, W.hi, W.lo, P.hi, P.lo};
        for (int q = 0; q < MT_PW; ++q) ma.pw[q] = pw[q];
        for (int q = 0; q < 8; ++q) ma.out[q] = ou[q];
        ma.phi[0] = Phi.hi; ma.phi[1] = Phi.lo;
        ma.zruns = d.march_runs;
        ma.depth = d.march_depth;
        k_march_tma<<<d.march_ctas, MT_THREADS, march_tma_smem(g, d.march_depth), s>>>(ma, g, mc, d.cnt);
    } else {
        k_march_df<<<pgrid, pblk, 0, s>>>(U, V, W, P, d.dUf[0], d.dUf[1], d.dUf[2], Phi, g, mc, d.cnt);
    }
    count_launch();
    kmark(F8_KERNEL_MARCH, 1);
    F8_CUDA_RET(launch_bc_set(state_bc_set(d), g, s));
    if (gbranch) {
        // join the ghost-row branch (when the Helmholtz branches did not)
        F8_CUDA_RET(cudaEventRecord(d.ev_g[2], sg));
        F8_CUDA_RET(cudaStreamWaitEvent(s, d.ev_g[2], 0));
    }
    if (tp && o.polymer) {
        F8_CUDA_RET(cudaMemcpyAsync(tp->codes, d.codes, (size_t)d.ni, cudaMemcpyDeviceToDevice, s));
        if (g.walls)
            F8_CUDA_RET(cudaMemcpyAsync(tp->codes_g, d.codes_g, (size_t)2 * g.nx * g.nz, cudaMemcpyDeviceToDevice, s));
    }
    mark(7);
    return cudaGetLastError();
}

}  // namespace f8
