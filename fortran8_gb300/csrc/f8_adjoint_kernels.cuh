// f8_adjoint_kernels.cuh — kernels of the discrete adjoint of the 3D step,
// templated on the arithmetic type T of the adjoint fields and of the tape:
// double for the FP64 step (f8_adjoint.cu, compiled without FMA contraction),
// float for the FP32-mixed step (f8_adjoint_mixed.cu).  The gradient with
// respect to the parameters is accumulated in FP64 in both (per-block sums
// added to one FP64 array).
//
// The reverse of one step runs the transposes of its stages in reverse order:
//   projection + pressure update  (fenep.f90:1562-1604)       k_march_adj
//   Poisson solve                  (1529-1560; walls fenep_2d.f90:1179-1342)
//                                  the forward solve again: its operator is
//                                  symmetric, and the adjoint right-hand side
//                                  has zero mean, so the pseudo-inverse's
//                                  null-space choice does not reach a gradient
//   divergence                     k_div_adj
//   Helmholtz solves               (1430-1527) the forward solves again
//   IBM direct forcing             (fenep_mpi.f90:1794-1929)   k_ibm_adj
//   momentum right-hand side       (fenep.f90:645-770, 1469)   k_momadj_src, k_momadj_gather
//   Lyapunov Newton + Cstar        (fenep.f90:464-643)         k_polyadj_mu, k_polyadj_cstar,
//                                                               k_polyadj_gather
// Halo fills (fenep.f90:147-166, fenep_2d.f90:1098-1143) are linear maps of
// the interior; their transposes (k_fold_*) move the adjoint gathered on halo
// cells back to the interior cells they were copied from.
//
// Differentiation conventions: the SPD candidate choice of the face
// reconstruction (fenep.f90:220-230) is frozen (the derivative flows through
// the chosen candidate); the Newton solution C* of G(C) = A C + C A^T - b = 0
// is differentiated by the implicit-function theorem with the exact 6x6
// Jacobian at C*; d|u|/du = sign(u), 0 at 0.
//
// The momentum and polymer transposes are gathers (each position sums, in a
// fixed order, the contributions of the cells whose stencils read it); the
// IBM transpose scatters with atomics onto the few stencil cells of the
// markers, and the parameter gradient is a sum of per-block partials added
// atomically, so the gradient is reproducible to round-off.
#pragma once
#include <initializer_list>
#include <utility>
#include "f8_common.cuh"
#include "f8_df64.cuh"

namespace f8 {
namespace {

__device__ inline bool adj_inner(const Geo &g, int i, int j, int k) {
    return i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz;
}

// value of an adjoint field at (i, j, k) if that cell is interior, else 0
template <typename T>
__device__ inline T lin(const T *A, const Geo &g, int i, int j, int k) {
    return adj_inner(g, i, j, k) ? A[hix(g, i, j, k)] : T(0);
}

template <typename T>
__device__ inline T sgn(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// Grid coefficients of the adjoint stencils in the arithmetic type T,
// formed once on the host in FP64, so the kernels multiply instead of divide.
template <typename T>
struct AdjCoef {
    T dt;
    T id[3];     // 1/dX, 1/dY, 1/dZ
    T id2[3];    // 1/dX^2, ...
    T i4[3];     // 1/(4 dX), ...
    T dtd[3];    // dt/dX, ...
    T dt2d[3];   // dt/(2 dX), ...
    T dt4d[3];   // dt/(4 dX), ...
};

template <typename T>
inline AdjCoef<T> adj_coef(const Geo &g) {
    AdjCoef<T> c{};
    const double d[3] = {g.dx, g.dy, g.dz};
    c.dt = T(g.dt);
    for (int q = 0; q < 3; ++q) {
        c.id[q] = T(1.0 / d[q]);
        c.id2[q] = T(1.0 / (d[q] * d[q]));
        c.i4[q] = T(1.0 / (4.0 * d[q]));
        c.dtd[q] = T(g.dt / d[q]);
        c.dt2d[q] = T(g.dt / (2.0 * d[q]));
        c.dt4d[q] = T(g.dt / (4.0 * d[q]));
    }
    return c;
}

// Block sum of v added to *dst in FP64 (every thread of the block calls it).
// Block sum of a float partial added to *dst: the partials are summed as
// double-float pairs (two-sums on the FP32 pipes), converted to double once
// per block.  A double reduction tree would run on GB300's FP64 pipe, a small
// fraction of its FP32 rate, and cost more than the FP32 kernels around it.
__device__ inline void block_atomic_add(float v, double *dst) {
    __shared__ float shh[32], shl[32];
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    df s{v, 0.0f};
    for (int o = 16; o > 0; o >>= 1)
        s = df_add(s, df{__shfl_down_sync(0xffffffffu, s.hi, o), __shfl_down_sync(0xffffffffu, s.lo, o)});
    __syncthreads();
    if ((t & 31) == 0) { shh[t >> 5] = s.hi; shl[t >> 5] = s.lo; }
    __syncthreads();
    if (t < 32) {
        df r = t < (nt >> 5) ? df{shh[t], shl[t]} : df{0.0f, 0.0f};
        for (int o = 16; o > 0; o >>= 1)
            r = df_add(r, df{__shfl_down_sync(0xffffffffu, r.hi, o), __shfl_down_sync(0xffffffffu, r.lo, o)});
        if (t == 0 && (r.hi != 0.0f || r.lo != 0.0f)) atomicAdd(dst, (double)r.hi + (double)r.lo);
    }
}

__device__ inline void block_atomic_add(double v, double *dst) {
    __shared__ double sh[32];
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        double s = t < (nt >> 5) ? sh[t] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (t == 0 && s != 0.0) atomicAdd(dst, s);
    }
}

// ---------------------------------------------------------------------------
// Transposed halo fills.  The forward fill is x, then y, then z (each copy
// reading cells the earlier copies may have written), so the transpose folds
// z, then y, then x.

template <typename T>
struct FoldSet {
    T *A[12];
    int kind[12];
    int n;
};

template <typename T>
__global__ void k_fold_z(FoldSet<T> f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.sy) return;
    const int i = t % g.sx, j = t / g.sx;
    const int lo = hix(g, i, j, 0), hi = hix(g, i, j, g.sz - 1), top = hix(g, i, j, g.nz), bot = hix(g, i, j, 1);
    T *A = f.A[blockIdx.y];
    const T a = A[lo], b = A[hi];
    A[top] += a;
    A[bot] += b;
    A[lo] = T(0);
    A[hi] = T(0);
}

template <typename T>
__global__ void k_fold_y(FoldSet<T> f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.nz) return;
    const int i = t % g.sx, k = 1 + t / g.sx;
    const int g0 = hix(g, i, 0, k), g1 = hix(g, i, g.ny + 1, k), r1 = hix(g, i, 1, k), rn = hix(g, i, g.ny, k);
    const int q = blockIdx.y;
    T *A = f.A[q];
    const T a = A[g0], b = A[g1];
    if (!g.walls) {
        A[rn] += a;
        A[r1] += b;
    } else {
        switch (f.kind[q]) {
        case BC_U:
        case BC_W: A[r1] -= a; A[rn] -= b; break;     // ghost = -U (2 Uwall - U)
        case BC_V: A[rn] = T(0); break;               // V(:,0) = V(:,NY) = V(:,NY+1) = 0
        case BC_P: A[r1] += a; A[rn] += b; break;     // Neumann copies
        default:                                      // C: 2 C(1) - C(2), 2 C(NY) - C(NY-1)
            A[r1] += T(2) * a; A[hix(g, i, 2, k)] -= a;
            A[rn] += T(2) * b; A[hix(g, i, g.ny - 1, k)] -= b;
        }
    }
    A[g0] = T(0);
    A[g1] = T(0);
}

// rows: 1..NY, or every row 0..NY+1 (rows_all) for the periodic x/z fill of
// the updated wall ghost rows
template <typename T>
__global__ void k_fold_x(FoldSet<T> f, Geo g, int rows_all) {
    const int ny = rows_all ? g.sy : g.ny, j0 = rows_all ? 0 : 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ny * g.nz) return;
    const int j = j0 + t % ny, k = 1 + t / ny;
    const int lo = hix(g, 0, j, k), hi = hix(g, g.sx - 1, j, k);
    T *A = f.A[blockIdx.y];
    const T a = A[lo], b = A[hi];
    A[hix(g, g.nx, j, k)] += a;
    A[hix(g, 1, j, k)] += b;
    A[lo] = T(0);
    A[hi] = T(0);
}

// one block row (blockIdx.y) per field of the set: the fields are independent
template <typename T>
cudaError_t fold(const FoldSet<T> &f, const Geo &g, cudaStream_t s) {
    const unsigned n = (unsigned)f.n;
    if (n == 0) return cudaSuccess;
    k_fold_z<T><<<dim3((g.sx * g.sy + 255) / 256, n), 256, 0, s>>>(f, g); count_launch();
    k_fold_y<T><<<dim3((g.sx * g.nz + 255) / 256, n), 256, 0, s>>>(f, g); count_launch();
    k_fold_x<T><<<dim3((g.ny * g.nz + 255) / 256, n), 256, 0, s>>>(f, g, 0); count_launch();
    return cudaGetLastError();
}

// the z pass of fold alone: for a set whose values outside the z faces'
// planes lie only in interior columns below row NY, where the y and x passes
// would move and zero nothing
template <typename T>
cudaError_t fold_z_only(const FoldSet<T> &f, const Geo &g, cudaStream_t s) {
    const unsigned n = (unsigned)f.n;
    if (n == 0) return cudaSuccess;
    k_fold_z<T><<<dim3((g.sx * g.sy + 255) / 256, n), 256, 0, s>>>(f, g); count_launch();
    return cudaGetLastError();
}

// transpose of the periodic x and z copies of every row (k_bc_c_pet_xz): the
// wall ghost rows stay (they are updated cells)
template <typename T>
cudaError_t fold_xz(const FoldSet<T> &f, const Geo &g, cudaStream_t s) {
    const unsigned n = (unsigned)f.n;
    if (n == 0) return cudaSuccess;
    k_fold_z<T><<<dim3((g.sx * g.sy + 255) / 256, n), 256, 0, s>>>(f, g); count_launch();
    k_fold_x<T><<<dim3((g.sy * g.nz + 255) / 256, n), 256, 0, s>>>(f, g, 1); count_launch();
    return cudaGetLastError();
}

template <typename T>
FoldSet<T> fold_set(std::initializer_list<std::pair<T *, int>> fields) {
    FoldSet<T> f{};
    for (auto &p : fields) { f.A[f.n] = p.first; f.kind[f.n] = p.second; ++f.n; }
    return f;
}

template <typename T>
FoldSet<T> fold_c(T *C, int cs, int ncomp = 6) {
    FoldSet<T> f{};
    for (int m = 0; m < ncomp; ++m) { f.A[m] = C + (size_t)m * cs; f.kind[m] = BC_C; }
    f.n = ncomp;
    return f;
}

// the fields of a and then those of C (ncomp components), folded in one pass
template <typename T>
FoldSet<T> fold_with_c(FoldSet<T> a, T *C, int cs, int ncomp) {
    for (int m = 0; m < ncomp; ++m) { a.A[a.n] = C + (size_t)m * cs; a.kind[a.n] = BC_C; ++a.n; }
    return a;
}

// ---------------------------------------------------------------------------
// Projection and pressure update:  U = Up - dt dPhi/dx ..., P += Phi - pc lap Phi.
// One thread per cell of the full halo box gathers the adjoint of Phi there.

template <typename T>
__global__ void k_march_adj(const T *lU, const T *lV, const T *lW, const T *lP, T *lPhi, const T *Phi, Geo g, T pc,
                            T c_beta, AdjCoef<T> kc, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    T gb = T(0);
    if (t < cs) {
        const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
        T lam = kc.dtd[0] * (lin(lU, g, i, j, k) - lin(lU, g, i - 1, j, k))
              + kc.dtd[1] * (lin(lV, g, i, j, k) - lin(lV, g, i, j - 1, k))
              + kc.dtd[2] * (lin(lW, g, i, j, k) - lin(lW, g, i, j, k - 1));
        const T p0 = lin(lP, g, i, j, k);
        const T lap = (lin(lP, g, i - 1, j, k) - 2 * p0 + lin(lP, g, i + 1, j, k)) * kc.id2[0]
                    + (lin(lP, g, i, j - 1, k) - 2 * p0 + lin(lP, g, i, j + 1, k)) * kc.id2[1]
                    + (lin(lP, g, i, j, k - 1) - 2 * p0 + lin(lP, g, i, j, k + 1)) * kc.id2[2];
        lPhi[t] = lam + p0 - pc * lap;
        if (adj_inner(g, i, j, k) && p0 != T(0)) {
            const T ph = Phi[t];
            const T lf = (Phi[hix(g, i - 1, j, k)] - 2 * ph + Phi[hix(g, i + 1, j, k)]) * kc.id2[0]
                       + (Phi[hix(g, i, j - 1, k)] - 2 * ph + Phi[hix(g, i, j + 1, k)]) * kc.id2[1]
                       + (Phi[hix(g, i, j, k - 1)] - 2 * ph + Phi[hix(g, i, j, k + 1)]) * kc.id2[2];
            gb = -c_beta * p0 * lf;
        }
    }
    block_atomic_add(gb, grad + 1);
}

// interior of a halo field -> packed interior array
template <typename T>
__global__ void k_pack(const T *A, T *out, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    out[qix(g, i, j, k)] = A[hix(g, i, j, k)];
}

// k_pack of three fields in one launch
template <typename T>
__global__ void k_pack3(const T *A0, const T *A1, const T *A2, T *out0, T *out1, T *out2, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const int q = qix(g, i, j, k), h = hix(g, i, j, k);
    const T a = A0[h], b = A1[h], c = A2[h];
    out0[q] = a;
    out1[q] = b;
    out2[q] = c;
}

// Divergence right-hand side q = div(Up)/dt (fenep.f90:1547-1555) transposed,
// plus the identity part U = Up + ... of the projection; full halo box.
template <typename T>
__global__ void k_div_adj(const T *lU, const T *lV, const T *lW, const T *lq, T *lUp, T *lVp, T *lWp, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const T dt = T(g.dt);
    const T q0 = lin(lq, g, i, j, k);
    lUp[t] = lin(lU, g, i, j, k) + (q0 - lin(lq, g, i + 1, j, k)) / T(g.dx) / dt;
    lVp[t] = lin(lV, g, i, j, k) + (q0 - lin(lq, g, i, j + 1, k)) / T(g.dy) / dt;
    lWp[t] = lin(lW, g, i, j, k) + (q0 - lin(lq, g, i, j, k + 1)) / T(g.dz) / dt;
}

// ---------------------------------------------------------------------------
// IBM.  Roma kernel (fenep.f90:2045-2055) and its derivative.

template <typename T>
__device__ inline T roma_t(T r) {
    const T ar = fabs(r);
    if (ar < T(1.5) && ar >= T(0.5)) return (T(5) - T(3) * ar - sqrt(T(-3) * ((T(1) - ar) * (T(1) - ar)) + T(1))) / T(6);
    if (ar < T(0.5)) return (T(1) + sqrt(T(-3) * (r * r) + T(1))) / T(3);
    return T(0);
}

template <typename T>
__device__ inline T droma_t(T r) {
    const T ar = fabs(r);
    if (ar < T(0.5)) return -r / sqrt(T(1) - T(3) * r * r);
    if (ar < T(1.5)) {
        const T s = T(1) - ar;
        return sgn(r) * (T(-3) - T(3) * s / sqrt(T(1) - T(3) * s * s)) / T(6);
    }
    return T(0);
}

constexpr int MAX_CYL_SHARED = 64;

template <typename T>
struct IbmAdjArgs {
    const double *mx, *my;
    const int *mcyl;
    int nm, ncyl;
    double dvol, dxn;
    const double *mvol;      // per marker: spreading volume
    const double *cylvol;    // per cylinder: drag volume
    const T *Ua[3];          // forward Ua (halo, with boundary values)
    const double *Fc[3];     // forward marker forces
    const T *lQ[3];          // adjoint of the Helmholtz right-hand sides (interior)
    T *lUa[3];               // out: adjoint of Ua (full halo box, scattered)
    const double *w;         // drag weights of this step (ncyl x 3)
    double *grad;            // grad[3 + 2 l], grad[4 + 2 l]: cylinder centre
    int d3;                  // 0: the 2D step (one marker plane, no z weight, fenep_2d.f90:1726-1819)
};

// One thread per (marker, plane, component).  Forward: Ub = sum Ua delta dX^3,
// Fc = (Uc - Ub)/dt, drag = -dv sum Fc, f = fold(sum Fc delta dX^3),
// Q = Ua + dt f - dt B/2.  Marker offsets from the grid points are formed in
// FP64 (the marker positions are FP64) and the kernel weights in T.
template <typename T>
__global__ void k_ibm_adj(IbmAdjArgs<T> a, Geo g) {
    __shared__ double gc[2 * MAX_CYL_SHARED];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y + 1;
    const int comp = blockIdx.z;
    const bool use_sh = a.ncyl <= MAX_CYL_SHARED;
    for (int q = threadIdx.x; q < 2 * MAX_CYL_SHARED; q += blockDim.x) gc[q] = 0.0;
    __syncthreads();
    if (m < a.nm) {
        const double dX = g.dx, dY = g.dy, dZ = g.dz;
        // reciprocals: one FP64 division each instead of one per stencil
        // weight (GB300's FP64 pipe is a small fraction of its FP32 rate)
        const double idX = 1.0 / dX, idY = 1.0 / dY, idZ = 1.0 / dZ;
        const T dt = T(g.dt);
        const double xc = a.mx[m], yc = a.my[m], zc = (n - 0.25) * dZ;
        int i0, j0;
        if (comp == 0) { j0 = (int)(yc / dY); i0 = (int)(xc / dX - 0.5); }
        else if (comp == 1) { j0 = (int)(yc / dY - 0.5); i0 = (int)(xc / dX); }
        else { j0 = (int)(yc / dY); i0 = (int)(xc / dX); }
        const int l = a.mcyl[m];
        const size_t fo = (size_t)m + (size_t)a.nm * (n - 1);
        const T fc = T(a.Fc[comp][fo]);
        const T *lQ = a.lQ[comp];
        const T *Ua = a.Ua[comp];
        const T dvn = T(a.dxn / a.dvol);          // interpolation: dX^3 / (dX dY dZ)
        const T svn = T(a.mvol[m] / a.dvol);      // spreading: marker volume / (dX dY dZ)
        T wxs[3], wys[3], wzs[3], dwx[3], dwy[3];
        for (int q = 0; q < 3; ++q) {
            double x = (i0 + q - 0.5) * dX, y = (j0 + q - 0.5) * dY, z = (n - 1 + q - 0.5) * dZ;
            if (comp == 0) x = x + 0.5 * dX;
            else if (comp == 1) y = y + 0.5 * dY;
            else z = z + 0.5 * dZ;
            const T rx = T((x - xc) * idX), ry = T((y - yc) * idY), rz = T((z - zc) * idZ);
            wxs[q] = roma_t(rx);
            wys[q] = roma_t(ry);
            wzs[q] = a.d3 ? roma_t(rz) : (q == 1 ? T(1) : T(0));
            dwx[q] = -droma_t(rx) * T(idX);   // d/dxc
            dwy[q] = -droma_t(ry) * T(idY);
        }
        // adjoint of Fc: drag weight + the folded spreading
        T lfc = T(-a.cylvol[l] * a.w[3 * l + comp]);
        T gx = T(0), gy = T(0);
        for (int kk = 0; kk < 3; ++kk) {
            const int k = n - 1 + kk;
            const int fk = k == 0 ? g.nz : (k == g.nz + 1 ? 1 : k);
            for (int jj = 0; jj < 3; ++jj) {
                const int j = j0 + jj;
                int fj = j;
                bool drop = false;
                if (j == 0 || j == g.ny + 1) {
                    if (g.walls) drop = true;
                    else fj = j == 0 ? g.ny : 1;
                }
                for (int ii = 0; ii < 3; ++ii) {
                    const int i = i0 + ii;
                    const int fi = i == 0 ? g.nx : (i == g.nx + 1 ? 1 : i);
                    const T lf = drop ? T(0) : dt * lQ[hix(g, fi, fj, fk)];
                    const T del = wxs[ii] * wys[jj] * wzs[kk];
                    lfc += lf * del * svn;
                    gx += lf * fc * svn * (dwx[ii] * wys[jj] * wzs[kk]);
                    gy += lf * fc * svn * (wxs[ii] * dwy[jj] * wzs[kk]);
                }
            }
        }
        const T lub = -lfc / dt;
        T *lUa = a.lUa[comp];
        for (int kk = 0; kk < 3; ++kk) {
            const int k = n - 1 + kk;
            for (int jj = 0; jj < 3; ++jj) {
                const int j = j0 + jj;
                for (int ii = 0; ii < 3; ++ii) {
                    const int i = i0 + ii;
                    const int h = hix(g, i, j, k);
                    const T del = wxs[ii] * wys[jj] * wzs[kk];
                    atomicAdd(&lUa[h], lub * del * dvn);
                    const T u = Ua[h];
                    gx += lub * u * dvn * (dwx[ii] * wys[jj] * wzs[kk]);
                    gy += lub * u * dvn * (wxs[ii] * dwy[jj] * wzs[kk]);
                }
            }
        }
        if (use_sh) {
            atomicAdd(&gc[2 * l], (double)gx);
            atomicAdd(&gc[2 * l + 1], (double)gy);
        } else {
            atomicAdd(&a.grad[3 + 2 * l], (double)gx);
            atomicAdd(&a.grad[4 + 2 * l], (double)gy);
        }
    }
    __syncthreads();
    if (use_sh)
        for (int q = threadIdx.x; q < 2 * a.ncyl; q += blockDim.x)
            if (gc[q] != 0.0) atomicAdd(&a.grad[3 + q], gc[q]);
}

// ---------------------------------------------------------------------------
// Momentum right-hand side (fenep.f90:645-770, 1469-1474, with the IBM form
// Ua = U + gp + dt(3A - A0)/2 + dt B + dt(T + T0)/2 + dt F) transposed.

template <typename T>
struct MomAdjArgs {
    const T *U, *V, *W;               // forward U^n (halo)
    const T *Up[3];                   // forward Helmholtz solutions (halo)
    const T *lQ[3];                   // adjoint of Q (interior of halo arrays)
    const T *lUa[3];                  // adjoint of Ua from the interpolation (interior)
    T *lA0[3], *lT0[3];               // in: adjoint of the new history; out: of the old
    AdjCoef<T> kc;
    int cs, ab2_first, polymer;
    T vis, coef_t, c_helm;            // beta/Re, (1-beta)/(Re Wi), dt/(2 Re)
    T inv_re;
    double *grad;
};

// ---------------------------------------------------------------------------
// Polymer update transposed: implicit-function adjoint of the Lyapunov Newton
// solve and the Cstar upwind sum (fenep.f90:464-643).

template <typename T>
struct W3 {
    T m, c, p;   // weights of C at the - neighbour, the cell, the + neighbour
};

template <typename T>
__device__ inline W3<T> wface_p(int idx) {
    switch (idx) {
    case 1: return {T(0), T(1.5), T(-0.5)};
    case 2: return {T(0.5), T(0.5), T(0)};
    case 3: return {T(0.25), T(1), T(-0.25)};
    default: return {T(0), T(1), T(0)};
    }
}
template <typename T>
__device__ inline W3<T> wface_n(int idx) {
    switch (idx) {
    case 1: return {T(0), T(0.5), T(0.5)};
    case 2: return {T(-0.5), T(1.5), T(0)};
    case 3: return {T(-0.25), T(1), T(0.25)};
    default: return {T(0), T(1), T(0)};
    }
}

template <typename T>
struct PolyAdjArgs {
    const T *C, *Cn;                  // C^n (the state) and C after the update (halo, 6 SoA fields)
    const uint8_t *codes, *codes_g;
    const T *U, *V, *W;               // U^n (halo)
    const T *lX;                      // adjoint of C^{n+1} (interior)
    AdjCoef<T> kc;
    int cs;
    T dt, wi, lp2;
    T dtwi, dtwi2;                    // dt/Wi, dt/Wi^2
    double *grad;
};

// value of a halo field at row jj of column (i, k); zero beyond the ghost rows
// of a wall channel (the reference wall mode's outside rows)
template <typename T>
__device__ inline T rowv(const T *A, const Geo &g, int i, int jj, int k) {
    return (jj < 0 || jj > g.ny + 1) ? T(0) : A[hix(g, i, jj, k)];
}

__device__ inline int code_of(const uint8_t *codes, const uint8_t *codes_g, const Geo &g, int i, int j, int k) {
    return (j >= 1 && j <= g.ny) ? codes[qix(g, i, j, k)] : codes_g[gcix(g, i, j, k)];
}

// mu = J^-T lx for the Jacobian J = dG/dx of the Lyapunov residual
// G(x) = A x + x A^T + (1 + f(x) dt/Wi) x - b at the Newton solution x
// (fenep.f90:588-605, component order xx, xy, xz, yy, yz, zz): Gaussian
// elimination with partial pivoting on the 6 x 7 augmented transpose.  The
// pivot row is found by compare-and-exchange with each lower row, so every
// index is a compile-time constant and the matrix stays in registers.
template <typename T>
__device__ inline void solve_jt6(const T (&A)[3][3], T dd2, T cf, const T (&x)[6], const T (&lx)[6], T (&mu)[6]) {
    T J[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int q = 0; q < 6; ++q) J[r][q] = T(0);
    J[0][0] = 2 * A[0][0]; J[0][1] = 2 * A[0][1]; J[0][2] = 2 * A[0][2];
    J[1][0] = A[1][0]; J[1][1] = A[1][1] + A[0][0]; J[1][2] = A[1][2]; J[1][3] = A[0][1]; J[1][4] = A[0][2];
    J[2][0] = A[2][0]; J[2][1] = A[2][1]; J[2][2] = A[2][2] + A[0][0]; J[2][4] = A[0][1]; J[2][5] = A[0][2];
    J[3][1] = 2 * A[1][0]; J[3][3] = 2 * A[1][1]; J[3][4] = 2 * A[1][2];
    J[4][1] = A[2][0]; J[4][2] = A[1][0]; J[4][3] = A[2][1]; J[4][4] = A[2][2] + A[1][1]; J[4][5] = A[1][2];
    J[5][2] = 2 * A[2][0]; J[5][4] = 2 * A[2][1]; J[5][5] = 2 * A[2][2];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        J[r][r] += dd2;
        J[r][0] += cf * x[r];
        J[r][3] += cf * x[r];
        J[r][5] += cf * x[r];
    }
    T M[6][7];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
        for (int q = 0; q < 6; ++q) M[r][q] = J[q][r];
        M[r][6] = lx[r];
    }
    T inv[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
#pragma unroll
        for (int r = c + 1; r < 6; ++r) {
            const bool sw = fabs(M[r][c]) > fabs(M[c][c]);
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                if (q < c) continue;
                const T u0 = M[c][q], u1 = M[r][q];
                M[c][q] = sw ? u1 : u0;
                M[r][q] = sw ? u0 : u1;
            }
        }
        inv[c] = T(1) / M[c][c];
#pragma unroll
        for (int r = c + 1; r < 6; ++r) {
            const T fr = M[r][c] * inv[c];
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                if (q < c) continue;
                M[r][q] -= fr * M[c][q];
            }
        }
    }
#pragma unroll
    for (int r = 5; r >= 0; --r) {
        T s = M[r][6];
#pragma unroll
        for (int q = 0; q < 6; ++q)
            if (q > r) s -= M[r][q] * mu[q];
        mu[r] = s * inv[r];
    }
}

// ---------------------------------------------------------------------------
// Gather forms of the momentum and polymer transposes (no atomics; the result
// at each position is a fixed-order sum, so those stages are deterministic).
// Pass 1 of each writes per-cell sources; pass 2 gathers, at every position,
// the contributions of the cells whose stencils read that position.  The
// coefficients are those of the momentum stencils (fenep.f90:645-770), of
// C0 = f(C) C - I, and of Cstar and the Lyapunov update (fenep.f90:464-643),
// regrouped by target position.

constexpr int MOM_SRC = 12;    // lua (3), ga = -lA (3), vis lB (3), coef_t lT (3)
constexpr int POLY_SRC = 34;   // mu (6), Cstar weights (13), A0 adjoint (9), upwind-face adjoint (6)
enum { PS_MU = 0, PS_KC = 6, PS_KX = 7, PS_KY = 11, PS_KZ = 15, PS_GU = 19, PS_GV = 22, PS_GW = 25, PS_SF = 28 };

// Momentum, pass 1 (interior cells): the sources, the history adjoints
// lA0 / lT0 (updated in place: each cell reads and writes only its own) and
// the beta terms of the viscous and Helmholtz coefficients.
template <typename T>
__global__ void __launch_bounds__(256) k_momadj_src(MomAdjArgs<T> a, T *src, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    T gb = T(0);
    if (i <= g.nx && j <= g.ny) {
        const AdjCoef<T> &kc = a.kc;
        const T dt = kc.dt;
        const T h2 = T(0.5), h15 = T(1.5);
        const int o = qix(g, i, j, k), h = hix(g, i, j, k);
        const int sx = g.sx, sxy = g.sx * g.sy;
        const size_t cs = (size_t)a.cs;
        const T *F[3] = {a.U, a.V, a.W};
        // every load of the three components precedes the first store: the
        // stores may alias the inputs as far as the compiler knows, so loads
        // after a store would each wait for their own round trip
        T lq[3], lu0[3], la0[3], lt0[3], xp[3][7], xf[3][7];
        auto load7 = [&](const T *X, T (&x)[7]) {
            x[0] = X[h];
            x[1] = X[h - 1]; x[2] = X[h + 1];
            x[3] = X[h - sx]; x[4] = X[h + sx];
            x[5] = X[h - sxy]; x[6] = X[h + sxy];
        };
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lq[c] = a.lQ[c][h];
            lu0[c] = a.lUa[c][h];
            la0[c] = a.lA0[c][o];
            lt0[c] = a.lT0[c][o];
            load7(a.Up[c], xp[c]);
            load7(F[c], xf[c]);
        }
        auto lap = [&](const T (&x)[7]) {
            return (x[1] - 2 * x[0] + x[2]) * kc.id2[0] + (x[3] - 2 * x[0] + x[4]) * kc.id2[1]
                 + (x[5] - 2 * x[0] + x[6]) * kc.id2[2];
        };
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T lua = lq[c] + lu0[c];
            T lA = h15 * dt * lua + la0[c];
            T lT = h2 * dt * lua + lt0[c];
            if (a.ab2_first) {
                lA += -h2 * dt * lua;
                lT += h2 * dt * lua;
                a.lA0[c][o] = T(0);
                a.lT0[c][o] = T(0);
            } else {
                a.lA0[c][o] = -h2 * dt * lua;
                a.lT0[c][o] = h2 * dt * lua;
            }
            const T lB = dt * lua - h2 * dt * lq[c];
            src[(size_t)(0 + c) * cs + h] = lua;
            src[(size_t)(3 + c) * cs + h] = -lA;
            src[(size_t)(6 + c) * cs + h] = a.vis * lB;
            src[(size_t)(9 + c) * cs + h] = a.polymer ? a.coef_t * lT : T(0);
            // Helmholtz coefficient dt beta/(2 Re) and viscous coefficient beta/Re
            if (lq[c] != T(0)) gb += a.c_helm * lq[c] * lap(xp[c]);
            gb += a.inv_re * lB * lap(xf[c]);
        }
    }
    block_atomic_add(gb, a.grad + 1);
}

template <typename T>
struct MomGatherArgs {
    const T *U, *V, *W;       // forward U^n (halo)
    const T *src;             // MOM_SRC halo-layout arrays of k_momadj_src (interior cells)
    T *lU, *lV, *lW;          // out: adjoint of U^n from the momentum stage (full halo box)
    T *lP;                    // adjoint of P^n, += the pressure-gradient transpose
    const T *C;               // C as the stress read it (6 SoA halo fields)
    T *lC;                    // += the transpose of C0 = f(C) C - I (6 fields)
    AdjCoef<T> kc;
    int cs, polymer;
    T lp2, inv_1mb, inv_wi;
    double *grad;
};

// Momentum, pass 2 (every position of the halo box): the adjoint of U, V, W
// at the position from the momentum stencils of the (up to 9 per component)
// interior cells that read it, the pressure-gradient transpose, and with the
// polymer the adjoint of C0 (stress divergence) followed by the C0 = f(C) C - I
// linearisation.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_momadj_gather(MomGatherArgs<T> a, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = a.cs;
    T g_coef = T(0), g_l2 = T(0);
    if (t < cs) {
        const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
        const AdjCoef<T> &kc = a.kc;
        const T iX = kc.id[0], iY = kc.id[1], iZ = kc.id[2];
        const T ix2 = kc.id2[0], iy2 = kc.id2[1], iz2 = kc.id2[2];
        const T *U = a.U, *V = a.V, *W = a.W;
        // all stencil coordinates below are offsets (x, y, z) from this
        // position; a source cell at offset (x, y, z) with |x|, |y|, |z| <= 1
        // is an interior cell when ex[x + 1] && ey[y + 1] && ez[z + 1]
        const int sx = g.sx, sxy = g.sx * g.sy;
        const bool ex[3] = {i - 1 >= 1 && i - 1 <= g.nx, i >= 1 && i <= g.nx, i + 1 >= 1 && i + 1 <= g.nx};
        const bool ey[3] = {j - 1 >= 1 && j - 1 <= g.ny, j >= 1 && j <= g.ny, j + 1 >= 1 && j + 1 <= g.ny};
        const bool ez[3] = {k - 1 >= 1 && k - 1 <= g.nz, k >= 1 && k <= g.nz, k + 1 >= 1 && k + 1 <= g.nz};
        auto ev = [&](int x, int y, int z) { return ex[x + 1] && ey[y + 1] && ez[z + 1]; };
        auto at = [&](int x, int y, int z) { return t + x + sx * y + sxy * z; };
        auto S = [&](int q, int x, int y, int z) { return a.src[(size_t)q * cs + at(x, y, z)]; };
        auto u = [&](int x, int y, int z) { return U[at(x, y, z)]; };
        auto v = [&](int x, int y, int z) { return V[at(x, y, z)]; };
        auto w = [&](int x, int y, int z) { return W[at(x, y, z)]; };
        const T h = T(0.5);
        // velocity averages of the convection stencils around source cell (x, y, z)
        auto ax_t1 = [&](int x, int y, int z) { return (u(x - 1, y, z) + u(x, y, z)) * h; };
        auto ax_t2 = [&](int x, int y, int z) { return (u(x, y, z) + u(x + 1, y, z)) * h; };
        auto axy_a1 = [&](int x, int y, int z) { return (v(x, y - 1, z) + v(x + 1, y - 1, z)) * h; };
        auto axy_b1 = [&](int x, int y, int z) { return (u(x, y - 1, z) + u(x, y, z)) * h; };
        auto axy_a2 = [&](int x, int y, int z) { return (v(x, y, z) + v(x + 1, y, z)) * h; };
        auto axy_b2 = [&](int x, int y, int z) { return (u(x, y, z) + u(x, y + 1, z)) * h; };
        auto axz_c1 = [&](int x, int y, int z) { return (w(x, y, z - 1) + w(x + 1, y, z - 1)) * h; };
        auto axz_d1 = [&](int x, int y, int z) { return (u(x, y, z - 1) + u(x, y, z)) * h; };
        auto axz_c2 = [&](int x, int y, int z) { return (w(x, y, z) + w(x + 1, y, z)) * h; };
        auto axz_d2 = [&](int x, int y, int z) { return (u(x, y, z) + u(x, y, z + 1)) * h; };
        auto ayx_a1 = [&](int x, int y, int z) { return (u(x - 1, y, z) + u(x - 1, y + 1, z)) * h; };
        auto ayx_b1 = [&](int x, int y, int z) { return (v(x - 1, y, z) + v(x, y, z)) * h; };
        auto ayx_a2 = [&](int x, int y, int z) { return (u(x, y, z) + u(x, y + 1, z)) * h; };
        auto ayx_b2 = [&](int x, int y, int z) { return (v(x, y, z) + v(x + 1, y, z)) * h; };
        auto ay_t3 = [&](int x, int y, int z) { return (v(x, y - 1, z) + v(x, y, z)) * h; };
        auto ay_t4 = [&](int x, int y, int z) { return (v(x, y, z) + v(x, y + 1, z)) * h; };
        auto ayz_c1 = [&](int x, int y, int z) { return (w(x, y, z - 1) + w(x, y + 1, z - 1)) * h; };
        auto ayz_d1 = [&](int x, int y, int z) { return (v(x, y, z - 1) + v(x, y, z)) * h; };
        auto ayz_c2 = [&](int x, int y, int z) { return (w(x, y, z) + w(x, y + 1, z)) * h; };
        auto ayz_d2 = [&](int x, int y, int z) { return (v(x, y, z) + v(x, y, z + 1)) * h; };
        auto azx_a1 = [&](int x, int y, int z) { return (u(x - 1, y, z) + u(x - 1, y, z + 1)) * h; };
        auto azx_b1 = [&](int x, int y, int z) { return (w(x - 1, y, z) + w(x, y, z)) * h; };
        auto azx_a2 = [&](int x, int y, int z) { return (u(x, y, z) + u(x, y, z + 1)) * h; };
        auto azx_b2 = [&](int x, int y, int z) { return (w(x, y, z) + w(x + 1, y, z)) * h; };
        auto azy_c1 = [&](int x, int y, int z) { return (v(x, y - 1, z) + v(x, y - 1, z + 1)) * h; };
        auto azy_d1 = [&](int x, int y, int z) { return (w(x, y - 1, z) + w(x, y, z)) * h; };
        auto azy_c2 = [&](int x, int y, int z) { return (v(x, y, z) + v(x, y, z + 1)) * h; };
        auto azy_d2 = [&](int x, int y, int z) { return (w(x, y, z) + w(x, y + 1, z)) * h; };
        auto az_t5 = [&](int x, int y, int z) { return (w(x, y, z - 1) + w(x, y, z)) * h; };
        auto az_t6 = [&](int x, int y, int z) { return (w(x, y, z) + w(x, y, z + 1)) * h; };
        // sources: lua 0-2, ga 3-5 (ga, gbv, gc of the x, y, z fluxes), lb 6-8, st 9-11
        T lu = T(0), lv = T(0), lw = T(0), lp = T(0);
        // ---- U ----
        if (ev(0, 0, 0)) {
            const int x = 0, y = 0, z = 0;
            const T ga = S(3, x, y, z), gbv = S(4, x, y, z), gc = S(5, x, y, z);
            lu += S(0, x, y, z) - 2 * S(6, x, y, z) * (ix2 + iy2 + iz2) + ga * (ax_t2(x, y, z) - ax_t1(x, y, z)) * iX
                + ga * iY * (axy_a2(x, y, z) - axy_a1(x, y, z)) * h + ga * iZ * (axz_c2(x, y, z) - axz_c1(x, y, z)) * h
                + gbv * iX * ayx_b2(x, y, z) * h + gc * iX * azx_b2(x, y, z) * h;
        }
        if (ev(1, 0, 0)) {
            const int x = 1, y = 0, z = 0;
            lu += S(6, x, y, z) * ix2 - S(3, x, y, z) * ax_t1(x, y, z) * iX - S(4, x, y, z) * iX * ayx_b1(x, y, z) * h
                - S(5, x, y, z) * iX * azx_b1(x, y, z) * h;
        }
        if (ev(-1, 0, 0)) {
            const int x = -1, y = 0, z = 0;
            lu += S(6, x, y, z) * ix2 + S(3, x, y, z) * ax_t2(x, y, z) * iX;
        }
        if (ev(0, 1, 0)) {
            const int x = 0, y = 1, z = 0;
            lu += S(6, x, y, z) * iy2 - S(3, x, y, z) * iY * axy_a1(x, y, z) * h;
        }
        if (ev(0, -1, 0)) {
            const int x = 0, y = -1, z = 0;
            lu += S(6, x, y, z) * iy2 + S(3, x, y, z) * iY * axy_a2(x, y, z) * h + S(4, x, y, z) * iX * ayx_b2(x, y, z) * h;
        }
        if (ev(0, 0, 1)) {
            const int x = 0, y = 0, z = 1;
            lu += S(6, x, y, z) * iz2 - S(3, x, y, z) * iZ * axz_c1(x, y, z) * h;
        }
        if (ev(0, 0, -1)) {
            const int x = 0, y = 0, z = -1;
            lu += S(6, x, y, z) * iz2 + S(3, x, y, z) * iZ * axz_c2(x, y, z) * h + S(5, x, y, z) * iX * azx_b2(x, y, z) * h;
        }
        if (ev(1, -1, 0)) {
            const int x = 1, y = -1, z = 0;
            lu -= S(4, x, y, z) * iX * ayx_b1(x, y, z) * h;
        }
        if (ev(1, 0, -1)) {
            const int x = 1, y = 0, z = -1;
            lu -= S(5, x, y, z) * iX * azx_b1(x, y, z) * h;
        }
        // ---- V ----
        if (ev(0, 0, 0)) {
            const int x = 0, y = 0, z = 0;
            const T ga = S(3, x, y, z), gbv = S(4, x, y, z), gc = S(5, x, y, z);
            lv += S(1, x, y, z) - 2 * S(7, x, y, z) * (ix2 + iy2 + iz2) + ga * iY * axy_b2(x, y, z) * h
                + gbv * iX * (ayx_a2(x, y, z) - ayx_a1(x, y, z)) * h + gbv * (ay_t4(x, y, z) - ay_t3(x, y, z)) * iY
                + gbv * iZ * (ayz_c2(x, y, z) - ayz_c1(x, y, z)) * h + gc * iY * azy_d2(x, y, z) * h;
        }
        if (ev(1, 0, 0)) {
            const int x = 1, y = 0, z = 0;
            lv += S(7, x, y, z) * ix2 - S(4, x, y, z) * iX * ayx_a1(x, y, z) * h;
        }
        if (ev(-1, 0, 0)) {
            const int x = -1, y = 0, z = 0;
            lv += S(7, x, y, z) * ix2 + S(3, x, y, z) * iY * axy_b2(x, y, z) * h + S(4, x, y, z) * iX * ayx_a2(x, y, z) * h;
        }
        if (ev(0, 1, 0)) {
            const int x = 0, y = 1, z = 0;
            lv += S(7, x, y, z) * iy2 - S(3, x, y, z) * iY * axy_b1(x, y, z) * h - S(4, x, y, z) * ay_t3(x, y, z) * iY
                - S(5, x, y, z) * iY * azy_d1(x, y, z) * h;
        }
        if (ev(0, -1, 0)) {
            const int x = 0, y = -1, z = 0;
            lv += S(7, x, y, z) * iy2 + S(4, x, y, z) * ay_t4(x, y, z) * iY;
        }
        if (ev(0, 0, 1)) {
            const int x = 0, y = 0, z = 1;
            lv += S(7, x, y, z) * iz2 - S(4, x, y, z) * iZ * ayz_c1(x, y, z) * h;
        }
        if (ev(0, 0, -1)) {
            const int x = 0, y = 0, z = -1;
            lv += S(7, x, y, z) * iz2 + S(4, x, y, z) * iZ * ayz_c2(x, y, z) * h + S(5, x, y, z) * iY * azy_d2(x, y, z) * h;
        }
        if (ev(-1, 1, 0)) {
            const int x = -1, y = 1, z = 0;
            lv -= S(3, x, y, z) * iY * axy_b1(x, y, z) * h;
        }
        if (ev(0, 1, -1)) {
            const int x = 0, y = 1, z = -1;
            lv -= S(5, x, y, z) * iY * azy_d1(x, y, z) * h;
        }
        // ---- W ----
        if (ev(0, 0, 0)) {
            const int x = 0, y = 0, z = 0;
            const T ga = S(3, x, y, z), gbv = S(4, x, y, z), gc = S(5, x, y, z);
            lw += S(2, x, y, z) - 2 * S(8, x, y, z) * (ix2 + iy2 + iz2) + ga * iZ * axz_d2(x, y, z) * h
                + gbv * iZ * ayz_d2(x, y, z) * h + gc * iX * (azx_a2(x, y, z) - azx_a1(x, y, z)) * h
                + gc * iY * (azy_c2(x, y, z) - azy_c1(x, y, z)) * h + gc * (az_t6(x, y, z) - az_t5(x, y, z)) * iZ;
        }
        if (ev(1, 0, 0)) {
            const int x = 1, y = 0, z = 0;
            lw += S(8, x, y, z) * ix2 - S(5, x, y, z) * iX * azx_a1(x, y, z) * h;
        }
        if (ev(-1, 0, 0)) {
            const int x = -1, y = 0, z = 0;
            lw += S(8, x, y, z) * ix2 + S(3, x, y, z) * iZ * axz_d2(x, y, z) * h + S(5, x, y, z) * iX * azx_a2(x, y, z) * h;
        }
        if (ev(0, 1, 0)) {
            const int x = 0, y = 1, z = 0;
            lw += S(8, x, y, z) * iy2 - S(5, x, y, z) * iY * azy_c1(x, y, z) * h;
        }
        if (ev(0, -1, 0)) {
            const int x = 0, y = -1, z = 0;
            lw += S(8, x, y, z) * iy2 + S(4, x, y, z) * iZ * ayz_d2(x, y, z) * h + S(5, x, y, z) * iY * azy_c2(x, y, z) * h;
        }
        if (ev(0, 0, 1)) {
            const int x = 0, y = 0, z = 1;
            lw += S(8, x, y, z) * iz2 - S(3, x, y, z) * iZ * axz_d1(x, y, z) * h - S(4, x, y, z) * iZ * ayz_d1(x, y, z) * h
                - S(5, x, y, z) * az_t5(x, y, z) * iZ;
        }
        if (ev(0, 0, -1)) {
            const int x = 0, y = 0, z = -1;
            lw += S(8, x, y, z) * iz2 + S(5, x, y, z) * az_t6(x, y, z) * iZ;
        }
        if (ev(-1, 0, 1)) {
            const int x = -1, y = 0, z = 1;
            lw -= S(3, x, y, z) * iZ * axz_d1(x, y, z) * h;
        }
        if (ev(0, -1, 1)) {
            const int x = 0, y = -1, z = 1;
            lw -= S(4, x, y, z) * iZ * ayz_d1(x, y, z) * h;
        }
        // pressure gradient gp_c = -dt (P(o + e_c) - P(o)) / d_c, transposed
        if (ev(0, 0, 0)) lp += kc.dtd[0] * S(0, 0, 0, 0) + kc.dtd[1] * S(1, 0, 0, 0) + kc.dtd[2] * S(2, 0, 0, 0);
        if (ev(-1, 0, 0)) lp -= kc.dtd[0] * S(0, -1, 0, 0);
        if (ev(0, -1, 0)) lp -= kc.dtd[1] * S(1, 0, -1, 0);
        if (ev(0, 0, -1)) lp -= kc.dtd[2] * S(2, 0, 0, -1);
        const T lp0 = a.lP[t];
        if (a.polymer) {
            // adjoint of C0 from the stress divergence (fenep.f90:645-691):
            // sT = coef_t lT of the interior cells whose stencils read C0 here
            auto st = [&](int c, int x, int y, int z) { return ev(x, y, z) ? S(9 + c, x, y, z) : T(0); };
            const T q4x = kc.i4[0], q4y = kc.i4[1], q4z = kc.i4[2];
            T l0[6];
            l0[0] = (st(0, -1, 0, 0) - st(0, 0, 0, 0)) * iX;
            l0[3] = (st(1, 0, -1, 0) - st(1, 0, 0, 0)) * iY;
            l0[5] = (st(2, 0, 0, -1) - st(2, 0, 0, 0)) * iZ;
            l0[1] = q4y * (st(0, 0, -1, 0) + st(0, -1, -1, 0) - st(0, 0, 1, 0) - st(0, -1, 1, 0))
                  + q4x * (st(1, -1, 0, 0) + st(1, -1, -1, 0) - st(1, 1, 0, 0) - st(1, 1, -1, 0));
            l0[2] = q4z * (st(0, 0, 0, -1) + st(0, -1, 0, -1) - st(0, 0, 0, 1) - st(0, -1, 0, 1))
                  + q4x * (st(2, -1, 0, 0) + st(2, -1, 0, -1) - st(2, 1, 0, 0) - st(2, 1, 0, -1));
            l0[4] = q4z * (st(1, 0, 0, -1) + st(1, 0, -1, -1) - st(1, 0, 0, 1) - st(1, 0, -1, 1))
                  + q4y * (st(2, 0, -1, 0) + st(2, 0, -1, -1) - st(2, 0, 1, 0) - st(2, 0, 1, -1));
            bool any = false;
            for (int m = 0; m < 6; ++m) any = any || l0[m] != T(0);
            if (any) {
                // C0 = f(C) C - I linearised
                const T E[6] = {T(1), T(0), T(0), T(1), T(0), T(1)};
                T c[6], lc[6];
#pragma unroll
                for (int m = 0; m < 6; ++m) {
                    c[m] = a.C[(size_t)m * cs + t];
                    lc[m] = a.lC[(size_t)m * cs + t];
                }
                const T tr3 = (c[0] - T(1)) + (c[3] - T(1)) + (c[5] - T(1));
                const T den = (a.lp2 - 3) - tr3;
                const T iden = T(1) / den;
                const T f = (a.lp2 - 3) * iden;
                const T fm1 = tr3 * iden;
                T lf = T(0);
#pragma unroll
                for (int m = 0; m < 6; ++m) {
                    lc[m] += f * l0[m];
                    lf += c[m] * l0[m];
                    g_coef += (fm1 * c[m] + (c[m] - E[m])) * l0[m];
                }
                const T dfdtr = f * iden;
                lc[0] += lf * dfdtr;
                lc[3] += lf * dfdtr;
                lc[5] += lf * dfdtr;
#pragma unroll
                for (int m = 0; m < 6; ++m) a.lC[(size_t)m * cs + t] = lc[m];
                g_l2 = -lf * tr3 * (iden * iden);
            }
        }
        // the stores last: loads after a store could not be moved ahead of it
        a.lU[t] = lu;
        a.lV[t] = lv;
        a.lW[t] = lw;
        a.lP[t] = lp0 + lp;
    }
    if (a.polymer) {
        block_atomic_add(-g_coef * a.inv_1mb, a.grad + 1);
        block_atomic_add(-g_coef * a.inv_wi, a.grad + 0);
        block_atomic_add(g_l2, a.grad + 2);
    }
}

// Polymer, pass 1 (the updated cells; with walls also the ghost rows), in two
// kernels so that neither holds the registers of both halves.  Pass 1a: the
// implicit-function adjoint mu = J^-T lC^{n+1} at the Newton solution, the
// adjoint of the velocity-gradient entries and the Wi and L^2 terms.
template <typename T>
__global__ void __launch_bounds__(128) k_polyadj_mu(PolyAdjArgs<T> a, T *__restrict__ src, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j < prow0(g) + prows(g);
    T gwi = T(0), gl2 = T(0);
    if (active) {
        const size_t cs = (size_t)a.cs;
        const int h = hix(g, i, j, k);
        auto put = [&](int q, T v) { src[(size_t)q * cs + h] = v; };
        const AdjCoef<T> &kc = a.kc;
        const T lp2 = a.lp2;
        T lx[6], x[6];
        bool any = false;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            lx[m] = a.lX[m * cs + h];
            x[m] = a.Cn[m * cs + h];
            any = any || lx[m] != T(0);
        }
        if (!any) {
#pragma unroll
            for (int m = 0; m < 6; ++m) put(PS_MU + m, T(0));
#pragma unroll
            for (int q = PS_GU; q < PS_SF; ++q) put(q, T(0));
        } else {
            const T *U = a.U, *V = a.V, *W = a.W;
            auto u = [&](int p, int q, int r) { return rowv(U, g, p, q, r); };
            auto v = [&](int p, int q, int r) { return rowv(V, g, p, q, r); };
            auto w = [&](int p, int q, int r) { return rowv(W, g, p, q, r); };
            T A0[3][3];
            A0[0][0] = -(-u(i - 1, j, k) + u(i, j, k)) * kc.dtd[0];
            A0[0][1] = -(-v(i - 1, j - 1, k) + v(i + 1, j - 1, k) - v(i - 1, j, k) + v(i + 1, j, k)) * kc.dt4d[0];
            A0[0][2] = -(-w(i - 1, j, k - 1) + w(i + 1, j, k - 1) - w(i - 1, j, k) + w(i + 1, j, k)) * kc.dt4d[0];
            A0[1][0] = -(-u(i - 1, j - 1, k) - u(i, j - 1, k) + u(i - 1, j + 1, k) + u(i, j + 1, k)) * kc.dt4d[1];
            A0[1][1] = -(-v(i, j - 1, k) + v(i, j, k)) * kc.dtd[1];
            A0[1][2] = -(-w(i, j - 1, k - 1) + w(i, j + 1, k - 1) - w(i, j - 1, k) + w(i, j + 1, k)) * kc.dt4d[1];
            A0[2][0] = -(-u(i - 1, j, k - 1) - u(i, j, k - 1) + u(i - 1, j, k + 1) + u(i, j, k + 1)) * kc.dt4d[2];
            A0[2][1] = -(-v(i, j - 1, k - 1) - v(i, j, k - 1) + v(i, j - 1, k + 1) + v(i, j, k + 1)) * kc.dt4d[2];
            A0[2][2] = -(-w(i, j, k - 1) + w(i, j, k)) * kc.dtd[2];
            T A[3][3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) A[r][q] = A0[q][r];
            const T tr3 = (x[0] - T(1)) + (x[3] - T(1)) + (x[5] - T(1));
            const T den = (lp2 - 3) - tr3;
            const T iden = T(1) / den;
            const T f = (lp2 - 3) * iden;
            const T fm1 = tr3 * iden;
            const T dd2 = T(1) + f * a.dtwi;
            const T cf = a.dtwi * f * iden;
            T mu[6];
            solve_jt6(A, dd2, cf, x, lx, mu);
            T mx = T(0), mxe = T(0);
            const T E[6] = {T(1), T(0), T(0), T(1), T(0), T(1)};
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                mx += mu[m] * x[m];
                mxe += mu[m] * (x[m] - E[m]);
                put(PS_MU + m, mu[m]);
            }
            gwi = a.dtwi2 * (fm1 * mx + mxe);
            gl2 = a.dtwi * tr3 * (iden * iden) * mx;
            // adjoint of the velocity-gradient entries, each scaled by the
            // coefficient of its stencil (A0 entries / dt d or dt 4d)
            T lAt[3][3];
            lAt[0][0] = -(2 * mu[0] * x[0] + mu[1] * x[1] + mu[2] * x[2]);
            lAt[0][1] = -(2 * mu[0] * x[1] + mu[1] * x[3] + mu[2] * x[4]);
            lAt[0][2] = -(2 * mu[0] * x[2] + mu[1] * x[4] + mu[2] * x[5]);
            lAt[1][0] = -(mu[1] * x[0] + 2 * mu[3] * x[1] + mu[4] * x[2]);
            lAt[1][1] = -(mu[1] * x[1] + 2 * mu[3] * x[3] + mu[4] * x[4]);
            lAt[1][2] = -(mu[1] * x[2] + 2 * mu[3] * x[4] + mu[4] * x[5]);
            lAt[2][0] = -(mu[2] * x[0] + mu[4] * x[1] + 2 * mu[5] * x[2]);
            lAt[2][1] = -(mu[2] * x[1] + mu[4] * x[3] + 2 * mu[5] * x[4]);
            lAt[2][2] = -(mu[2] * x[2] + mu[4] * x[4] + 2 * mu[5] * x[5]);
            put(PS_GU + 0, lAt[0][0] * kc.dtd[0]);
            put(PS_GU + 1, lAt[0][1] * kc.dt4d[1]);
            put(PS_GU + 2, lAt[0][2] * kc.dt4d[2]);
            put(PS_GV + 0, lAt[1][0] * kc.dt4d[0]);
            put(PS_GV + 1, lAt[1][1] * kc.dtd[1]);
            put(PS_GV + 2, lAt[1][2] * kc.dt4d[2]);
            put(PS_GW + 0, lAt[2][0] * kc.dt4d[0]);
            put(PS_GW + 1, lAt[2][1] * kc.dt4d[1]);
            put(PS_GW + 2, lAt[2][2] * kc.dtd[2]);
        }
    }
    block_atomic_add(gwi, a.grad + 0);
    block_atomic_add(gl2, a.grad + 2);
}

// Pass 1b: the 13 Cstar weights of the cell (the same for the 6 components:
// centre, x/y/z at offsets -2, -1, +1, +2) and the adjoint of the upwind
// coefficients, from the mu of pass 1a.  Where mu vanishes the gather reads
// the weights only multiplied by it, and they are stored as zero.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_polyadj_cstar(PolyAdjArgs<T> a, T *__restrict__ src, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const int k = blockIdx.z + 1;
    if (i > g.nx || j >= prow0(g) + prows(g)) return;
    const size_t cs = (size_t)a.cs;
    const int h = hix(g, i, j, k);
    auto put = [&](int q, T v) { src[(size_t)q * cs + h] = v; };
    const AdjCoef<T> &kc = a.kc;
    T mu[6];
    bool any = false;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        mu[m] = src[(size_t)(PS_MU + m) * cs + h];
        any = any || mu[m] != T(0);
    }
    if (!any) {
#pragma unroll
        for (int q = PS_KC; q < PS_GU; ++q) put(q, T(0));
#pragma unroll
        for (int q = PS_SF; q < POLY_SRC; ++q) put(q, T(0));
        return;
    }
    const T *U = a.U, *V = a.V, *W = a.W;
    // Cstar: upwind coefficients s1..s12 and the selection codes
    const T u1 = U[hix(g, i - 1, j, k)], u2 = U[h];
    const T v1 = rowv(V, g, i, j - 1, k), v2 = V[h];
    const T w1 = W[hix(g, i, j, k - 1)], w2 = W[h];
    const T sixth = T(1) / T(6);
    const int cself = code_of(a.codes, a.codes_g, g, i, j, k);
    const int cxm = code_of(a.codes, a.codes_g, g, wrapx(g, i - 1), j, k) & 3;
    const int cxp = code_of(a.codes, a.codes_g, g, wrapx(g, i + 1), j, k) & 3;
    const int czm = (code_of(a.codes, a.codes_g, g, i, j, wrapz(g, k - 1)) >> 4) & 3;
    const int czp = (code_of(a.codes, a.codes_g, g, i, j, wrapz(g, k + 1)) >> 4) & 3;
    int jm = j - 1, jp = j + 1;
    if (!g.walls) { jm = wrapy(g, jm); jp = wrapy(g, jp); }
    const int cym = jm < 0 ? 3 : (code_of(a.codes, a.codes_g, g, i, jm, k) >> 2) & 3;
    const int cyp = jp > g.ny + 1 ? 3 : (code_of(a.codes, a.codes_g, g, i, jp, k) >> 2) & 3;
    const int isx = (cself & 3) + 1, isy = ((cself >> 2) & 3) + 1, isz = ((cself >> 4) & 3) + 1;
    // One direction at a time (x, y, z), so that only its face weights and
    // sums are live: the weights of the cell's own p / n faces (coefficients
    // sp, sn), of the + neighbour's p face (sq) and of the - neighbour's n
    // face (sr) at offsets -2, -1, +1, +2, the centre weights summed in kcen;
    // then the adjoints of the direction's four upwind coefficients,
    // mu . (face value) with the faces rebuilt from C^n at positions
    // cm, c0, cp (own faces), q-, q0, q+ (+ neighbour's) and r-, r0, r+.
    T kcen = T(0);
    auto direction = [&](int isd, int cq, int cr, T vel2, T vel1, T dt2d, int base, int sf, auto &&cval) {
        const T sq = (-vel2 + fabs(vel2)) * dt2d, sn = sixth + (-vel2 - fabs(vel2)) * dt2d;
        const T sp = sixth + (vel1 - fabs(vel1)) * dt2d, sr = (vel1 + fabs(vel1)) * dt2d;
        const W3<T> wp_ = wface_p<T>(isd), wn_ = wface_n<T>(isd);
        const W3<T> wq = wface_p<T>(cq + 1), wr = wface_n<T>(cr + 1);
        put(base + 0, sr * wr.m);
        put(base + 1, sp * wp_.m + sn * wn_.m + sr * wr.c);
        put(base + 2, sp * wp_.p + sn * wn_.p + sq * wq.c);
        put(base + 3, sq * wq.p);
        kcen += sp * wp_.c + sn * wn_.c + sq * wq.m + sr * wr.p;
        auto face = [](W3<T> wt, T cmv, T c0v, T cpv) { return wt.m * cmv + wt.c * c0v + wt.p * cpv; };
        T lq = T(0), ln = T(0), lp_ = T(0), lr = T(0);
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            T v[9];
            cval(a.C + m * cs, v);
            const T mum = mu[m];
            lp_ += mum * face(wp_, v[0], v[1], v[2]);
            ln += mum * face(wn_, v[0], v[1], v[2]);
            lq += mum * face(wq, v[3], v[4], v[5]);
            lr += mum * face(wr, v[6], v[7], v[8]);
        }
        const T s2 = sgn(vel2), s1 = sgn(vel1);
        put(sf + 0, (lq * (T(-1) + s2) + ln * (T(-1) - s2)) * dt2d);    // -> the + face velocity
        put(sf + 1, (lp_ * (T(1) - s1) + lr * (T(1) + s1)) * dt2d);     // -> the - face velocity
    };
    const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
    const int hxm = hix(g, wrapx(g, i - 1), j, k), hxp = hix(g, wrapx(g, i + 1), j, k);
    direction(isx, cxp, cxm, u2, u1, kc.dt2d[0], PS_KX, PS_SF + 0, [&](const T *Cm, T (&v)[9]) {
        v[0] = Cm[h - ox]; v[1] = Cm[h]; v[2] = Cm[h + ox];
        v[3] = Cm[hxp - ox]; v[4] = Cm[hxp]; v[5] = Cm[hxp + ox];
        v[6] = Cm[hxm - ox]; v[7] = Cm[hxm]; v[8] = Cm[hxm + ox];
    });
    if (!g.walls) {
        const int hym = hix(g, i, jm, k), hyp = hix(g, i, jp, k);
        direction(isy, cyp, cym, v2, v1, kc.dt2d[1], PS_KY, PS_SF + 2, [&](const T *Cm, T (&v)[9]) {
            v[0] = Cm[h - oy]; v[1] = Cm[h]; v[2] = Cm[h + oy];
            v[3] = Cm[hyp - oy]; v[4] = Cm[hyp]; v[5] = Cm[hyp + oy];
            v[6] = Cm[hym - oy]; v[7] = Cm[hym]; v[8] = Cm[hym + oy];
        });
    } else {
        direction(isy, cyp, cym, v2, v1, kc.dt2d[1], PS_KY, PS_SF + 2, [&](const T *Cm, T (&v)[9]) {
            auto yv = [&](int jj) { return rowv(Cm, g, i, jj, k); };
            v[0] = yv(j - 1); v[1] = Cm[h]; v[2] = yv(j + 1);
            v[3] = v[1]; v[4] = v[2]; v[5] = yv(j + 2);
            v[6] = yv(j - 2); v[7] = v[0]; v[8] = v[1];
        });
    }
    const int hzm = hix(g, i, j, wrapz(g, k - 1)), hzp = hix(g, i, j, wrapz(g, k + 1));
    direction(isz, czp, czm, w2, w1, kc.dt2d[2], PS_KZ, PS_SF + 4, [&](const T *Cm, T (&v)[9]) {
        v[0] = Cm[h - oz]; v[1] = Cm[h]; v[2] = Cm[h + oz];
        v[3] = Cm[hzp - oz]; v[4] = Cm[hzp]; v[5] = Cm[hzp + oz];
        v[6] = Cm[hzm - oz]; v[7] = Cm[hzm]; v[8] = Cm[hzm + oz];
    });
    put(PS_KC, kcen);
}

template <typename T>
struct PolyGatherArgs {
    const T *src;             // POLY_SRC halo-layout arrays of k_polyadj_mu / _cstar (updated cells)
    T *lC;                    // out: adjoint of C^n (updated cells; zero elsewhere)
    T *lU, *lV, *lW;          // += the velocity adjoint (full halo box)
    int cs;
};

// Polymer, pass 2 (every position of the halo box): the adjoint of C^n at the
// updated cells from the Cstar weights of the cells whose upwind sums read it
// (periodic directions wrapped, as the forward reads them; with walls the
// rows beyond the ghost rows hold zero C and are not read), and the adjoint
// of U, V, W from the velocity-gradient and upwind-coefficient entries.
template <typename T>
__global__ void __launch_bounds__(256) k_polyadj_gather(PolyGatherArgs<T> a, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = a.cs;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const int r0 = prow0(g), r1 = prow0(g) + prows(g) - 1;
    auto upd = [&](int x, int y, int z) { return x >= 1 && x <= g.nx && y >= r0 && y <= r1 && z >= 1 && z <= g.nz; };
    auto S = [&](int q, int x, int y, int z) { return a.src[(size_t)q * cs + hix(g, x, y, z)]; };
    // velocity adjoint
    T lu = T(0), lv = T(0), lw = T(0);
    auto add = [&](T &acc, int q, int x, int y, int z, T sign) { if (upd(x, y, z)) acc += sign * S(q, x, y, z); };
    add(lu, PS_GU + 0, i, j, k, T(-1));        add(lu, PS_GU + 0, i + 1, j, k, T(1));
    add(lu, PS_GU + 1, i + 1, j + 1, k, T(1));  add(lu, PS_GU + 1, i, j + 1, k, T(1));
    add(lu, PS_GU + 1, i + 1, j - 1, k, T(-1)); add(lu, PS_GU + 1, i, j - 1, k, T(-1));
    add(lu, PS_GU + 2, i + 1, j, k + 1, T(1));  add(lu, PS_GU + 2, i, j, k + 1, T(1));
    add(lu, PS_GU + 2, i + 1, j, k - 1, T(-1)); add(lu, PS_GU + 2, i, j, k - 1, T(-1));
    add(lu, PS_SF + 0, i, j, k, T(1));          add(lu, PS_SF + 1, i + 1, j, k, T(1));
    add(lv, PS_GV + 0, i + 1, j + 1, k, T(1));  add(lv, PS_GV + 0, i - 1, j + 1, k, T(-1));
    add(lv, PS_GV + 0, i + 1, j, k, T(1));      add(lv, PS_GV + 0, i - 1, j, k, T(-1));
    add(lv, PS_GV + 1, i, j + 1, k, T(1));      add(lv, PS_GV + 1, i, j, k, T(-1));
    add(lv, PS_GV + 2, i, j + 1, k + 1, T(1));  add(lv, PS_GV + 2, i, j, k + 1, T(1));
    add(lv, PS_GV + 2, i, j + 1, k - 1, T(-1)); add(lv, PS_GV + 2, i, j, k - 1, T(-1));
    add(lv, PS_SF + 2, i, j, k, T(1));          add(lv, PS_SF + 3, i, j + 1, k, T(1));
    add(lw, PS_GW + 0, i + 1, j, k + 1, T(1));  add(lw, PS_GW + 0, i - 1, j, k + 1, T(-1));
    add(lw, PS_GW + 0, i + 1, j, k, T(1));      add(lw, PS_GW + 0, i - 1, j, k, T(-1));
    add(lw, PS_GW + 1, i, j + 1, k + 1, T(1));  add(lw, PS_GW + 1, i, j - 1, k + 1, T(-1));
    add(lw, PS_GW + 1, i, j + 1, k, T(1));      add(lw, PS_GW + 1, i, j - 1, k, T(-1));
    add(lw, PS_GW + 2, i, j, k + 1, T(1));      add(lw, PS_GW + 2, i, j, k, T(-1));
    add(lw, PS_SF + 4, i, j, k, T(1));          add(lw, PS_SF + 5, i, j, k + 1, T(1));
    const T lu0 = a.lU[t], lv0 = a.lV[t], lw0 = a.lW[t];
    // adjoint of C^n at the updated cells
    if (!upd(i, j, k)) {
        a.lU[t] = lu0 + lu;
        a.lV[t] = lv0 + lv;
        a.lW[t] = lw0 + lw;
        for (int m = 0; m < 6; ++m) a.lC[(size_t)m * cs + t] = T(0);
        return;
    }
    T l[6];
    {
        const T kc = S(PS_KC, i, j, k);
        for (int m = 0; m < 6; ++m) l[m] = kc * S(PS_MU + m, i, j, k);
    }
    // source cell n = p - o e reads p with its offset-o weight
    auto line = [&](int base, int x, int y, int z, int oq) {
        const T kw = S(base + oq, x, y, z);
        for (int m = 0; m < 6; ++m) l[m] += kw * S(PS_MU + m, x, y, z);
    };
    const int offs[4] = {-2, -1, 1, 2};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int o = offs[q];
        line(PS_KX, wrapx(g, i - o), j, k, q);
        line(PS_KZ, i, j, wrapz(g, k - o), q);
        if (!g.walls) line(PS_KY, i, wrapy(g, j - o), k, q);
        else if (j - o >= r0 && j - o <= r1) line(PS_KY, i, j - o, k, q);
    }
    // the stores last: loads after a store could not be moved ahead of it
    a.lU[t] = lu0 + lu;
    a.lV[t] = lv0 + lv;
    a.lW[t] = lw0 + lw;
    for (int m = 0; m < 6; ++m) a.lC[(size_t)m * cs + t] = l[m];
}

// interior of a halo field (reference layout) into an adjoint field, zero halo
template <typename T>
__global__ void k_take_interior(const T *src, T *dst, Geo g, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int cs = g.sx * g.sy * g.sz;
    const int h = t % cs;
    const int i = h % g.sx, j = (h / g.sx) % g.sy, k = h / (g.sx * g.sy);
    dst[t] = adj_inner(g, i, j, k) ? src[t] : T(0);
}

inline dim3 adj_cells(const Geo &g, dim3 b) { return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, g.nz); }

}  // namespace
}  // namespace f8
