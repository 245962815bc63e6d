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
//   momentum right-hand side       (fenep.f90:645-770, 1469)   k_momentum_adj, k_c0_adj
//   Lyapunov Newton + Cstar        (fenep.f90:464-643)         k_polymer_adj3
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
// Stencil transposes scatter with atomics into full halo arrays, so the
// adjoint fields are reproducible to round-off, not bit for bit.
#pragma once
#include <initializer_list>
#include <utility>
#include "f8_common.cuh"

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

// Block sum of v added to *dst in FP64 (every thread of the block calls it).
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
    T *A[8];
    int kind[8];
    int n;
};

template <typename T>
__global__ void k_fold_z(FoldSet<T> f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.sy) return;
    const int i = t % g.sx, j = t / g.sx;
    const int lo = hix(g, i, j, 0), hi = hix(g, i, j, g.sz - 1), top = hix(g, i, j, g.nz), bot = hix(g, i, j, 1);
    for (int q = 0; q < f.n; ++q) {
        T *A = f.A[q];
        const T a = A[lo], b = A[hi];
        A[top] += a;
        A[bot] += b;
        A[lo] = T(0);
        A[hi] = T(0);
    }
}

template <typename T>
__global__ void k_fold_y(FoldSet<T> f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.nz) return;
    const int i = t % g.sx, k = 1 + t / g.sx;
    const int g0 = hix(g, i, 0, k), g1 = hix(g, i, g.ny + 1, k), r1 = hix(g, i, 1, k), rn = hix(g, i, g.ny, k);
    for (int q = 0; q < f.n; ++q) {
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
    for (int q = 0; q < f.n; ++q) {
        T *A = f.A[q];
        const T a = A[lo], b = A[hi];
        A[hix(g, g.nx, j, k)] += a;
        A[hix(g, 1, j, k)] += b;
        A[lo] = T(0);
        A[hi] = T(0);
    }
}

template <typename T>
cudaError_t fold(const FoldSet<T> &f, const Geo &g, cudaStream_t s) {
    k_fold_z<T><<<(g.sx * g.sy + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_y<T><<<(g.sx * g.nz + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_x<T><<<(g.ny * g.nz + 255) / 256, 256, 0, s>>>(f, g, 0); count_launch();
    return cudaGetLastError();
}

// transpose of the periodic x and z copies of every row (k_bc_c_pet_xz): the
// wall ghost rows stay (they are updated cells)
template <typename T>
cudaError_t fold_xz(const FoldSet<T> &f, const Geo &g, cudaStream_t s) {
    k_fold_z<T><<<(g.sx * g.sy + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_x<T><<<(g.sy * g.nz + 255) / 256, 256, 0, s>>>(f, g, 1); count_launch();
    return cudaGetLastError();
}

template <typename T>
FoldSet<T> fold_set(std::initializer_list<std::pair<T *, int>> fields) {
    FoldSet<T> f{};
    for (auto &p : fields) { f.A[f.n] = p.first; f.kind[f.n] = p.second; ++f.n; }
    return f;
}

template <typename T>
FoldSet<T> fold_c(T *C, int cs) {
    FoldSet<T> f{};
    for (int m = 0; m < 6; ++m) { f.A[m] = C + (size_t)m * cs; f.kind[m] = BC_C; }
    f.n = 6;
    return f;
}

// ---------------------------------------------------------------------------
// Projection and pressure update:  U = Up - dt dPhi/dx ..., P += Phi - pc lap Phi.
// One thread per cell of the full halo box gathers the adjoint of Phi there.

template <typename T>
__global__ void k_march_adj(const T *lU, const T *lV, const T *lW, const T *lP, T *lPhi, const T *Phi, Geo g, T pc,
                            T c_beta, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    T gb = T(0);
    if (t < cs) {
        const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
        const T dt = T(g.dt), dX = T(g.dx), dY = T(g.dy), dZ = T(g.dz);
        T lam = dt / dX * (lin(lU, g, i, j, k) - lin(lU, g, i - 1, j, k))
              + dt / dY * (lin(lV, g, i, j, k) - lin(lV, g, i, j - 1, k))
              + dt / dZ * (lin(lW, g, i, j, k) - lin(lW, g, i, j, k - 1));
        const T p0 = lin(lP, g, i, j, k);
        const T lap = (lin(lP, g, i - 1, j, k) - 2 * p0 + lin(lP, g, i + 1, j, k)) / (dX * dX)
                    + (lin(lP, g, i, j - 1, k) - 2 * p0 + lin(lP, g, i, j + 1, k)) / (dY * dY)
                    + (lin(lP, g, i, j, k - 1) - 2 * p0 + lin(lP, g, i, j, k + 1)) / (dZ * dZ);
        lPhi[t] = lam + p0 - pc * lap;
        if (adj_inner(g, i, j, k) && p0 != T(0)) {
            const T ph = Phi[t];
            const T lf = (Phi[hix(g, i - 1, j, k)] - 2 * ph + Phi[hix(g, i + 1, j, k)]) / (dX * dX)
                       + (Phi[hix(g, i, j - 1, k)] - 2 * ph + Phi[hix(g, i, j + 1, k)]) / (dY * dY)
                       + (Phi[hix(g, i, j, k - 1)] - 2 * ph + Phi[hix(g, i, j, k + 1)]) / (dZ * dZ);
            gb = -c_beta * p0 * lf;
        }
    }
    block_atomic_add((double)gb, grad + 1);
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
    double dvol, dxn, dv;
    const T *Ua[3];          // forward Ua (halo, with boundary values)
    const double *Fc[3];     // forward marker forces
    const T *lQ[3];          // adjoint of the Helmholtz right-hand sides (interior)
    T *lUa[3];               // out: adjoint of Ua (full halo box, scattered)
    const double *w;         // drag weights of this step (ncyl x 3)
    double *grad;            // grad[3 + 2 l], grad[4 + 2 l]: cylinder centre
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
        const T dvn = T(a.dxn / a.dvol);    // dX^3 / (dX dY dZ)
        T wxs[3], wys[3], wzs[3], dwx[3], dwy[3];
        for (int q = 0; q < 3; ++q) {
            double x = (i0 + q - 0.5) * dX, y = (j0 + q - 0.5) * dY, z = (n - 1 + q - 0.5) * dZ;
            if (comp == 0) x = x + 0.5 * dX;
            else if (comp == 1) y = y + 0.5 * dY;
            else z = z + 0.5 * dZ;
            const T rx = T((x - xc) / dX), ry = T((y - yc) / dY), rz = T((z - zc) / dZ);
            wxs[q] = roma_t(rx);
            wys[q] = roma_t(ry);
            wzs[q] = roma_t(rz);
            dwx[q] = -droma_t(rx) / T(dX);   // d/dxc
            dwy[q] = -droma_t(ry) / T(dY);
        }
        // adjoint of Fc: drag weight + the folded spreading
        T lfc = T(-a.dv * a.w[3 * l + comp]);
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
                    lfc += lf * del * dvn;
                    gx += lf * fc * dvn * (dwx[ii] * wys[jj] * wzs[kk]);
                    gy += lf * fc * dvn * (wxs[ii] * dwy[jj] * wzs[kk]);
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
    T *lU, *lV, *lW, *lP;             // scattered adjoint of U^n, P^n (full halo box)
    T *lC0;                           // scattered adjoint of C0 = f C - I (6 x full halo box)
    int cs, ab2_first, polymer;
    T vis, coef_t, c_helm;            // beta/Re, (1-beta)/(Re Wi), dt/(2 Re)
    T inv_re;
    double *grad;
};

// per-thread accumulation of a stencil transpose: 9 positions per velocity
// component (offsets listed below), added with one atomic each
template <typename T>
struct Acc9 {
    T v[9];
    __device__ void zero() {
        for (int q = 0; q < 9; ++q) v[q] = T(0);
    }
};

template <typename T>
__global__ void __launch_bounds__(256) k_momentum_adj(MomAdjArgs<T> a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j <= g.ny;
    T gb = T(0);
    if (active) {
        const T dX = T(g.dx), dY = T(g.dy), dZ = T(g.dz), dt = T(g.dt);
        const T h2 = T(0.5), h15 = T(1.5);
        const T *U = a.U, *V = a.V, *W = a.W;
        auto u = [&](int x, int y, int z) { return U[hix(g, i + x, j + y, k + z)]; };
        auto v = [&](int x, int y, int z) { return V[hix(g, i + x, j + y, k + z)]; };
        auto w = [&](int x, int y, int z) { return W[hix(g, i + x, j + y, k + z)]; };
        const int o = qix(g, i, j, k), h = hix(g, i, j, k);
        T lua[3], lA[3], lT[3], lB[3];
        for (int c = 0; c < 3; ++c) {
            const T lq = a.lQ[c][h];
            lua[c] = lq + a.lUa[c][h];
            lA[c] = h15 * dt * lua[c] + a.lA0[c][o];
            lT[c] = h2 * dt * lua[c] + a.lT0[c][o];
            if (a.ab2_first) {
                lA[c] += -h2 * dt * lua[c];
                lT[c] += h2 * dt * lua[c];
                a.lA0[c][o] = T(0);
                a.lT0[c][o] = T(0);
            } else {
                a.lA0[c][o] = -h2 * dt * lua[c];
                a.lT0[c][o] = h2 * dt * lua[c];
            }
            lB[c] = dt * lua[c] - h2 * dt * lq;
            // Helmholtz coefficient dt beta/(2 Re): d/dbeta = (dt/2Re) lQ . L(Up)
            if (lq != T(0)) {
                const T *X = a.Up[c];
                const T x0 = X[h];
                const T L = (X[hix(g, i - 1, j, k)] - 2 * x0 + X[hix(g, i + 1, j, k)]) / (dX * dX)
                          + (X[hix(g, i, j - 1, k)] - 2 * x0 + X[hix(g, i, j + 1, k)]) / (dY * dY)
                          + (X[hix(g, i, j, k - 1)] - 2 * x0 + X[hix(g, i, j, k + 1)]) / (dZ * dZ);
                gb += a.c_helm * lq * L;
            }
        }
        // positions of the U, V, W transposes (offsets from (i, j, k))
        //   U: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (-1,1,0) 8 (-1,0,1)
        //   V: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (1,-1,0) 8 (0,-1,1)
        //   W: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (1,0,-1) 8 (0,1,-1)
        Acc9<T> aU, aV, aW;
        aU.zero(); aV.zero(); aW.zero();
        aU.v[0] += lua[0];
        aV.v[0] += lua[1];
        aW.v[0] += lua[2];
        // viscous terms B = vis lap(U) and d/dbeta (B/beta = lap/Re)
        {
            const T ib[3] = {T(1) / (dX * dX), T(1) / (dY * dY), T(1) / (dZ * dZ)};
            Acc9<T> *acc[3] = {&aU, &aV, &aW};
            const T *F[3] = {U, V, W};
            for (int c = 0; c < 3; ++c) {
                const T lb = a.vis * lB[c];
                Acc9<T> &A = *acc[c];
                A.v[1] += lb * ib[0]; A.v[2] += lb * ib[0];
                A.v[3] += lb * ib[1]; A.v[4] += lb * ib[1];
                A.v[5] += lb * ib[2]; A.v[6] += lb * ib[2];
                A.v[0] += T(-2) * lb * (ib[0] + ib[1] + ib[2]);
                const T *X = F[c];
                const T x0 = X[h];
                const T L = (X[hix(g, i - 1, j, k)] - 2 * x0 + X[hix(g, i + 1, j, k)]) / (dX * dX)
                          + (X[hix(g, i, j - 1, k)] - 2 * x0 + X[hix(g, i, j + 1, k)]) / (dY * dY)
                          + (X[hix(g, i, j, k - 1)] - 2 * x0 + X[hix(g, i, j, k + 1)]) / (dZ * dZ);
                gb += a.inv_re * lB[c] * L;
            }
        }
        // convection: A = -a.  a "square" term s (p1 + p2)^2/4 id and a "cross"
        // term s (a1 + a2)/2 (b1 + b2)/2 id; ga = adjoint of a
        {
            const T ga = -lA[0], gbv = -lA[1], gc = -lA[2];
            // ax
            {
                const T t1 = (u(-1, 0, 0) + u(0, 0, 0)) / 2, t2 = (u(0, 0, 0) + u(1, 0, 0)) / 2;
                aU.v[1] += ga * (-t1) / dX;
                aU.v[0] += ga * (-t1 + t2) / dX;
                aU.v[2] += ga * t2 / dX;
                // y: -(v(0,-1)+v(1,-1))/2 (u(0,-1)+u(0,0))/2 + (v(0,0)+v(1,0))/2 (u(0,0)+u(0,1))/2
                const T a1 = (v(0, -1, 0) + v(1, -1, 0)) / 2, b1 = (u(0, -1, 0) + u(0, 0, 0)) / 2;
                const T a2 = (v(0, 0, 0) + v(1, 0, 0)) / 2, b2 = (u(0, 0, 0) + u(0, 1, 0)) / 2;
                const T s = ga / dY;
                aV.v[3] += -s * b1 / 2; aV.v[7] += -s * b1 / 2;
                aU.v[3] += -s * a1 / 2; aU.v[0] += -s * a1 / 2;
                aV.v[0] += s * b2 / 2; aV.v[2] += s * b2 / 2;
                aU.v[0] += s * a2 / 2; aU.v[4] += s * a2 / 2;
                // z: -(w(0,0,-1)+w(1,0,-1))/2 (u(0,0,-1)+u)/2 + (w+w(1,0,0))/2 (u+u(0,0,1))/2
                const T c1 = (w(0, 0, -1) + w(1, 0, -1)) / 2, d1 = (u(0, 0, -1) + u(0, 0, 0)) / 2;
                const T c2 = (w(0, 0, 0) + w(1, 0, 0)) / 2, d2 = (u(0, 0, 0) + u(0, 0, 1)) / 2;
                const T sz = ga / dZ;
                aW.v[5] += -sz * d1 / 2; aW.v[7] += -sz * d1 / 2;
                aU.v[5] += -sz * c1 / 2; aU.v[0] += -sz * c1 / 2;
                aW.v[0] += sz * d2 / 2; aW.v[2] += sz * d2 / 2;
                aU.v[0] += sz * c2 / 2; aU.v[6] += sz * c2 / 2;
            }
            // ay
            {
                // x: -(u(-1,0)+u(-1,1))/2 (v(-1,0)+v)/2 + (u+u(0,1))/2 (v+v(1,0))/2
                const T a1 = (u(-1, 0, 0) + u(-1, 1, 0)) / 2, b1 = (v(-1, 0, 0) + v(0, 0, 0)) / 2;
                const T a2 = (u(0, 0, 0) + u(0, 1, 0)) / 2, b2 = (v(0, 0, 0) + v(1, 0, 0)) / 2;
                const T s = gbv / dX;
                aU.v[1] += -s * b1 / 2; aU.v[7] += -s * b1 / 2;
                aV.v[1] += -s * a1 / 2; aV.v[0] += -s * a1 / 2;
                aU.v[0] += s * b2 / 2; aU.v[4] += s * b2 / 2;
                aV.v[0] += s * a2 / 2; aV.v[2] += s * a2 / 2;
                const T t3 = (v(0, -1, 0) + v(0, 0, 0)) / 2, t4 = (v(0, 0, 0) + v(0, 1, 0)) / 2;
                aV.v[3] += gbv * (-t3) / dY;
                aV.v[0] += gbv * (-t3 + t4) / dY;
                aV.v[4] += gbv * t4 / dY;
                // z: -(w(0,0,-1)+w(0,1,-1))/2 (v(0,0,-1)+v)/2 + (w+w(0,1,0))/2 (v+v(0,0,1))/2
                const T c1 = (w(0, 0, -1) + w(0, 1, -1)) / 2, d1 = (v(0, 0, -1) + v(0, 0, 0)) / 2;
                const T c2 = (w(0, 0, 0) + w(0, 1, 0)) / 2, d2 = (v(0, 0, 0) + v(0, 0, 1)) / 2;
                const T sz = gbv / dZ;
                aW.v[5] += -sz * d1 / 2; aW.v[8] += -sz * d1 / 2;
                aV.v[5] += -sz * c1 / 2; aV.v[0] += -sz * c1 / 2;
                aW.v[0] += sz * d2 / 2; aW.v[4] += sz * d2 / 2;
                aV.v[0] += sz * c2 / 2; aV.v[6] += sz * c2 / 2;
            }
            // az
            {
                // x: -(u(-1,0,0)+u(-1,0,1))/2 (w(-1)+w)/2 + (u+u(0,0,1))/2 (w+w(1))/2
                const T a1 = (u(-1, 0, 0) + u(-1, 0, 1)) / 2, b1 = (w(-1, 0, 0) + w(0, 0, 0)) / 2;
                const T a2 = (u(0, 0, 0) + u(0, 0, 1)) / 2, b2 = (w(0, 0, 0) + w(1, 0, 0)) / 2;
                const T s = gc / dX;
                aU.v[1] += -s * b1 / 2; aU.v[8] += -s * b1 / 2;
                aW.v[1] += -s * a1 / 2; aW.v[0] += -s * a1 / 2;
                aU.v[0] += s * b2 / 2; aU.v[6] += s * b2 / 2;
                aW.v[0] += s * a2 / 2; aW.v[2] += s * a2 / 2;
                // y: -(v(0,-1,0)+v(0,-1,1))/2 (w(0,-1)+w)/2 + (v+v(0,0,1))/2 (w+w(0,1))/2
                const T c1 = (v(0, -1, 0) + v(0, -1, 1)) / 2, d1 = (w(0, -1, 0) + w(0, 0, 0)) / 2;
                const T c2 = (v(0, 0, 0) + v(0, 0, 1)) / 2, d2 = (w(0, 0, 0) + w(0, 1, 0)) / 2;
                const T sy = gc / dY;
                aV.v[3] += -sy * d1 / 2; aV.v[8] += -sy * d1 / 2;
                aW.v[3] += -sy * c1 / 2; aW.v[0] += -sy * c1 / 2;
                aV.v[0] += sy * d2 / 2; aV.v[6] += sy * d2 / 2;
                aW.v[0] += sy * c2 / 2; aW.v[4] += sy * c2 / 2;
                const T t5 = (w(0, 0, -1) + w(0, 0, 0)) / 2, t6 = (w(0, 0, 0) + w(0, 0, 1)) / 2;
                aW.v[5] += gc * (-t5) / dZ;
                aW.v[0] += gc * (-t5 + t6) / dZ;
                aW.v[6] += gc * t6 / dZ;
            }
        }
        {
            const int offU[9][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {-1, 1, 0}, {-1, 0, 1}};
            const int offV[9][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {1, -1, 0}, {0, -1, 1}};
            const int offW[9][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}, {1, 0, -1}, {0, 1, -1}};
            for (int q = 0; q < 9; ++q) {
                if (aU.v[q] != T(0)) atomicAdd(&a.lU[hix(g, i + offU[q][0], j + offU[q][1], k + offU[q][2])], aU.v[q]);
                if (aV.v[q] != T(0)) atomicAdd(&a.lV[hix(g, i + offV[q][0], j + offV[q][1], k + offV[q][2])], aV.v[q]);
                if (aW.v[q] != T(0)) atomicAdd(&a.lW[hix(g, i + offW[q][0], j + offW[q][1], k + offW[q][2])], aW.v[q]);
            }
        }
        // pressure gradient gp_c = -dt (P(o + e_c) - P(o)) / d_c
        {
            const T px = dt / dX * lua[0], py = dt / dY * lua[1], pz = dt / dZ * lua[2];
            atomicAdd(&a.lP[h], px + py + pz);
            atomicAdd(&a.lP[hix(g, i + 1, j, k)], -px);
            atomicAdd(&a.lP[hix(g, i, j + 1, k)], -py);
            atomicAdd(&a.lP[hix(g, i, j, k + 1)], -pz);
        }
        // polymer stress T = coef_t div(C0), C0 = f C - I (fenep.f90:645-691)
        if (a.polymer) {
            const T sx = a.coef_t * lT[0], sy = a.coef_t * lT[1], sz = a.coef_t * lT[2];
            T *L = a.lC0;
            const size_t cs = (size_t)a.cs;
            auto add = [&](int m, int x, int y, int z, T val) {
                atomicAdd(&L[(size_t)(m - 1) * cs + hix(g, i + x, j + y, k + z)], val);
            };
            // tx
            add(1, 0, 0, 0, -sx / dX); add(1, 1, 0, 0, sx / dX);
            add(2, 0, -1, 0, -sx / (4 * dY)); add(2, 1, -1, 0, -sx / (4 * dY));
            add(2, 0, 1, 0, sx / (4 * dY)); add(2, 1, 1, 0, sx / (4 * dY));
            add(3, 0, 0, -1, -sx / (4 * dZ)); add(3, 1, 0, -1, -sx / (4 * dZ));
            add(3, 0, 0, 1, sx / (4 * dZ)); add(3, 1, 0, 1, sx / (4 * dZ));
            // ty
            add(2, -1, 0, 0, -sy / (4 * dX)); add(2, 1, 0, 0, sy / (4 * dX));
            add(2, -1, 1, 0, -sy / (4 * dX)); add(2, 1, 1, 0, sy / (4 * dX));
            add(4, 0, 0, 0, -sy / dY); add(4, 0, 1, 0, sy / dY);
            add(5, 0, 0, -1, -sy / (4 * dZ)); add(5, 0, 1, -1, -sy / (4 * dZ));
            add(5, 0, 0, 1, sy / (4 * dZ)); add(5, 0, 1, 1, sy / (4 * dZ));
            // tz
            add(3, -1, 0, 0, -sz / (4 * dX)); add(3, 1, 0, 0, sz / (4 * dX));
            add(3, -1, 0, 1, -sz / (4 * dX)); add(3, 1, 0, 1, sz / (4 * dX));
            add(5, 0, -1, 0, -sz / (4 * dY)); add(5, 0, 1, 0, sz / (4 * dY));
            add(5, 0, -1, 1, -sz / (4 * dY)); add(5, 0, 1, 1, sz / (4 * dY));
            add(6, 0, 0, 0, -sz / dZ); add(6, 0, 0, 1, sz / dZ);
        }
    }
    block_atomic_add((double)gb, a.grad + 1);
}

// C0 = f(C) C - I on every cell (halo included), f = (L^2 - 3)/(L^2 - tr C):
// adds the adjoint of C^{n+1} and the L^2, beta, Wi terms (the stress
// coefficient (1-beta)/(Re Wi) enters through sum C0 . lC0).
template <typename T>
__global__ void k_c0_adj(const T *C, const T *lC0, T *lC, int cs, T lp2, T inv_1mb, T inv_wi, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    T g_coef = T(0), g_l2 = T(0);
    if (t < cs) {
        T c[6], l[6];
        bool any = false;
        for (int m = 0; m < 6; ++m) {
            l[m] = lC0[(size_t)m * cs + t];
            any = any || l[m] != T(0);
        }
        if (any) {
            const T E[6] = {T(1), T(0), T(0), T(1), T(0), T(1)};
            for (int m = 0; m < 6; ++m) c[m] = C[(size_t)m * cs + t];
            // tr C - 3 from the diagonal deviations (exact differences near
            // C = I), f - 1 = (tr C - 3)/(L^2 - tr C): the parameter terms
            // below then carry no cancellation of the O(1) parts
            const T tr3 = (c[0] - T(1)) + (c[3] - T(1)) + (c[5] - T(1));
            const T den = (lp2 - 3) - tr3;
            const T f = (lp2 - 3) / den;
            const T fm1 = tr3 / den;
            T lf = T(0);
            for (int m = 0; m < 6; ++m) {
                lC[(size_t)m * cs + t] += f * l[m];
                lf += c[m] * l[m];
                g_coef += (fm1 * c[m] + (c[m] - E[m])) * l[m];   // (f C - I) . lC0
            }
            const T dfdtr = f / den;
            lC[t] += lf * dfdtr;
            lC[(size_t)3 * cs + t] += lf * dfdtr;
            lC[(size_t)5 * cs + t] += lf * dfdtr;
            g_l2 = -lf * tr3 / (den * den);
        }
    }
    block_atomic_add((double)(-g_coef * inv_1mb), grad + 1);
    block_atomic_add((double)(-g_coef * inv_wi), grad + 0);
    block_atomic_add((double)g_l2, grad + 2);
}

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
    T *lC;                            // out: adjoint of C^n (full halo box, scattered)
    T *lU, *lV, *lW;
    int cs;
    T dt, wi, lp2;
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

// Rows: the cells of the polymer update (with walls also the ghost rows,
// whose faces towards the outside rows carry zero C)
template <typename T>
__global__ void __launch_bounds__(128) k_polymer_adj3(PolyAdjArgs<T> a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j < prow0(g) + prows(g);
    T gwi = T(0), gl2 = T(0);
    if (active) {
        const size_t cs = (size_t)a.cs;
        const int h = hix(g, i, j, k);
        const T dt = a.dt, wi = a.wi, lp2 = a.lp2, dX = T(g.dx), dY = T(g.dy), dZ = T(g.dz);
        T lx[6], x[6];
        bool any = false;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            lx[m] = a.lX[m * cs + h];
            x[m] = a.Cn[m * cs + h];
            any = any || lx[m] != T(0);
        }
        if (any) {
            const T *U = a.U, *V = a.V, *W = a.W;
            auto u = [&](int p, int q, int r) { return rowv(U, g, p, q, r); };
            auto v = [&](int p, int q, int r) { return rowv(V, g, p, q, r); };
            auto w = [&](int p, int q, int r) { return rowv(W, g, p, q, r); };
            T A0[3][3];
            A0[0][0] = -dt * (-u(i - 1, j, k) + u(i, j, k)) / dX;
            A0[0][1] = -dt * (-v(i - 1, j - 1, k) + v(i + 1, j - 1, k) - v(i - 1, j, k) + v(i + 1, j, k)) / (4 * dX);
            A0[0][2] = -dt * (-w(i - 1, j, k - 1) + w(i + 1, j, k - 1) - w(i - 1, j, k) + w(i + 1, j, k)) / (4 * dX);
            A0[1][0] = -dt * (-u(i - 1, j - 1, k) - u(i, j - 1, k) + u(i - 1, j + 1, k) + u(i, j + 1, k)) / (4 * dY);
            A0[1][1] = -dt * (-v(i, j - 1, k) + v(i, j, k)) / dY;
            A0[1][2] = -dt * (-w(i, j - 1, k - 1) + w(i, j + 1, k - 1) - w(i, j - 1, k) + w(i, j + 1, k)) / (4 * dY);
            A0[2][0] = -dt * (-u(i - 1, j, k - 1) - u(i, j, k - 1) + u(i - 1, j, k + 1) + u(i, j, k + 1)) / (4 * dZ);
            A0[2][1] = -dt * (-v(i, j - 1, k - 1) - v(i, j, k - 1) + v(i, j - 1, k + 1) + v(i, j, k + 1)) / (4 * dZ);
            A0[2][2] = -dt * (-w(i, j, k - 1) + w(i, j, k)) / dZ;
            // A = A0^T (the matrix the Newton solve uses)
            T A[3][3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) A[r][q] = A0[q][r];
            // tr C - 3 from the diagonal deviations and f - 1 = (tr C - 3)/den,
            // so that the parameter terms carry no cancellation of O(1) parts
            const T tr3 = (x[0] - T(1)) + (x[3] - T(1)) + (x[5] - T(1));
            const T den = (lp2 - 3) - tr3;
            const T f = (lp2 - 3) / den;
            const T fm1 = tr3 / den;
            const T dd2 = T(1) + f * dt / wi;
            const T cf = dt / wi * f / den;    // (dt/Wi) df/dx_d, d in {0, 3, 5}
            // M = J^T, augmented with the right-hand side lx
            T M[6][7];
            {
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
#pragma unroll
                for (int r = 0; r < 6; ++r) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) M[r][q] = J[q][r];
                    M[r][6] = lx[r];
                }
            }
            // Gaussian elimination with partial pivoting.  The pivot row is found
            // by compare-and-exchange with each lower row (a running maximum),
            // so every index is a compile-time constant and M stays in registers.
#pragma unroll
            for (int c = 0; c < 6; ++c) {
#pragma unroll
                for (int r = c + 1; r < 6; ++r) {
                    const bool sw = fabs(M[r][c]) > fabs(M[c][c]);
#pragma unroll
                    for (int q = c; q < 7; ++q) {
                        const T u0 = M[c][q], u1 = M[r][q];
                        M[c][q] = sw ? u1 : u0;
                        M[r][q] = sw ? u0 : u1;
                    }
                }
                const T inv = T(1) / M[c][c];
#pragma unroll
                for (int r = c + 1; r < 6; ++r) {
                    const T fr = M[r][c] * inv;
#pragma unroll
                    for (int q = c; q < 7; ++q) M[r][q] -= fr * M[c][q];
                }
            }
            T mu[6];
#pragma unroll
            for (int r = 5; r >= 0; --r) {
                T s = M[r][6];
#pragma unroll
                for (int q = r + 1; q < 6; ++q) s -= M[r][q] * mu[q];
                mu[r] = s / M[r][r];
            }
            // parameters: G = L(x) + (1 + f dt/Wi) x - b, b includes dt/Wi on
            // the diagonal: dG/dWi = -dt/Wi^2 (f x - I), formed as
            // (f - 1) x + (x - I); dG/dL^2 = dt/Wi df/dL^2 x
            T mx = T(0), mxe = T(0);
            const T E[6] = {T(1), T(0), T(0), T(1), T(0), T(1)};
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                mx += mu[m] * x[m];
                mxe += mu[m] * (x[m] - E[m]);
            }
            gwi = dt / (wi * wi) * (fm1 * mx + mxe);
            gl2 = dt / wi * tr3 / (den * den) * mx;
            // adjoint of A = A0^T, then of the velocity-gradient stencils
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
            // scatters to rows beyond the ghost rows are dropped (constant zeros)
            auto inrow = [&](int q) { return q >= 0 && q <= g.ny + 1; };
            auto addu = [&](int p, int q, int r, T val) { if (inrow(q)) atomicAdd(&a.lU[hix(g, p, q, r)], val); };
            auto addv = [&](int p, int q, int r, T val) { if (inrow(q)) atomicAdd(&a.lV[hix(g, p, q, r)], val); };
            auto addw = [&](int p, int q, int r, T val) { if (inrow(q)) atomicAdd(&a.lW[hix(g, p, q, r)], val); };
            {
                T l = lAt[0][0] * dt / dX;   // A0[0][0]
                addu(i - 1, j, k, l); addu(i, j, k, -l);
                l = lAt[1][0] * dt / (4 * dX);    // A0[0][1]
                addv(i - 1, j - 1, k, l); addv(i + 1, j - 1, k, -l); addv(i - 1, j, k, l); addv(i + 1, j, k, -l);
                l = lAt[2][0] * dt / (4 * dX);    // A0[0][2]
                addw(i - 1, j, k - 1, l); addw(i + 1, j, k - 1, -l); addw(i - 1, j, k, l); addw(i + 1, j, k, -l);
                l = lAt[0][1] * dt / (4 * dY);    // A0[1][0]
                addu(i - 1, j - 1, k, l); addu(i, j - 1, k, l); addu(i - 1, j + 1, k, -l); addu(i, j + 1, k, -l);
                l = lAt[1][1] * dt / dY;          // A0[1][1]
                addv(i, j - 1, k, l); addv(i, j, k, -l);
                l = lAt[2][1] * dt / (4 * dY);    // A0[1][2]
                addw(i, j - 1, k - 1, l); addw(i, j + 1, k - 1, -l); addw(i, j - 1, k, l); addw(i, j + 1, k, -l);
                l = lAt[0][2] * dt / (4 * dZ);    // A0[2][0]
                addu(i - 1, j, k - 1, l); addu(i, j, k - 1, l); addu(i - 1, j, k + 1, -l); addu(i, j, k + 1, -l);
                l = lAt[1][2] * dt / (4 * dZ);    // A0[2][1]
                addv(i, j - 1, k - 1, l); addv(i, j, k - 1, l); addv(i, j - 1, k + 1, -l); addv(i, j, k + 1, -l);
                l = lAt[2][2] * dt / dZ;          // A0[2][2]
                addw(i, j, k - 1, l); addw(i, j, k, -l);
            }
            // Cstar: b = s3 pxm + s1 pxp + s4 nxm + s2 nxp + (y: s7 s5 s8 s6) + (z: s11 s9 s12 s10)
            const T u1 = U[hix(g, i - 1, j, k)], u2 = U[h];
            const T v1 = rowv(V, g, i, j - 1, k), v2 = V[h];
            const T w1 = W[hix(g, i, j, k - 1)], w2 = W[h];
            const T sixth = T(1) / T(6);
            T s[13];
            s[1] = (-u2 + fabs(u2)) * dt / (2 * dX);
            s[2] = sixth + (-u2 - fabs(u2)) * dt / (2 * dX);
            s[3] = sixth + (u1 - fabs(u1)) * dt / (2 * dX);
            s[4] = (u1 + fabs(u1)) * dt / (2 * dX);
            s[5] = (-v2 + fabs(v2)) * dt / (2 * dY);
            s[6] = sixth + (-v2 - fabs(v2)) * dt / (2 * dY);
            s[7] = sixth + (v1 - fabs(v1)) * dt / (2 * dY);
            s[8] = (v1 + fabs(v1)) * dt / (2 * dY);
            s[9] = (-w2 + fabs(w2)) * dt / (2 * dZ);
            s[10] = sixth + (-w2 - fabs(w2)) * dt / (2 * dZ);
            s[11] = sixth + (w1 - fabs(w1)) * dt / (2 * dZ);
            s[12] = (w1 + fabs(w1)) * dt / (2 * dZ);
            T ls[13];
#pragma unroll
            for (int q = 0; q < 13; ++q) ls[q] = T(0);
            // selection codes (as the forward kernel reads them)
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
            const int hxm = hix(g, wrapx(g, i - 1), j, k), hxp = hix(g, wrapx(g, i + 1), j, k);
            const int hym = g.walls ? h : hix(g, i, jm, k), hyp = g.walls ? h : hix(g, i, jp, k);
            const int hzm = hix(g, i, j, wrapz(g, k - 1)), hzp = hix(g, i, j, wrapz(g, k + 1));
            const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
            // face weights of the cell's own faces and of the neighbours' faces,
            // by selection code
            const W3<T> wpx = wface_p<T>(isx), wnx = wface_n<T>(isx), wpy = wface_p<T>(isy), wny = wface_n<T>(isy);
            const W3<T> wpz = wface_p<T>(isz), wnz = wface_n<T>(isz);
            const W3<T> qx = wface_p<T>(cxp + 1), rx = wface_n<T>(cxm + 1), qy = wface_p<T>(cyp + 1), ry = wface_n<T>(cym + 1);
            const W3<T> qz = wface_p<T>(czp + 1), rz = wface_n<T>(czm + 1);
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                const T *Cm = a.C + m * cs;
                T *Lm = a.lC + m * cs;
                const T mum = mu[m];
                T lc0 = T(0);   // accumulated weight at the cell itself
                // one direction: own faces (code is, coefficients sp on the p face, sn on the n face),
                // the + neighbour's p face (code cp_, coefficient sq), the - neighbour's n face (code cm_, sr)
                auto dir = [&](W3<T> wp_, W3<T> wn_, int off, int hp, W3<T> wq, int hm, W3<T> wr, T sp, T sn,
                               T sq, T sr, T &lsp, T &lsn, T &lsq, T &lsr) {
                    const T cmv = Cm[h - off], c0v = Cm[h], cpv = Cm[h + off];
                    lsp += mum * (wp_.m * cmv + wp_.c * c0v + wp_.p * cpv);
                    lsn += mum * (wn_.m * cmv + wn_.c * c0v + wn_.p * cpv);
                    const T am = mum * (sp * wp_.m + sn * wn_.m);
                    const T ap = mum * (sp * wp_.p + sn * wn_.p);
                    lc0 += mum * (sp * wp_.c + sn * wn_.c);
                    if (am != T(0)) atomicAdd(&Lm[h - off], am);
                    if (ap != T(0)) atomicAdd(&Lm[h + off], ap);
                    // + neighbour's p face
                    lsq += mum * (wq.m * Cm[hp - off] + wq.c * Cm[hp] + wq.p * Cm[hp + off]);
                    {
                        const T b = mum * sq;
                        if (b != T(0)) {
                            if (wq.m != T(0)) atomicAdd(&Lm[hp - off], b * wq.m);
                            atomicAdd(&Lm[hp], b * wq.c);
                            if (wq.p != T(0)) atomicAdd(&Lm[hp + off], b * wq.p);
                        }
                    }
                    // - neighbour's n face
                    lsr += mum * (wr.m * Cm[hm - off] + wr.c * Cm[hm] + wr.p * Cm[hm + off]);
                    {
                        const T b = mum * sr;
                        if (b != T(0)) {
                            if (wr.m != T(0)) atomicAdd(&Lm[hm - off], b * wr.m);
                            atomicAdd(&Lm[hm], b * wr.c);
                            if (wr.p != T(0)) atomicAdd(&Lm[hm + off], b * wr.p);
                        }
                    }
                };
                // x: pxm (s3, own p), nxp (s2, own n), pxp (s1, neighbour i+1), nxm (s4, neighbour i-1)
                dir(wpx, wnx, ox, hxp, qx, hxm, rx, s[3], s[2], s[1], s[4], ls[3], ls[2], ls[1], ls[4]);
                if (!g.walls) {
                    dir(wpy, wny, oy, hyp, qy, hym, ry, s[7], s[6], s[5], s[8], ls[7], ls[6], ls[5], ls[8]);
                } else {
                    // rows j-2 .. j+2 of the column, zero beyond the ghost rows
                    auto yv = [&](int jj) { return rowv(Cm, g, i, jj, k); };
                    auto yadd = [&](int jj, T val) {
                        if (val != T(0) && jj >= 0 && jj <= g.ny + 1) atomicAdd(&Lm[hix(g, i, jj, k)], val);
                    };
                    const T cmv = yv(j - 1), c0v = Cm[h], cpv = yv(j + 1);
                    ls[7] += mum * (wpy.m * cmv + wpy.c * c0v + wpy.p * cpv);
                    ls[6] += mum * (wny.m * cmv + wny.c * c0v + wny.p * cpv);
                    yadd(j - 1, mum * (s[7] * wpy.m + s[6] * wny.m));
                    yadd(j + 1, mum * (s[7] * wpy.p + s[6] * wny.p));
                    lc0 += mum * (s[7] * wpy.c + s[6] * wny.c);
                    // the p face of cell j+1 (rows j .. j+2), the n face of cell j-1 (rows j-2 .. j)
                    ls[5] += mum * (qy.m * c0v + qy.c * cpv + qy.p * yv(j + 2));
                    const T bq = mum * s[5];
                    lc0 += bq * qy.m;
                    yadd(j + 1, bq * qy.c);
                    yadd(j + 2, bq * qy.p);
                    ls[8] += mum * (ry.m * yv(j - 2) + ry.c * cmv + ry.p * c0v);
                    const T br = mum * s[8];
                    yadd(j - 2, br * ry.m);
                    yadd(j - 1, br * ry.c);
                    lc0 += br * ry.p;
                }
                dir(wpz, wnz, oz, hzp, qz, hzm, rz, s[11], s[10], s[9], s[12], ls[11], ls[10], ls[9], ls[12]);
                atomicAdd(&Lm[h], lc0);
            }
            // s coefficients -> velocities
            {
                const T cx = dt / (2 * dX), cy = dt / (2 * dY), cz = dt / (2 * dZ);
                const T su2 = sgn(u2), su1 = sgn(u1), sv2 = sgn(v2), sv1 = sgn(v1), sw2 = sgn(w2), sw1 = sgn(w1);
                addu(i, j, k, (ls[1] * (T(-1) + su2) + ls[2] * (T(-1) - su2)) * cx);
                addu(i - 1, j, k, (ls[3] * (T(1) - su1) + ls[4] * (T(1) + su1)) * cx);
                addv(i, j, k, (ls[5] * (T(-1) + sv2) + ls[6] * (T(-1) - sv2)) * cy);
                addv(i, j - 1, k, (ls[7] * (T(1) - sv1) + ls[8] * (T(1) + sv1)) * cy);
                addw(i, j, k, (ls[9] * (T(-1) + sw2) + ls[10] * (T(-1) - sw2)) * cz);
                addw(i, j, k - 1, (ls[11] * (T(1) - sw1) + ls[12] * (T(1) + sw1)) * cz);
            }
        }
    }
    block_atomic_add((double)gwi, a.grad + 0);
    block_atomic_add((double)gl2, a.grad + 2);
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
