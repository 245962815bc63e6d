// f8_adjoint.cu — discrete adjoint of the FP64 3D step (the gradient of f8_grad).
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
// Stencil transposes scatter with FP64 atomics into full halo arrays, so the
// adjoint fields are reproducible to round-off, not bit for bit.
#include <algorithm>
#include <cstdio>
#include <initializer_list>
#include <utility>
#include "f8_common.cuh"
#include "f8_kernels.h"

namespace f8 {

namespace {

__device__ inline bool inner(const Geo &g, int i, int j, int k) {
    return i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz;
}

// value of an adjoint field at (i, j, k) if that cell is interior, else 0
__device__ inline double lin(const double *A, const Geo &g, int i, int j, int k) {
    return inner(g, i, j, k) ? A[hix(g, i, j, k)] : 0.0;
}

__device__ inline double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// Block sum of v added to *dst (every thread of the block calls it).
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

struct FoldSet {
    double *A[8];
    int kind[8];
    int n;
};

__global__ void k_fold_z(FoldSet f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.sy) return;
    const int i = t % g.sx, j = t / g.sx;
    const int lo = hix(g, i, j, 0), hi = hix(g, i, j, g.sz - 1), top = hix(g, i, j, g.nz), bot = hix(g, i, j, 1);
    for (int q = 0; q < f.n; ++q) {
        double *A = f.A[q];
        const double a = A[lo], b = A[hi];
        A[top] += a;
        A[bot] += b;
        A[lo] = 0.0;
        A[hi] = 0.0;
    }
}

__global__ void k_fold_y(FoldSet f, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.sx * g.nz) return;
    const int i = t % g.sx, k = 1 + t / g.sx;
    const int g0 = hix(g, i, 0, k), g1 = hix(g, i, g.ny + 1, k), r1 = hix(g, i, 1, k), rn = hix(g, i, g.ny, k);
    for (int q = 0; q < f.n; ++q) {
        double *A = f.A[q];
        const double a = A[g0], b = A[g1];
        if (!g.walls) {
            A[rn] += a;
            A[r1] += b;
        } else {
            switch (f.kind[q]) {
            case BC_U:
            case BC_W: A[r1] -= a; A[rn] -= b; break;     // ghost = -U (2 Uwall - U)
            case BC_V: A[rn] = 0.0; break;                // V(:,0) = V(:,NY) = V(:,NY+1) = 0
            case BC_P: A[r1] += a; A[rn] += b; break;     // Neumann copies
            default:                                      // C: 2 C(1) - C(2), 2 C(NY) - C(NY-1)
                A[r1] += 2.0 * a; A[hix(g, i, 2, k)] -= a;
                A[rn] += 2.0 * b; A[hix(g, i, g.ny - 1, k)] -= b;
            }
        }
        A[g0] = 0.0;
        A[g1] = 0.0;
    }
}

// rows: 1..NY, or every row 0..NY+1 (rows_all) for the periodic x/z fill of
// the updated wall ghost rows
__global__ void k_fold_x(FoldSet f, Geo g, int rows_all) {
    const int ny = rows_all ? g.sy : g.ny, j0 = rows_all ? 0 : 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ny * g.nz) return;
    const int j = j0 + t % ny, k = 1 + t / ny;
    const int lo = hix(g, 0, j, k), hi = hix(g, g.sx - 1, j, k);
    for (int q = 0; q < f.n; ++q) {
        double *A = f.A[q];
        const double a = A[lo], b = A[hi];
        A[hix(g, g.nx, j, k)] += a;
        A[hix(g, 1, j, k)] += b;
        A[lo] = 0.0;
        A[hi] = 0.0;
    }
}

cudaError_t fold(const FoldSet &f, const Geo &g, cudaStream_t s) {
    k_fold_z<<<(g.sx * g.sy + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_y<<<(g.sx * g.nz + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_x<<<(g.ny * g.nz + 255) / 256, 256, 0, s>>>(f, g, 0); count_launch();
    return cudaGetLastError();
}

// transpose of the periodic x and z copies of every row (k_bc_c_pet_xz): the
// wall ghost rows stay (they are updated cells)
cudaError_t fold_xz(const FoldSet &f, const Geo &g, cudaStream_t s) {
    k_fold_z<<<(g.sx * g.sy + 255) / 256, 256, 0, s>>>(f, g); count_launch();
    k_fold_x<<<(g.sy * g.nz + 255) / 256, 256, 0, s>>>(f, g, 1); count_launch();
    return cudaGetLastError();
}

FoldSet fold_set(std::initializer_list<std::pair<double *, int>> fields) {
    FoldSet f{};
    for (auto &p : fields) { f.A[f.n] = p.first; f.kind[f.n] = p.second; ++f.n; }
    return f;
}

FoldSet fold_c(double *C, int cs) {
    FoldSet f{};
    for (int m = 0; m < 6; ++m) { f.A[m] = C + (size_t)m * cs; f.kind[m] = BC_C; }
    f.n = 6;
    return f;
}

// ---------------------------------------------------------------------------
// Projection and pressure update:  U = Up - dt dPhi/dx ..., P += Phi - pc lap Phi.
// One thread per cell of the full halo box gathers the adjoint of Phi there.

__global__ void k_march_adj(const double *lU, const double *lV, const double *lW, const double *lP, double *lPhi,
                            const double *Phi, Geo g, double pc, double c_beta, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    double gb = 0.0;
    if (t < cs) {
        const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
        const double dt = g.dt, dX = g.dx, dY = g.dy, dZ = g.dz;
        double lam = dt / dX * (lin(lU, g, i, j, k) - lin(lU, g, i - 1, j, k))
                   + dt / dY * (lin(lV, g, i, j, k) - lin(lV, g, i, j - 1, k))
                   + dt / dZ * (lin(lW, g, i, j, k) - lin(lW, g, i, j, k - 1));
        const double p0 = lin(lP, g, i, j, k);
        const double lap = (lin(lP, g, i - 1, j, k) - 2 * p0 + lin(lP, g, i + 1, j, k)) / (dX * dX)
                         + (lin(lP, g, i, j - 1, k) - 2 * p0 + lin(lP, g, i, j + 1, k)) / (dY * dY)
                         + (lin(lP, g, i, j, k - 1) - 2 * p0 + lin(lP, g, i, j, k + 1)) / (dZ * dZ);
        lPhi[t] = lam + p0 - pc * lap;
        if (inner(g, i, j, k) && p0 != 0.0) {
            const double ph = Phi[t];
            const double lf = (Phi[hix(g, i - 1, j, k)] - 2 * ph + Phi[hix(g, i + 1, j, k)]) / (dX * dX)
                            + (Phi[hix(g, i, j - 1, k)] - 2 * ph + Phi[hix(g, i, j + 1, k)]) / (dY * dY)
                            + (Phi[hix(g, i, j, k - 1)] - 2 * ph + Phi[hix(g, i, j, k + 1)]) / (dZ * dZ);
            gb = -c_beta * p0 * lf;
        }
    }
    block_atomic_add(gb, grad + 1);
}

// interior of a halo field -> packed interior array
__global__ void k_pack(const double *A, double *out, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    out[qix(g, i, j, k)] = A[hix(g, i, j, k)];
}

// Divergence right-hand side q = div(Up)/dt (fenep.f90:1547-1555) transposed,
// plus the identity part U = Up + ... of the projection; full halo box.
__global__ void k_div_adj(const double *lU, const double *lV, const double *lW, const double *lq, double *lUp,
                          double *lVp, double *lWp, Geo g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    const double dt = g.dt;
    const double q0 = lin(lq, g, i, j, k);
    lUp[t] = lin(lU, g, i, j, k) + (q0 - lin(lq, g, i + 1, j, k)) / g.dx / dt;
    lVp[t] = lin(lV, g, i, j, k) + (q0 - lin(lq, g, i, j + 1, k)) / g.dy / dt;
    lWp[t] = lin(lW, g, i, j, k) + (q0 - lin(lq, g, i, j, k + 1)) / g.dz / dt;
}

// ---------------------------------------------------------------------------
// IBM.  Roma kernel (fenep.f90:2045-2055) and its derivative.

__device__ inline double roma(double r) {
    double ar = fabs(r);
    if (ar < 1.5 && ar >= 0.5) return (5.0 - 3.0 * ar - sqrt(-3.0 * ((1 - ar) * (1 - ar)) + 1.0)) / 6.0;
    if (ar < 0.5) return (1.0 + sqrt(-3.0 * (r * r) + 1.0)) / 3.0;
    return 0.0;
}

__device__ inline double droma(double r) {
    const double ar = fabs(r);
    if (ar < 0.5) return -r / sqrt(1.0 - 3.0 * r * r);
    if (ar < 1.5) {
        const double s = 1.0 - ar;
        return sgn(r) * (-3.0 - 3.0 * s / sqrt(1.0 - 3.0 * s * s)) / 6.0;
    }
    return 0.0;
}

constexpr int MAX_CYL_SHARED = 64;

struct IbmAdjArgs {
    const double *mx, *my;
    const int *mcyl;
    int nm, ncyl;
    double dvol, dxn, dv;
    const double *Ua[3];     // forward Ua (halo, with boundary values)
    const double *Fc[3];     // forward marker forces
    const double *lQ[3];     // adjoint of the Helmholtz right-hand sides (interior)
    double *lUa[3];          // out: adjoint of Ua (full halo box, scattered)
    const double *w;         // drag weights of this step (ncyl x 3)
    double *grad;            // grad[3 + 2 l], grad[4 + 2 l]: cylinder centre
};

// One thread per (marker, plane, component).  Forward: Ub = sum Ua delta dX^3,
// Fc = (Uc - Ub)/dt, drag = -dv sum Fc, f = fold(sum Fc delta dX^3),
// Q = Ua + dt f - dt B/2.
__global__ void k_ibm_adj(IbmAdjArgs a, Geo g) {
    __shared__ double gc[2 * MAX_CYL_SHARED];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y + 1;
    const int comp = blockIdx.z;
    const bool use_sh = a.ncyl <= MAX_CYL_SHARED;
    for (int q = threadIdx.x; q < 2 * MAX_CYL_SHARED; q += blockDim.x) gc[q] = 0.0;
    __syncthreads();
    if (m < a.nm) {
        const double dX = g.dx, dY = g.dy, dZ = g.dz, dt = g.dt;
        const double xc = a.mx[m], yc = a.my[m], zc = (n - 0.25) * dZ;
        int i0, j0;
        if (comp == 0) { j0 = (int)(yc / dY); i0 = (int)(xc / dX - 0.5); }
        else if (comp == 1) { j0 = (int)(yc / dY - 0.5); i0 = (int)(xc / dX); }
        else { j0 = (int)(yc / dY); i0 = (int)(xc / dX); }
        const int l = a.mcyl[m];
        const size_t fo = (size_t)m + (size_t)a.nm * (n - 1);
        const double fc = a.Fc[comp][fo];
        const double *lQ = a.lQ[comp];
        const double *Ua = a.Ua[comp];
        double wxs[3], wys[3], wzs[3], dwx[3], dwy[3];
        for (int q = 0; q < 3; ++q) {
            double x = (i0 + q - 0.5) * dX, y = (j0 + q - 0.5) * dY, z = (n - 1 + q - 0.5) * dZ;
            if (comp == 0) x = x + 0.5 * dX;
            else if (comp == 1) y = y + 0.5 * dY;
            else z = z + 0.5 * dZ;
            wxs[q] = roma((x - xc) / dX);
            wys[q] = roma((y - yc) / dY);
            wzs[q] = roma((z - zc) / dZ);
            dwx[q] = -droma((x - xc) / dX) / dX;   // d/dxc
            dwy[q] = -droma((y - yc) / dY) / dY;
        }
        // adjoint of Fc: drag weight + the folded spreading
        double lfc = -a.dv * a.w[3 * l + comp];
        double gx = 0.0, gy = 0.0;
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
                    const double lf = drop ? 0.0 : dt * lQ[hix(g, fi, fj, fk)];
                    const double del = wxs[ii] * wys[jj] * wzs[kk] / a.dvol;
                    lfc += lf * del * a.dxn;
                    gx += lf * fc * a.dxn * (dwx[ii] * wys[jj] * wzs[kk] / a.dvol);
                    gy += lf * fc * a.dxn * (wxs[ii] * dwy[jj] * wzs[kk] / a.dvol);
                }
            }
        }
        const double lub = -lfc / dt;
        double *lUa = a.lUa[comp];
        for (int kk = 0; kk < 3; ++kk) {
            const int k = n - 1 + kk;
            for (int jj = 0; jj < 3; ++jj) {
                const int j = j0 + jj;
                for (int ii = 0; ii < 3; ++ii) {
                    const int i = i0 + ii;
                    const int h = hix(g, i, j, k);
                    const double del = wxs[ii] * wys[jj] * wzs[kk] / a.dvol;
                    atomicAdd(&lUa[h], lub * del * a.dxn);
                    const double u = Ua[h];
                    gx += lub * u * a.dxn * (dwx[ii] * wys[jj] * wzs[kk] / a.dvol);
                    gy += lub * u * a.dxn * (wxs[ii] * dwy[jj] * wzs[kk] / a.dvol);
                }
            }
        }
        if (use_sh) {
            atomicAdd(&gc[2 * l], gx);
            atomicAdd(&gc[2 * l + 1], gy);
        } else {
            atomicAdd(&a.grad[3 + 2 * l], gx);
            atomicAdd(&a.grad[4 + 2 * l], gy);
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

struct MomAdjArgs {
    const double *U, *V, *W;          // forward U^n (halo)
    const double *Up[3];              // forward Helmholtz solutions (halo)
    const double *lQ[3];              // adjoint of Q (interior of halo arrays)
    const double *lUa[3];             // adjoint of Ua from the interpolation (interior)
    double *lA0[3], *lT0[3];          // in: adjoint of the new history; out: of the old
    double *lU, *lV, *lW, *lP;        // scattered adjoint of U^n, P^n (full halo box)
    double *lC0;                      // scattered adjoint of C0 = f C - I (6 x full halo box)
    int cs, ab2_first, polymer;
    double vis, coef_t, c_helm;       // beta/Re, (1-beta)/(Re Wi), dt/(2 Re)
    double inv_re;
    double *grad;
};

// per-thread accumulation of a stencil transpose: 9 positions per velocity
// component (offsets listed below), added with one atomic each
struct Acc9 {
    double v[9];
    __device__ void zero() {
        for (int q = 0; q < 9; ++q) v[q] = 0.0;
    }
};

__global__ void __launch_bounds__(256) k_momentum_adj(MomAdjArgs a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j <= g.ny;
    double gb = 0.0;
    if (active) {
        const double dX = g.dx, dY = g.dy, dZ = g.dz, dt = g.dt;
        const double *U = a.U, *V = a.V, *W = a.W;
        auto u = [&](int x, int y, int z) { return U[hix(g, i + x, j + y, k + z)]; };
        auto v = [&](int x, int y, int z) { return V[hix(g, i + x, j + y, k + z)]; };
        auto w = [&](int x, int y, int z) { return W[hix(g, i + x, j + y, k + z)]; };
        const int o = qix(g, i, j, k), h = hix(g, i, j, k);
        double lua[3], lA[3], lT[3], lB[3];
        for (int c = 0; c < 3; ++c) {
            const double lq = a.lQ[c][h];
            lua[c] = lq + a.lUa[c][h];
            lA[c] = 1.5 * dt * lua[c] + a.lA0[c][o];
            lT[c] = 0.5 * dt * lua[c] + a.lT0[c][o];
            if (a.ab2_first) {
                lA[c] += -0.5 * dt * lua[c];
                lT[c] += 0.5 * dt * lua[c];
                a.lA0[c][o] = 0.0;
                a.lT0[c][o] = 0.0;
            } else {
                a.lA0[c][o] = -0.5 * dt * lua[c];
                a.lT0[c][o] = 0.5 * dt * lua[c];
            }
            lB[c] = dt * lua[c] - 0.5 * dt * lq;
            // Helmholtz coefficient dt beta/(2 Re): d/dbeta = (dt/2Re) lQ . L(Up)
            if (lq != 0.0) {
                const double *X = a.Up[c];
                const double x0 = X[h];
                const double L = (X[hix(g, i - 1, j, k)] - 2 * x0 + X[hix(g, i + 1, j, k)]) / (dX * dX)
                               + (X[hix(g, i, j - 1, k)] - 2 * x0 + X[hix(g, i, j + 1, k)]) / (dY * dY)
                               + (X[hix(g, i, j, k - 1)] - 2 * x0 + X[hix(g, i, j, k + 1)]) / (dZ * dZ);
                gb += a.c_helm * lq * L;
            }
        }
        // positions of the U, V, W transposes (offsets from (i, j, k))
        //   U: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (-1,1,0) 8 (-1,0,1)
        //   V: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (1,-1,0) 8 (0,-1,1)
        //   W: 0 (0,0,0) 1 (-1,0,0) 2 (1,0,0) 3 (0,-1,0) 4 (0,1,0) 5 (0,0,-1) 6 (0,0,1) 7 (1,0,-1) 8 (0,1,-1)
        Acc9 aU, aV, aW;
        aU.zero(); aV.zero(); aW.zero();
        aU.v[0] += lua[0];
        aV.v[0] += lua[1];
        aW.v[0] += lua[2];
        // viscous terms B = vis lap(U) and d/dbeta (B/beta = lap/Re)
        {
            const double ib[3] = {1.0 / (dX * dX), 1.0 / (dY * dY), 1.0 / (dZ * dZ)};
            Acc9 *acc[3] = {&aU, &aV, &aW};
            const double *F[3] = {U, V, W};
            for (int c = 0; c < 3; ++c) {
                const double lb = a.vis * lB[c];
                Acc9 &A = *acc[c];
                A.v[1] += lb * ib[0]; A.v[2] += lb * ib[0];
                A.v[3] += lb * ib[1]; A.v[4] += lb * ib[1];
                A.v[5] += lb * ib[2]; A.v[6] += lb * ib[2];
                A.v[0] += -2.0 * lb * (ib[0] + ib[1] + ib[2]);
                const double *X = F[c];
                const double x0 = X[h];
                const double L = (X[hix(g, i - 1, j, k)] - 2 * x0 + X[hix(g, i + 1, j, k)]) / (dX * dX)
                               + (X[hix(g, i, j - 1, k)] - 2 * x0 + X[hix(g, i, j + 1, k)]) / (dY * dY)
                               + (X[hix(g, i, j, k - 1)] - 2 * x0 + X[hix(g, i, j, k + 1)]) / (dZ * dZ);
                gb += a.inv_re * lB[c] * L;
            }
        }
        // convection: A = -a.  a "square" term s (p1 + p2)^2/4 id and a "cross"
        // term s (a1 + a2)/2 (b1 + b2)/2 id; ga = adjoint of a
        {
            const double ga = -lA[0], gbv = -lA[1], gc = -lA[2];
            // ax
            {
                const double t1 = (u(-1, 0, 0) + u(0, 0, 0)) / 2, t2 = (u(0, 0, 0) + u(1, 0, 0)) / 2;
                aU.v[1] += ga * (-t1) / dX;
                aU.v[0] += ga * (-t1 + t2) / dX;
                aU.v[2] += ga * t2 / dX;
                // y: -(v(0,-1)+v(1,-1))/2 (u(0,-1)+u(0,0))/2 + (v(0,0)+v(1,0))/2 (u(0,0)+u(0,1))/2
                const double a1 = (v(0, -1, 0) + v(1, -1, 0)) / 2, b1 = (u(0, -1, 0) + u(0, 0, 0)) / 2;
                const double a2 = (v(0, 0, 0) + v(1, 0, 0)) / 2, b2 = (u(0, 0, 0) + u(0, 1, 0)) / 2;
                const double s = ga / dY;
                aV.v[3] += -s * b1 / 2; aV.v[7] += -s * b1 / 2;
                aU.v[3] += -s * a1 / 2; aU.v[0] += -s * a1 / 2;
                aV.v[0] += s * b2 / 2; aV.v[2] += s * b2 / 2;
                aU.v[0] += s * a2 / 2; aU.v[4] += s * a2 / 2;
                // z: -(w(0,0,-1)+w(1,0,-1))/2 (u(0,0,-1)+u)/2 + (w+w(1,0,0))/2 (u+u(0,0,1))/2
                const double c1 = (w(0, 0, -1) + w(1, 0, -1)) / 2, d1 = (u(0, 0, -1) + u(0, 0, 0)) / 2;
                const double c2 = (w(0, 0, 0) + w(1, 0, 0)) / 2, d2 = (u(0, 0, 0) + u(0, 0, 1)) / 2;
                const double sz = ga / dZ;
                aW.v[5] += -sz * d1 / 2; aW.v[7] += -sz * d1 / 2;
                aU.v[5] += -sz * c1 / 2; aU.v[0] += -sz * c1 / 2;
                aW.v[0] += sz * d2 / 2; aW.v[2] += sz * d2 / 2;
                aU.v[0] += sz * c2 / 2; aU.v[6] += sz * c2 / 2;
            }
            // ay
            {
                // x: -(u(-1,0)+u(-1,1))/2 (v(-1,0)+v)/2 + (u+u(0,1))/2 (v+v(1,0))/2
                const double a1 = (u(-1, 0, 0) + u(-1, 1, 0)) / 2, b1 = (v(-1, 0, 0) + v(0, 0, 0)) / 2;
                const double a2 = (u(0, 0, 0) + u(0, 1, 0)) / 2, b2 = (v(0, 0, 0) + v(1, 0, 0)) / 2;
                const double s = gbv / dX;
                aU.v[1] += -s * b1 / 2; aU.v[7] += -s * b1 / 2;
                aV.v[1] += -s * a1 / 2; aV.v[0] += -s * a1 / 2;
                aU.v[0] += s * b2 / 2; aU.v[4] += s * b2 / 2;
                aV.v[0] += s * a2 / 2; aV.v[2] += s * a2 / 2;
                const double t3 = (v(0, -1, 0) + v(0, 0, 0)) / 2, t4 = (v(0, 0, 0) + v(0, 1, 0)) / 2;
                aV.v[3] += gbv * (-t3) / dY;
                aV.v[0] += gbv * (-t3 + t4) / dY;
                aV.v[4] += gbv * t4 / dY;
                // z: -(w(0,0,-1)+w(0,1,-1))/2 (v(0,0,-1)+v)/2 + (w+w(0,1,0))/2 (v+v(0,0,1))/2
                const double c1 = (w(0, 0, -1) + w(0, 1, -1)) / 2, d1 = (v(0, 0, -1) + v(0, 0, 0)) / 2;
                const double c2 = (w(0, 0, 0) + w(0, 1, 0)) / 2, d2 = (v(0, 0, 0) + v(0, 0, 1)) / 2;
                const double sz = gbv / dZ;
                aW.v[5] += -sz * d1 / 2; aW.v[8] += -sz * d1 / 2;
                aV.v[5] += -sz * c1 / 2; aV.v[0] += -sz * c1 / 2;
                aW.v[0] += sz * d2 / 2; aW.v[4] += sz * d2 / 2;
                aV.v[0] += sz * c2 / 2; aV.v[6] += sz * c2 / 2;
            }
            // az
            {
                // x: -(u(-1,0,0)+u(-1,0,1))/2 (w(-1)+w)/2 + (u+u(0,0,1))/2 (w+w(1))/2
                const double a1 = (u(-1, 0, 0) + u(-1, 0, 1)) / 2, b1 = (w(-1, 0, 0) + w(0, 0, 0)) / 2;
                const double a2 = (u(0, 0, 0) + u(0, 0, 1)) / 2, b2 = (w(0, 0, 0) + w(1, 0, 0)) / 2;
                const double s = gc / dX;
                aU.v[1] += -s * b1 / 2; aU.v[8] += -s * b1 / 2;
                aW.v[1] += -s * a1 / 2; aW.v[0] += -s * a1 / 2;
                aU.v[0] += s * b2 / 2; aU.v[6] += s * b2 / 2;
                aW.v[0] += s * a2 / 2; aW.v[2] += s * a2 / 2;
                // y: -(v(0,-1,0)+v(0,-1,1))/2 (w(0,-1)+w)/2 + (v+v(0,0,1))/2 (w+w(0,1))/2
                const double c1 = (v(0, -1, 0) + v(0, -1, 1)) / 2, d1 = (w(0, -1, 0) + w(0, 0, 0)) / 2;
                const double c2 = (v(0, 0, 0) + v(0, 0, 1)) / 2, d2 = (w(0, 0, 0) + w(0, 1, 0)) / 2;
                const double sy = gc / dY;
                aV.v[3] += -sy * d1 / 2; aV.v[8] += -sy * d1 / 2;
                aW.v[3] += -sy * c1 / 2; aW.v[0] += -sy * c1 / 2;
                aV.v[0] += sy * d2 / 2; aV.v[6] += sy * d2 / 2;
                aW.v[0] += sy * c2 / 2; aW.v[4] += sy * c2 / 2;
                const double t5 = (w(0, 0, -1) + w(0, 0, 0)) / 2, t6 = (w(0, 0, 0) + w(0, 0, 1)) / 2;
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
                if (aU.v[q] != 0.0) atomicAdd(&a.lU[hix(g, i + offU[q][0], j + offU[q][1], k + offU[q][2])], aU.v[q]);
                if (aV.v[q] != 0.0) atomicAdd(&a.lV[hix(g, i + offV[q][0], j + offV[q][1], k + offV[q][2])], aV.v[q]);
                if (aW.v[q] != 0.0) atomicAdd(&a.lW[hix(g, i + offW[q][0], j + offW[q][1], k + offW[q][2])], aW.v[q]);
            }
        }
        // pressure gradient gp_c = -dt (P(o + e_c) - P(o)) / d_c
        {
            const double px = dt / dX * lua[0], py = dt / dY * lua[1], pz = dt / dZ * lua[2];
            atomicAdd(&a.lP[h], px + py + pz);
            atomicAdd(&a.lP[hix(g, i + 1, j, k)], -px);
            atomicAdd(&a.lP[hix(g, i, j + 1, k)], -py);
            atomicAdd(&a.lP[hix(g, i, j, k + 1)], -pz);
        }
        // polymer stress T = coef_t div(C0), C0 = f C - I (fenep.f90:645-691)
        if (a.polymer) {
            const double sx = a.coef_t * lT[0], sy = a.coef_t * lT[1], sz = a.coef_t * lT[2];
            double *L = a.lC0;
            const size_t cs = (size_t)a.cs;
            auto add = [&](int m, int x, int y, int z, double val) {
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
    block_atomic_add(gb, a.grad + 1);
}

// C0 = f(C) C - I on every cell (halo included), f = (L^2 - 3)/(L^2 - tr C):
// adds the adjoint of C^{n+1} and the L^2, beta, Wi terms (the stress
// coefficient (1-beta)/(Re Wi) enters through sum C0 . lC0).
__global__ void k_c0_adj(const double *C, const double *lC0, double *lC, int cs, double lp2, double inv_1mb,
                         double inv_wi, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double g_coef = 0.0, g_l2 = 0.0;
    if (t < cs) {
        double c[6], l[6];
        bool any = false;
        for (int m = 0; m < 6; ++m) {
            l[m] = lC0[(size_t)m * cs + t];
            any = any || l[m] != 0.0;
        }
        if (any) {
            const double E[6] = {1.0, 0.0, 0.0, 1.0, 0.0, 1.0};
            for (int m = 0; m < 6; ++m) c[m] = C[(size_t)m * cs + t];
            const double tr = c[0] + c[3] + c[5];
            const double den = lp2 - tr;
            const double f = (lp2 - 3) / den;
            double lf = 0.0;
            for (int m = 0; m < 6; ++m) {
                lC[(size_t)m * cs + t] += f * l[m];
                lf += c[m] * l[m];
                g_coef += (f * c[m] - E[m]) * l[m];
            }
            const double dfdtr = f / den;
            lC[t] += lf * dfdtr;
            lC[(size_t)3 * cs + t] += lf * dfdtr;
            lC[(size_t)5 * cs + t] += lf * dfdtr;
            g_l2 = lf * (3.0 - tr) / (den * den);
        }
    }
    block_atomic_add(-g_coef * inv_1mb, grad + 1);
    block_atomic_add(-g_coef * inv_wi, grad + 0);
    block_atomic_add(g_l2, grad + 2);
}

// ---------------------------------------------------------------------------
// Polymer update transposed: implicit-function adjoint of the Lyapunov Newton
// solve and the Cstar upwind sum (fenep.f90:464-643).

struct W3 {
    double m, c, p;   // weights of C at the - neighbour, the cell, the + neighbour
};

__device__ inline void wface_p(int idx, double &wm, double &w0, double &wp) {
    switch (idx) {
    case 1: wm = 0.0; w0 = 1.5; wp = -0.5; break;
    case 2: wm = 0.5; w0 = 0.5; wp = 0.0; break;
    case 3: wm = 0.25; w0 = 1.0; wp = -0.25; break;
    default: wm = 0.0; w0 = 1.0; wp = 0.0;
    }
}
__device__ inline void wface_n(int idx, double &wm, double &w0, double &wp) {
    switch (idx) {
    case 1: wm = 0.0; w0 = 0.5; wp = 0.5; break;
    case 2: wm = -0.5; w0 = 1.5; wp = 0.0; break;
    case 3: wm = -0.25; w0 = 1.0; wp = 0.25; break;
    default: wm = 0.0; w0 = 1.0; wp = 0.0;
    }
}

struct PolyAdjArgs {
    const double *C, *Cn;             // C^n (the state) and C after the update (halo, 6 SoA fields)
    const uint8_t *codes, *codes_g;
    const double *U, *V, *W;          // U^n (halo)
    const double *lX;                 // adjoint of C^{n+1} (interior)
    double *lC;                       // out: adjoint of C^n (full halo box, scattered)
    double *lU, *lV, *lW;
    int cs;
    double dt, wi, lp2;
    double *grad;
};

// value of a halo field at row jj of column (i, k); zero beyond the ghost rows
// of a wall channel (the reference wall mode's outside rows)
__device__ inline double rowv(const double *A, const Geo &g, int i, int jj, int k) {
    return (jj < 0 || jj > g.ny + 1) ? 0.0 : A[hix(g, i, jj, k)];
}

__device__ inline int code_of(const uint8_t *codes, const uint8_t *codes_g, const Geo &g, int i, int j, int k) {
    return (j >= 1 && j <= g.ny) ? codes[qix(g, i, j, k)] : codes_g[gcix(g, i, j, k)];
}

// Rows: the cells of the polymer update (with walls also the ghost rows,
// whose faces towards the outside rows carry zero C)
__global__ void __launch_bounds__(128) k_polymer_adj3(PolyAdjArgs a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const int k = blockIdx.z + 1;
    const bool active = i <= g.nx && j < prow0(g) + prows(g);
    double gwi = 0.0, gl2 = 0.0;
    if (active) {
        const size_t cs = (size_t)a.cs;
        const int h = hix(g, i, j, k);
        const double dt = a.dt, wi = a.wi, lp2 = a.lp2, dX = g.dx, dY = g.dy, dZ = g.dz;
        double lx[6], x[6];
        bool any = false;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            lx[m] = a.lX[m * cs + h];
            x[m] = a.Cn[m * cs + h];
            any = any || lx[m] != 0.0;
        }
        if (any) {
            const double *U = a.U, *V = a.V, *W = a.W;
            auto u = [&](int p, int q, int r) { return rowv(U, g, p, q, r); };
            auto v = [&](int p, int q, int r) { return rowv(V, g, p, q, r); };
            auto w = [&](int p, int q, int r) { return rowv(W, g, p, q, r); };
            double A0[3][3];
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
            double A[3][3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) A[r][q] = A0[q][r];
            const double tr = x[0] + x[3] + x[5];
            const double den = lp2 - tr;
            const double f = (lp2 - 3) / den;
            const double dd2 = 1.0 + f * dt / wi;
            const double cf = dt / wi * f / den;    // (dt/Wi) df/dx_d, d in {0, 3, 5}
            // M = J^T, augmented with the right-hand side lx
            double M[6][7];
            {
                double J[6][6];
#pragma unroll
                for (int r = 0; r < 6; ++r)
#pragma unroll
                    for (int q = 0; q < 6; ++q) J[r][q] = 0.0;
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
                        const double u0 = M[c][q], u1 = M[r][q];
                        M[c][q] = sw ? u1 : u0;
                        M[r][q] = sw ? u0 : u1;
                    }
                }
                const double inv = 1.0 / M[c][c];
#pragma unroll
                for (int r = c + 1; r < 6; ++r) {
                    const double fr = M[r][c] * inv;
#pragma unroll
                    for (int q = c; q < 7; ++q) M[r][q] -= fr * M[c][q];
                }
            }
            double mu[6];
#pragma unroll
            for (int r = 5; r >= 0; --r) {
                double s = M[r][6];
#pragma unroll
                for (int q = r + 1; q < 6; ++q) s -= M[r][q] * mu[q];
                mu[r] = s / M[r][r];
            }
            // parameters: G = L(x) + (1 + f dt/Wi) x - b, b includes dt/Wi on the diagonal
            double mx = 0.0;
#pragma unroll
            for (int m = 0; m < 6; ++m) mx += mu[m] * x[m];
            gwi = f * dt / (wi * wi) * mx - dt / (wi * wi) * (mu[0] + mu[3] + mu[5]);
            gl2 = -dt / wi * (3.0 - tr) / (den * den) * mx;
            // adjoint of A = A0^T, then of the velocity-gradient stencils
            double lAt[3][3];
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
            auto addu = [&](int p, int q, int r, double val) { if (inrow(q)) atomicAdd(&a.lU[hix(g, p, q, r)], val); };
            auto addv = [&](int p, int q, int r, double val) { if (inrow(q)) atomicAdd(&a.lV[hix(g, p, q, r)], val); };
            auto addw = [&](int p, int q, int r, double val) { if (inrow(q)) atomicAdd(&a.lW[hix(g, p, q, r)], val); };
            {
                double l = lAt[0][0] * dt / dX;   // A0[0][0]
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
            const double u1 = U[hix(g, i - 1, j, k)], u2 = U[h];
            const double v1 = rowv(V, g, i, j - 1, k), v2 = V[h];
            const double w1 = W[hix(g, i, j, k - 1)], w2 = W[h];
            double s[13];
            s[1] = (-u2 + fabs(u2)) * dt / (2 * dX);
            s[2] = 1.0 / 6 + (-u2 - fabs(u2)) * dt / (2 * dX);
            s[3] = 1.0 / 6 + (u1 - fabs(u1)) * dt / (2 * dX);
            s[4] = (u1 + fabs(u1)) * dt / (2 * dX);
            s[5] = (-v2 + fabs(v2)) * dt / (2 * dY);
            s[6] = 1.0 / 6 + (-v2 - fabs(v2)) * dt / (2 * dY);
            s[7] = 1.0 / 6 + (v1 - fabs(v1)) * dt / (2 * dY);
            s[8] = (v1 + fabs(v1)) * dt / (2 * dY);
            s[9] = (-w2 + fabs(w2)) * dt / (2 * dZ);
            s[10] = 1.0 / 6 + (-w2 - fabs(w2)) * dt / (2 * dZ);
            s[11] = 1.0 / 6 + (w1 - fabs(w1)) * dt / (2 * dZ);
            s[12] = (w1 + fabs(w1)) * dt / (2 * dZ);
            double ls[13];
#pragma unroll
            for (int q = 0; q < 13; ++q) ls[q] = 0.0;
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
            auto wp = [](int code) { W3 w; wface_p(code, w.m, w.c, w.p); return w; };
            auto wn = [](int code) { W3 w; wface_n(code, w.m, w.c, w.p); return w; };
            const W3 wpx = wp(isx), wnx = wn(isx), wpy = wp(isy), wny = wn(isy), wpz = wp(isz), wnz = wn(isz);
            const W3 qx = wp(cxp + 1), rx = wn(cxm + 1), qy = wp(cyp + 1), ry = wn(cym + 1);
            const W3 qz = wp(czp + 1), rz = wn(czm + 1);
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                const double *Cm = a.C + m * cs;
                double *Lm = a.lC + m * cs;
                const double mum = mu[m];
                double lc0 = 0.0;   // accumulated weight at the cell itself
                // one direction: own faces (code is, coefficients sp on the p face, sn on the n face),
                // the + neighbour's p face (code cp_, coefficient sq), the - neighbour's n face (code cm_, sr)
                auto dir = [&](W3 wp_, W3 wn_, int off, int hp, W3 wq, int hm, W3 wr, double sp, double sn,
                               double sq, double sr, bool pghost, bool mghost, double &lsp, double &lsn,
                               double &lsq, double &lsr) {
                    const double cmv = Cm[h - off], c0v = Cm[h], cpv = Cm[h + off];
                    lsp += mum * (wp_.m * cmv + wp_.c * c0v + wp_.p * cpv);
                    lsn += mum * (wn_.m * cmv + wn_.c * c0v + wn_.p * cpv);
                    const double am = mum * (sp * wp_.m + sn * wn_.m);
                    const double ap = mum * (sp * wp_.p + sn * wn_.p);
                    lc0 += mum * (sp * wp_.c + sn * wn_.c);
                    if (am != 0.0) atomicAdd(&Lm[h - off], am);
                    if (ap != 0.0) atomicAdd(&Lm[h + off], ap);
                    // + neighbour's p face
                    if (pghost) {
                        lsq += mum * Cm[hp];
                        if (sq != 0.0) atomicAdd(&Lm[hp], mum * sq);
                    } else {
                        lsq += mum * (wq.m * Cm[hp - off] + wq.c * Cm[hp] + wq.p * Cm[hp + off]);
                        const double b = mum * sq;
                        if (b != 0.0) {
                            if (wq.m != 0.0) atomicAdd(&Lm[hp - off], b * wq.m);
                            atomicAdd(&Lm[hp], b * wq.c);
                            if (wq.p != 0.0) atomicAdd(&Lm[hp + off], b * wq.p);
                        }
                    }
                    // - neighbour's n face
                    if (mghost) {
                        lsr += mum * Cm[hm];
                        if (sr != 0.0) atomicAdd(&Lm[hm], mum * sr);
                    } else {
                        lsr += mum * (wr.m * Cm[hm - off] + wr.c * Cm[hm] + wr.p * Cm[hm + off]);
                        const double b = mum * sr;
                        if (b != 0.0) {
                            if (wr.m != 0.0) atomicAdd(&Lm[hm - off], b * wr.m);
                            atomicAdd(&Lm[hm], b * wr.c);
                            if (wr.p != 0.0) atomicAdd(&Lm[hm + off], b * wr.p);
                        }
                    }
                };
                // x: pxm (s3, own p), nxp (s2, own n), pxp (s1, neighbour i+1), nxm (s4, neighbour i-1)
                dir(wpx, wnx, ox, hxp, qx, hxm, rx, s[3], s[2], s[1], s[4], false, false, ls[3], ls[2], ls[1], ls[4]);
                if (!g.walls) {
                    dir(wpy, wny, oy, hyp, qy, hym, ry, s[7], s[6], s[5], s[8], false, false, ls[7], ls[6], ls[5],
                        ls[8]);
                } else {
                    // rows j-2 .. j+2 of the column, zero beyond the ghost rows
                    auto yv = [&](int jj) { return rowv(Cm, g, i, jj, k); };
                    auto yadd = [&](int jj, double val) {
                        if (val != 0.0 && jj >= 0 && jj <= g.ny + 1) atomicAdd(&Lm[hix(g, i, jj, k)], val);
                    };
                    const double cmv = yv(j - 1), c0v = Cm[h], cpv = yv(j + 1);
                    ls[7] += mum * (wpy.m * cmv + wpy.c * c0v + wpy.p * cpv);
                    ls[6] += mum * (wny.m * cmv + wny.c * c0v + wny.p * cpv);
                    yadd(j - 1, mum * (s[7] * wpy.m + s[6] * wny.m));
                    yadd(j + 1, mum * (s[7] * wpy.p + s[6] * wny.p));
                    lc0 += mum * (s[7] * wpy.c + s[6] * wny.c);
                    // the p face of cell j+1 (rows j .. j+2), the n face of cell j-1 (rows j-2 .. j)
                    ls[5] += mum * (qy.m * c0v + qy.c * cpv + qy.p * yv(j + 2));
                    const double bq = mum * s[5];
                    lc0 += bq * qy.m;
                    yadd(j + 1, bq * qy.c);
                    yadd(j + 2, bq * qy.p);
                    ls[8] += mum * (ry.m * yv(j - 2) + ry.c * cmv + ry.p * c0v);
                    const double br = mum * s[8];
                    yadd(j - 2, br * ry.m);
                    yadd(j - 1, br * ry.c);
                    lc0 += br * ry.p;
                }
                dir(wpz, wnz, oz, hzp, qz, hzm, rz, s[11], s[10], s[9], s[12], false, false, ls[11], ls[10], ls[9],
                    ls[12]);
                atomicAdd(&Lm[h], lc0);
            }
            // s coefficients -> velocities
            {
                const double cx = dt / (2 * dX), cy = dt / (2 * dY), cz = dt / (2 * dZ);
                const double su2 = sgn(u2), su1 = sgn(u1), sv2 = sgn(v2), sv1 = sgn(v1), sw2 = sgn(w2), sw1 = sgn(w1);
                addu(i, j, k, (ls[1] * (-1.0 + su2) + ls[2] * (-1.0 - su2)) * cx);
                addu(i - 1, j, k, (ls[3] * (1.0 - su1) + ls[4] * (1.0 + su1)) * cx);
                addv(i, j, k, (ls[5] * (-1.0 + sv2) + ls[6] * (-1.0 - sv2)) * cy);
                addv(i, j - 1, k, (ls[7] * (1.0 - sv1) + ls[8] * (1.0 + sv1)) * cy);
                addw(i, j, k, (ls[9] * (-1.0 + sw2) + ls[10] * (-1.0 - sw2)) * cz);
                addw(i, j, k - 1, (ls[11] * (1.0 - sw1) + ls[12] * (1.0 + sw1)) * cz);
            }
        }
    }
    block_atomic_add(gwi, a.grad + 0);
    block_atomic_add(gl2, a.grad + 2);
}

// interior of a halo field (reference layout) into an adjoint field, zero halo
__global__ void k_take_interior(const double *src, double *dst, Geo g, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int cs = g.sx * g.sy * g.sz;
    const int h = t % cs;
    const int i = h % g.sx, j = (h / g.sx) % g.sy, k = h / (g.sx * g.sy);
    dst[t] = inner(g, i, j, k) ? src[t] : 0.0;
}

inline dim3 cells(const Geo &g, dim3 b) { return dim3((g.nx + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, g.nz); }

}  // namespace

// ---------------------------------------------------------------------------
// host side

cudaError_t adjoint_fold_state(AdjState &A, const Dev &d, cudaStream_t s) {
    const Geo &g = d.g;
    F8_CUDA_RET(fold(fold_set({{A.lU, BC_U}, {A.lV, BC_V}, {A.lW, BC_W}, {A.lP, BC_P}}), g, s));
    return fold(fold_c(A.lC, d.cs), g, s);
}

cudaError_t take_interior(const double *src, double *dst, const Geo &g, int n, cudaStream_t s) {
    k_take_interior<<<(n + 255) / 256, 256, 0, s>>>(src, dst, g, n); count_launch();
    return cudaGetLastError();
}

cudaError_t step_fp64_adjoint(Dev &d, AdjState &A, const TapeStep &t, const double *drag_w, bool ab2_first,
                              bool polymer, cudaStream_t s) {
    const Geo &g = d.g;
    const int cs = d.cs;
    const size_t hb = (size_t)cs * sizeof(double);
    const double dt = d.ph.dt, re = d.ph.re, beta = d.ph.beta, wi = d.ph.wi;
    const double kap = dt * beta / re / 2.0;
    const unsigned nb = (unsigned)((cs + 255) / 256);
    dim3 blk(32, 8);
    // 6. projection / pressure update
    k_march_adj<<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lP, A.lPhi, t.Phi, g, kap, dt / (2.0 * re), A.grad); count_launch();
    F8_CUDA_RET(fold(fold_set({{A.lPhi, BC_P}}), g, s));
    // 5. Poisson
    k_pack<<<cells(g, blk), blk, 0, s>>>(A.lPhi, A.pack, g); count_launch();
    F8_CUDA_RET(poisson_solve_fp64(d, A.pack, A.lQ[0], s));
    k_div_adj<<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lQ[0], A.lUp[0], A.lUp[1], A.lUp[2], g); count_launch();
    F8_CUDA_RET(cudaMemsetAsync(A.lU, 0, hb, s));
    F8_CUDA_RET(cudaMemsetAsync(A.lV, 0, hb, s));
    F8_CUDA_RET(cudaMemsetAsync(A.lW, 0, hb, s));
    F8_CUDA_RET(fold(fold_set({{A.lUp[0], BC_U}, {A.lUp[1], BC_V}, {A.lUp[2], BC_W}}), g, s));
    // 4. Helmholtz
    for (int c = 0; c < 3; ++c) {
        k_pack<<<cells(g, blk), blk, 0, s>>>(A.lUp[c], A.pack, g); count_launch();
        F8_CUDA_RET(helmholtz_solve_fp64(d, c, A.pack, A.lQ[c], s));
    }
    // 3. IBM
    for (int c = 0; c < 3; ++c) F8_CUDA_RET(cudaMemsetAsync(A.lUa[c], 0, hb, s));
    if (d.nm > 0) {
        IbmAdjArgs ia{};
        ia.mx = d.mx; ia.my = d.my; ia.mcyl = d.mcyl; ia.nm = d.nm; ia.ncyl = d.ncyl;
        ia.dvol = (g.dx * g.dy) * g.dz; ia.dxn = g.dx * g.dx * g.dx; ia.dv = (g.dx * g.dy) * g.dz;
        for (int c = 0; c < 3; ++c) {
            ia.Ua[c] = t.Ua[c]; ia.Fc[c] = t.Fc[c]; ia.lQ[c] = A.lQ[c]; ia.lUa[c] = A.lUa[c];
        }
        ia.w = drag_w;
        ia.grad = A.grad;
        k_ibm_adj<<<dim3((d.nm + 127) / 128, g.nz, 3), 128, 0, s>>>(ia, g); count_launch();
        F8_CUDA_RET(fold(fold_set({{A.lUa[0], BC_U}, {A.lUa[1], BC_V}, {A.lUa[2], BC_W}}), g, s));
    }
    // 2. momentum right-hand side
    if (polymer) F8_CUDA_RET(cudaMemsetAsync(A.lC0, 0, 6 * hb, s));
    {
        MomAdjArgs ma{};
        ma.U = t.U; ma.V = t.V; ma.W = t.W;
        for (int c = 0; c < 3; ++c) {
            ma.Up[c] = t.Up[c]; ma.lQ[c] = A.lQ[c]; ma.lUa[c] = A.lUa[c];
            ma.lA0[c] = A.lA0[c]; ma.lT0[c] = A.lT0[c];
        }
        ma.lU = A.lU; ma.lV = A.lV; ma.lW = A.lW; ma.lP = A.lP; ma.lC0 = A.lC0;
        ma.cs = cs; ma.ab2_first = ab2_first ? 1 : 0; ma.polymer = polymer ? 1 : 0;
        ma.vis = beta / re; ma.coef_t = (1.0 - beta) / (re * wi); ma.c_helm = dt / (2.0 * re); ma.inv_re = 1.0 / re;
        ma.grad = A.grad;
        k_momentum_adj<<<cells(g, blk), blk, 0, s>>>(ma, g); count_launch();
    }
    // 1. polymer
    if (polymer) {
        k_c0_adj<<<nb, 256, 0, s>>>(t.Cn, A.lC0, A.lC, cs, d.ph.lp2, 1.0 / (1.0 - beta), 1.0 / wi, A.grad); count_launch();
        // with walls the stress read the updated ghost rows and their x/z
        // copies; the state's C (wall-extrapolated) adjoint is interior already
        if (g.walls) F8_CUDA_RET(fold_xz(fold_c(A.lC, cs), g, s));
        else F8_CUDA_RET(fold(fold_c(A.lC, cs), g, s));
        F8_CUDA_RET(cudaMemsetAsync(A.lC2, 0, 6 * hb, s));
        PolyAdjArgs pa{};
        pa.C = t.C; pa.Cn = t.Cn; pa.codes = t.codes; pa.codes_g = t.codes_g; pa.U = t.U; pa.V = t.V; pa.W = t.W;
        pa.lX = A.lC; pa.lC = A.lC2; pa.lU = A.lU; pa.lV = A.lV; pa.lW = A.lW;
        pa.cs = cs; pa.dt = dt; pa.wi = wi; pa.lp2 = d.ph.lp2; pa.grad = A.grad;
        dim3 pb(32, 4);
        const dim3 pg((g.nx + pb.x - 1) / pb.x, (prows(g) + pb.y - 1) / pb.y, g.nz);
        k_polymer_adj3<<<pg, pb, 0, s>>>(pa, g); count_launch();
        std::swap(A.lC, A.lC2);
    } else {
        F8_CUDA_RET(cudaMemsetAsync(A.lC, 0, 6 * hb, s));
    }
    return adjoint_fold_state(A, d, s);
}

}  // namespace f8
