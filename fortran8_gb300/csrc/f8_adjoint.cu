// f8_adjoint.cu — discrete adjoint of the FP64 3D step (the gradient of
// f8_grad on an F8_FP64 context).  The kernels, their conventions and the
// stage order are in f8_adjoint_kernels.cuh (instantiated here for double,
// compiled without FMA contraction like the FP64 step).
#include <algorithm>
#include <cstdio>
#include "f8_adjoint_kernels.cuh"
#include "f8_kernels.h"

namespace f8 {

// ---------------------------------------------------------------------------
// host side

cudaError_t adjoint_fold_state(AdjState &A, const Dev &d, cudaStream_t s) {
    const Geo &g = d.g;
    return fold(fold_with_c(fold_set<double>({{A.lU, BC_U}, {A.lV, BC_V}, {A.lW, BC_W}, {A.lP, BC_P}}), A.lC, d.cs, 6), g, s);
}

cudaError_t take_interior(const double *src, double *dst, const Geo &g, int n, cudaStream_t s) {
    k_take_interior<double><<<(n + 255) / 256, 256, 0, s>>>(src, dst, g, n); count_launch();
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
    const AdjCoef<double> kc = adj_coef<double>(g);
    // 6. projection / pressure update
    k_march_adj<double><<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lP, A.lPhi, t.Phi, g, kap, dt / (2.0 * re), kc, A.grad); count_launch();
    F8_CUDA_RET(fold(fold_set<double>({{A.lPhi, BC_P}}), g, s));
    // 5. Poisson.  The solve maps the right-hand side to the zero-mean Phi
    // through the pseudo-inverse of the symmetric Laplacian, so its transpose
    // is the same map applied to the zero-mean part of the adjoint: the FFT
    // solve (which drops the mean mode), or, for the SOR variant, the same
    // red-black SOR to the same tolerance (then shifted to zero mean)
    k_pack<double><<<adj_cells(g, blk), blk, 0, s>>>(A.lPhi, A.pack, g); count_launch();
    double *lq = A.lQ[0];
    if (A.sor) {
        F8_CUDA_RET(remove_mean_fp64(d, A.pack, d.ni, s));
        int it = 0;
        F8_CUDA_RET(sor_solve_fp64(d, A.pack, A.lsor, A.work, A.sor_omega, A.sor_eps, A.sor_itrmax, &it, s));
        if (it > A.sor_itrmax) ++A.sor_capped;
        lq = A.lsor;
    } else {
        F8_CUDA_RET(poisson_solve_fp64(d, A.pack, A.lQ[0], s));
    }
    k_div_adj<double><<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, lq, A.lUp[0], A.lUp[1], A.lUp[2], g); count_launch();
    F8_CUDA_RET(fold(fold_set<double>({{A.lUp[0], BC_U}, {A.lUp[1], BC_V}, {A.lUp[2], BC_W}}), g, s));
    // 4. Helmholtz
    for (int c = 0; c < 3; ++c) {
        k_pack<double><<<adj_cells(g, blk), blk, 0, s>>>(A.lUp[c], A.pack, g); count_launch();
        F8_CUDA_RET(helmholtz_solve_fp64(d, c, A.pack, A.lQ[c], s));
    }
    // 3. IBM
    for (int c = 0; c < 3; ++c) F8_CUDA_RET(cudaMemsetAsync(A.lUa[c], 0, hb, s));
    if (d.nm > 0) {
        IbmAdjArgs<double> ia{};
        ia.mx = d.mx; ia.my = d.my; ia.mcyl = d.mcyl; ia.nm = d.nm; ia.ncyl = d.ncyl;
        ia.dvol = (g.dx * g.dy) * g.dz; ia.dxn = g.dx * g.dx * g.dx; ia.mvol = d.mvol; ia.cylvol = d.cylvol;
        for (int c = 0; c < 3; ++c) {
            ia.Ua[c] = t.Ua[c]; ia.Fc[c] = t.Fc[c]; ia.lQ[c] = A.lQ[c]; ia.lUa[c] = A.lUa[c];
        }
        ia.w = drag_w;
        ia.grad = A.grad;
        ia.d3 = 1;
        k_ibm_adj<double><<<dim3((d.nm + 127) / 128, g.nz, 3), 128, 0, s>>>(ia, g); count_launch();
        F8_CUDA_RET(fold(fold_set<double>({{A.lUa[0], BC_U}, {A.lUa[1], BC_V}, {A.lUa[2], BC_W}}), g, s));
    }
    // 2. momentum right-hand side: per-cell sources, then the gather of the
    // velocity, pressure and (with the polymer) C0 / C adjoints
    {
        MomAdjArgs<double> ma{};
        ma.U = t.U; ma.V = t.V; ma.W = t.W;
        for (int c = 0; c < 3; ++c) {
            ma.Up[c] = t.Up[c]; ma.lQ[c] = A.lQ[c]; ma.lUa[c] = A.lUa[c];
            ma.lA0[c] = A.lA0[c]; ma.lT0[c] = A.lT0[c];
        }
        ma.cs = cs; ma.ab2_first = ab2_first ? 1 : 0; ma.polymer = polymer ? 1 : 0;
        ma.vis = beta / re; ma.coef_t = (1.0 - beta) / (re * wi);
        ma.c_helm = dt / (2.0 * re); ma.inv_re = 1.0 / re;
        ma.grad = A.grad;
        ma.kc = kc;
        k_momadj_src<double><<<adj_cells(g, blk), blk, 0, s>>>(ma, A.work, g); count_launch();
        MomGatherArgs<double> mg{};
        mg.U = t.U; mg.V = t.V; mg.W = t.W; mg.src = A.work;
        mg.lU = A.lU; mg.lV = A.lV; mg.lW = A.lW; mg.lP = A.lP; mg.C = t.Cn; mg.lC = A.lC;
        mg.cs = cs; mg.polymer = polymer ? 1 : 0;
        mg.lp2 = d.ph.lp2; mg.inv_1mb = 1.0 / (1.0 - beta); mg.inv_wi = 1.0 / wi;
        mg.grad = A.grad;
        mg.kc = kc;
        k_momadj_gather<double><<<nb, 256, 0, s>>>(mg, g); count_launch();
    }
    // 1. polymer: per-cell implicit-function adjoint and Cstar weights, then
    // the gather of the adjoint of C^n and of the velocity
    if (polymer) {
        // with walls the stress read the updated ghost rows and their x/z
        // copies; the state's C (wall-extrapolated) adjoint is interior already
        if (g.walls) F8_CUDA_RET(fold_xz(fold_c(A.lC, cs), g, s));
        else F8_CUDA_RET(fold(fold_c(A.lC, cs), g, s));
        PolyAdjArgs<double> pa{};
        pa.C = t.C; pa.Cn = t.Cn; pa.codes = t.codes; pa.codes_g = t.codes_g; pa.U = t.U; pa.V = t.V; pa.W = t.W;
        pa.lX = A.lC;
        pa.cs = cs; pa.dt = dt; pa.wi = wi; pa.lp2 = d.ph.lp2; pa.grad = A.grad;
        pa.kc = kc; pa.dtwi = dt / wi; pa.dtwi2 = dt / (wi * wi);
        dim3 pb(32, 4);
        const dim3 pg((g.nx + pb.x - 1) / pb.x, (prows(g) + pb.y - 1) / pb.y, g.nz);
        k_polyadj_mu<double><<<pg, pb, 0, s>>>(pa, A.work, g); count_launch();
        const dim3 pb2(32, 8), pg2((g.nx + pb2.x - 1) / pb2.x, (prows(g) + pb2.y - 1) / pb2.y, g.nz);
        k_polyadj_cstar<double><<<pg2, pb2, 0, s>>>(pa, A.work, g); count_launch();
        PolyGatherArgs<double> pga{};
        pga.src = A.work; pga.lC = A.lC2; pga.lU = A.lU; pga.lV = A.lV; pga.lW = A.lW; pga.cs = cs;
        k_polyadj_gather<double><<<nb, 256, 0, s>>>(pga, g); count_launch();
        std::swap(A.lC, A.lC2);
    } else {
        F8_CUDA_RET(cudaMemsetAsync(A.lC, 0, 6 * hb, s));
    }
    return adjoint_fold_state(A, d, s);
}

// ---------------------------------------------------------------------------
// The 2D step (fenep_2d.f90:1912-1966) transposed.  Its momentum and polymer
// transposes scatter with FP64 atomics (the 2D grids are small; the adjoint is
// reproducible to round-off); the projection, the solves and the IBM
// transposes are the 3D kernels with the z coefficients zero and one marker
// plane without z weights.

__device__ inline void scat(double *A, int h, double v) {
    if (v != 0.0) atomicAdd(&A[h], v);
}

// value of a halo field at row jj of column i (plane 1), zero beyond the
// ghost rows of a wall channel, and whether that position exists
__device__ inline double row2(const double *A, const Geo &g, int i, int jj, bool &in) {
    in = jj >= 0 && jj <= g.ny + 1;
    return in ? A[hix(g, i, jj, 1)] : 0.0;
}

struct Mom2AdjArgs {
    const double *U, *V;           // U^n, V^n (halo)
    const double *C;               // C as the stress read it (3 SoA halo fields)
    const double *Up[2];           // Helmholtz solutions (halo)
    const double *lQ[2], *lUa[2];  // adjoints of Q (interior cells) and Ua (halo)
    double *lA0[2], *lT0[2];       // in: adjoint of the new histories; out: of the old (interior)
    double *lU, *lV, *lP;          // += (halo)
    double *lC0;                   // += adjoint of C0 = f C - I (3 halo fields)
    int cs, ab2_first, polymer;
    double dt, vis, coef_t, c_helm, inv_re, lp2, inv_1mb, inv_wi;
    double *grad;
};

// Momentum right-hand side of the 2D step (stress, convection, viscous,
// AB2 / trapezoid histories, pressure gradient; fenep_2d.f90:396-470,
// 1660-1690), one thread per interior cell.
__global__ void __launch_bounds__(256) k_momadj2(Mom2AdjArgs a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    double gb = 0.0, gc = 0.0;
    if (i <= g.nx && j <= g.ny) {
        const int k = 1, h = hix(g, i, j, k), o = qix(g, i, j, k);
        const double dX = g.dx, dY = g.dy, dt = a.dt;
        auto H = [&](int x, int y) { return hix(g, x, y, k); };
        auto u = [&](int x, int y) { return a.U[H(x, y)]; };
        auto v = [&](int x, int y) { return a.V[H(x, y)]; };
        const double ix2 = 1.0 / (dX * dX), iy2 = 1.0 / (dY * dY);
        double lA[2], lT[2], lB[2];
        for (int c = 0; c < 2; ++c) {
            const double lq = a.lQ[c][h];
            const double lua = lq + a.lUa[c][h];
            double *X = c == 0 ? a.lU : a.lV;
            scat(X, h, lua);
            const int hp = c == 0 ? H(i + 1, j) : H(i, j + 1);
            const double dd = c == 0 ? dX : dY;
            scat(a.lP, h, dt / dd * lua);
            scat(a.lP, hp, -dt / dd * lua);
            double la = 1.5 * dt * lua + a.lA0[c][o], lt = 0.5 * dt * lua + a.lT0[c][o];
            if (a.ab2_first) {
                la += -0.5 * dt * lua;
                lt += 0.5 * dt * lua;
                a.lA0[c][o] = 0.0;
                a.lT0[c][o] = 0.0;
            } else {
                a.lA0[c][o] = -0.5 * dt * lua;
                a.lT0[c][o] = 0.5 * dt * lua;
            }
            lA[c] = la;
            lT[c] = lt;
            lB[c] = dt * lua - 0.5 * dt * lq;
            const double *Us = c == 0 ? a.U : a.V;
            auto lap = [&](const double *F) {
                const double x0 = F[h];
                return (F[H(i - 1, j)] - 2 * x0 + F[H(i + 1, j)]) * ix2 + (F[H(i, j - 1)] - 2 * x0 + F[H(i, j + 1)]) * iy2;
            };
            if (lq != 0.0) gb += a.c_helm * lq * lap(a.Up[c]);
            gb += a.inv_re * lB[c] * lap(Us);
            // viscous B = vis lap(U_c)
            const double wv = a.vis * lB[c];
            scat(X, H(i - 1, j), wv * ix2);
            scat(X, H(i + 1, j), wv * ix2);
            scat(X, H(i, j - 1), wv * iy2);
            scat(X, H(i, j + 1), wv * iy2);
            scat(X, h, -2 * wv * (ix2 + iy2));
        }
        // convection, A = -(ax, ay)
        const double lax = -lA[0], lay = -lA[1];
        {
            const double t1 = (u(i - 1, j) + u(i, j)) / 2, t2 = (u(i, j) + u(i + 1, j)) / 2;
            const double lt1 = -2 * t1 / dX * lax, lt2 = 2 * t2 / dX * lax;
            scat(a.lU, H(i - 1, j), lt1 / 2);
            scat(a.lU, h, lt1 / 2 + lt2 / 2);
            scat(a.lU, H(i + 1, j), lt2 / 2);
            const double a1 = (v(i, j - 1) + v(i + 1, j - 1)) / 2, b1 = (u(i, j - 1) + u(i, j)) / 2;
            const double a2 = (v(i, j) + v(i + 1, j)) / 2, b2 = (u(i, j) + u(i, j + 1)) / 2;
            const double la1 = -b1 / dY * lax, lb1 = -a1 / dY * lax, la2 = b2 / dY * lax, lb2 = a2 / dY * lax;
            scat(a.lV, H(i, j - 1), la1 / 2);
            scat(a.lV, H(i + 1, j - 1), la1 / 2);
            scat(a.lU, H(i, j - 1), lb1 / 2);
            scat(a.lU, h, lb1 / 2 + lb2 / 2);
            scat(a.lV, h, la2 / 2);
            scat(a.lV, H(i + 1, j), la2 / 2);
            scat(a.lU, H(i, j + 1), lb2 / 2);
        }
        {
            const double c1 = (u(i - 1, j) + u(i - 1, j + 1)) / 2, d1 = (v(i - 1, j) + v(i, j)) / 2;
            const double c2 = (u(i, j) + u(i, j + 1)) / 2, d2 = (v(i, j) + v(i + 1, j)) / 2;
            const double lc1 = -d1 / dX * lay, ld1 = -c1 / dX * lay, lc2 = d2 / dX * lay, ld2 = c2 / dX * lay;
            scat(a.lU, H(i - 1, j), lc1 / 2);
            scat(a.lU, H(i - 1, j + 1), lc1 / 2);
            scat(a.lV, H(i - 1, j), ld1 / 2);
            scat(a.lU, h, lc2 / 2);
            scat(a.lU, H(i, j + 1), lc2 / 2);
            const double t3 = (v(i, j - 1) + v(i, j)) / 2, t4 = (v(i, j) + v(i, j + 1)) / 2;
            const double lt3 = -2 * t3 / dY * lay, lt4 = 2 * t4 / dY * lay;
            scat(a.lV, h, ld1 / 2 + ld2 / 2 + lt3 / 2 + lt4 / 2);
            scat(a.lV, H(i + 1, j), ld2 / 2);
            scat(a.lV, H(i, j - 1), lt3 / 2);
            scat(a.lV, H(i, j + 1), lt4 / 2);
        }
        // polymer stress T = coef_t (sx, sy) of C0 = f C - I
        if (a.polymer) {
            const int cs = a.cs;
            const double E[3] = {1.0, 0.0, 1.0};
            auto c0 = [&](int m, int x, int y) {
                const int hh = H(x, y);
                const double x0 = a.C[hh], x2 = a.C[(size_t)2 * cs + hh];
                const double f = (a.lp2 - 2) / (a.lp2 - x0 - x2);
                return f * a.C[(size_t)m * cs + hh] - E[m];
            };
            const double sx = (-c0(0, i, j) + c0(0, i + 1, j)) / dX
                            + (-c0(1, i, j - 1) - c0(1, i + 1, j - 1) + c0(1, i, j + 1) + c0(1, i + 1, j + 1)) / (4 * dY);
            const double sy = (-c0(1, i - 1, j) + c0(1, i + 1, j) - c0(1, i - 1, j + 1) + c0(1, i + 1, j + 1)) / (4 * dX)
                            + (-c0(2, i, j) + c0(2, i, j + 1)) / dY;
            gc = a.coef_t * (lT[0] * sx + lT[1] * sy);
            const double lsx = a.coef_t * lT[0], lsy = a.coef_t * lT[1];
            double *L0 = a.lC0, *L1 = a.lC0 + cs, *L2 = a.lC0 + 2 * (size_t)cs;
            scat(L0, h, -lsx / dX);
            scat(L0, H(i + 1, j), lsx / dX);
            const double qy = lsx / (4 * dY), qx = lsy / (4 * dX);
            scat(L1, H(i, j - 1), -qy);
            scat(L1, H(i + 1, j - 1), -qy);
            scat(L1, H(i, j + 1), qy);
            scat(L1, H(i + 1, j + 1), qy);
            scat(L1, H(i - 1, j), -qx);
            scat(L1, H(i + 1, j), qx);
            scat(L1, H(i - 1, j + 1), -qx);
            scat(L1, H(i + 1, j + 1), qx);
            scat(L2, h, -lsy / dY);
            scat(L2, H(i, j + 1), lsy / dY);
        }
    }
    block_atomic_add(gb - gc * a.inv_1mb, a.grad + 1);
    block_atomic_add(-gc * a.inv_wi, a.grad + 0);
}

// C0 = f(C) C - I, f = (L^2 - 2)/(L^2 - tr C) (fenep_2d.f90:275-280, 396-430)
// transposed on every cell of the halo box: lC += the adjoint of C
__global__ void k_c0adj2(const double *C, const double *lC0, double *lC, int cs, double lp2, double *grad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double gl2 = 0.0;
    if (t < cs) {
        const double l0 = lC0[t], l1 = lC0[cs + t], l2 = lC0[2 * (size_t)cs + t];
        if (l0 != 0.0 || l1 != 0.0 || l2 != 0.0) {
            const double x0 = C[t], x1 = C[cs + t], x2 = C[2 * (size_t)cs + t];
            const double tr = x0 + x2, den = lp2 - tr;
            const double f = (lp2 - 2) / den, fp = f / den;
            const double lf = l0 * x0 + l1 * x1 + l2 * x2;
            lC[t] += f * l0 + lf * fp;
            lC[cs + t] += f * l1;
            lC[2 * (size_t)cs + t] += f * l2 + lf * fp;
            gl2 = lf * (2 - tr) / (den * den);
        }
    }
    block_atomic_add(gl2, grad + 2);
}

struct Poly2AdjArgs {
    const double *C, *Cn;              // C^n and C^{n+1} (3 SoA halo fields)
    const uint8_t *codes, *codes_g;
    const double *U, *V;               // U^n (halo)
    const double *lX;                  // adjoint of C^{n+1} (rows of the update)
    double *lC;                        // += adjoint of C^n
    double *lU, *lV;                   // +=
    int cs;
    double dt, wi, lp2;
    double *grad;
};

// weights (m, c, p) of the candidate faces face_p / face_n of the 2D and 3D
// steps (fenep.f90:179-184): index 1..3, 4 the cell value
__device__ inline void fw_p(int idx, double &wm, double &w0, double &wp) {
    switch (idx) {
    case 1: wm = 0.0; w0 = 1.5; wp = -0.5; break;
    case 2: wm = 0.5; w0 = 0.5; wp = 0.0; break;
    case 3: wm = 0.25; w0 = 1.0; wp = -0.25; break;
    default: wm = 0.0; w0 = 1.0; wp = 0.0;
    }
}
__device__ inline void fw_n(int idx, double &wm, double &w0, double &wp) {
    switch (idx) {
    case 1: wm = 0.0; w0 = 0.5; wp = 0.5; break;
    case 2: wm = -0.5; w0 = 1.5; wp = 0.0; break;
    case 3: wm = -0.25; w0 = 1.0; wp = 0.25; break;
    default: wm = 0.0; w0 = 1.0; wp = 0.0;
    }
}

// Polymer update of the 2D step (Cstar with 1/4 weights and the 3-unknown
// Lyapunov Newton, fenep_2d.f90:241-393) transposed by the implicit-function
// theorem at the Newton solution, with the forward's candidate codes frozen.
__global__ void __launch_bounds__(128) k_polyadj2(Poly2AdjArgs a, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + prow0(g);
    const bool active = i <= g.nx && j < prow0(g) + prows(g);
    double gwi = 0.0, gl2 = 0.0;
    if (active) {
        const int k = 1, h = hix(g, i, j, k);
        const size_t cs = (size_t)a.cs;
        double lx[3], x[3];
        bool any = false;
        for (int m = 0; m < 3; ++m) {
            lx[m] = a.lX[m * cs + h];
            x[m] = a.Cn[m * cs + h];
            any = any || lx[m] != 0.0;
        }
        if (any) {
            const double dt = a.dt, dX = g.dx, dY = g.dy, wi = a.wi, lp2 = a.lp2;
            bool in;
            auto u = [&](int p, int q) { return row2(a.U, g, p, q, in); };
            auto v = [&](int p, int q) { return row2(a.V, g, p, q, in); };
            double A0[2][2];
            A0[0][0] = -dt * (-u(i - 1, j) + u(i, j)) / dX;
            A0[0][1] = -dt * (-v(i - 1, j - 1) + v(i + 1, j - 1) - v(i - 1, j) + v(i + 1, j)) / (4 * dX);
            A0[1][0] = -dt * (-u(i - 1, j - 1) - u(i, j - 1) + u(i - 1, j + 1) + u(i, j + 1)) / (4 * dY);
            A0[1][1] = -dt * (-v(i, j - 1) + v(i, j)) / dY;
            const double tr = x[0] + x[2], den = lp2 - tr;
            const double f = (lp2 - 2) / den;
            const double dd = (1.0 + f * dt / wi) / 2.0;
            const double A00 = A0[0][0] + dd, A01 = A0[1][0], A10 = A0[0][1], A11 = A0[1][1] + dd;
            const double cf = (dt / wi) / 2.0 * f / den;
            double J[3][3] = {{2 * A00 + 2 * x[0] * cf, 2 * A01, 2 * x[0] * cf},
                              {A10 + 2 * x[1] * cf, A11 + A00, A01 + 2 * x[1] * cf},
                              {2 * x[2] * cf, 2 * A10, 2 * A11 + 2 * x[2] * cf}};
            // mu = J^-T lx by elimination with partial pivoting
            double M[3][4];
            for (int r = 0; r < 3; ++r) {
                for (int q = 0; q < 3; ++q) M[r][q] = J[q][r];
                M[r][3] = lx[r];
            }
            for (int c = 0; c < 3; ++c) {
                int piv = c;
                for (int r = c + 1; r < 3; ++r)
                    if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
                if (piv != c)
                    for (int q = 0; q < 4; ++q) { const double tq = M[c][q]; M[c][q] = M[piv][q]; M[piv][q] = tq; }
                for (int r = c + 1; r < 3; ++r) {
                    const double fr = M[r][c] / M[c][c];
                    for (int q = c; q < 4; ++q) M[r][q] -= fr * M[c][q];
                }
            }
            double mu[3];
            for (int r = 2; r >= 0; --r) {
                double sacc = M[r][3];
                for (int q = r + 1; q < 3; ++q) sacc -= M[r][q] * mu[q];
                mu[r] = sacc / M[r][r];
            }
            const double mx = mu[0] * x[0] + mu[1] * x[1] + mu[2] * x[2];
            gwi = dt / (wi * wi) * (f * mx - mu[0] - mu[2]);
            gl2 = dt / wi * (tr - 2) / (den * den) * mx;
            // velocity-gradient entries
            const double l00 = -(2 * mu[0] * x[0] + mu[1] * x[1]);
            const double l10 = -(2 * mu[0] * x[1] + mu[1] * x[2]);   // A0[1][0]
            const double l01 = -(mu[1] * x[0] + 2 * mu[2] * x[1]);   // A0[0][1]
            const double l11 = -(mu[1] * x[1] + 2 * mu[2] * x[2]);
            auto su = [&](int p, int q, double val) { bool ok = q >= 0 && q <= g.ny + 1; if (ok) scat(a.lU, hix(g, p, q, k), val); };
            auto sv = [&](int p, int q, double val) { bool ok = q >= 0 && q <= g.ny + 1; if (ok) scat(a.lV, hix(g, p, q, k), val); };
            su(i - 1, j, l00 * dt / dX);
            su(i, j, -l00 * dt / dX);
            const double e01 = l01 * dt / (4 * dX);
            sv(i - 1, j - 1, e01); sv(i + 1, j - 1, -e01); sv(i - 1, j, e01); sv(i + 1, j, -e01);
            const double e10 = l10 * dt / (4 * dY);
            su(i - 1, j - 1, e10); su(i, j - 1, e10); su(i - 1, j + 1, -e10); su(i, j + 1, -e10);
            sv(i, j - 1, l11 * dt / dY);
            sv(i, j, -l11 * dt / dY);
            // Cstar: b = s3 pxm + s1 pxp + s4 nxm + s2 nxp + s7 pym + s5 pyp + s8 nym + s6 nyp
            const double u1 = a.U[hix(g, i - 1, j, k)], u2 = a.U[h];
            const double v1 = row2(a.V, g, i, j - 1, in), v2 = a.V[h];
            const double hx = dt / (2 * dX), hy = dt / (2 * dY);
            const double s1 = (-u2 + fabs(u2)) * hx, s2 = 0.25 + (-u2 - fabs(u2)) * hx;
            const double s3 = 0.25 + (u1 - fabs(u1)) * hx, s4 = (u1 + fabs(u1)) * hx;
            const double s5 = (-v2 + fabs(v2)) * hy, s6 = 0.25 + (-v2 - fabs(v2)) * hy;
            const double s7 = 0.25 + (v1 - fabs(v1)) * hy, s8 = (v1 + fabs(v1)) * hy;
            const int cself = code_of(a.codes, a.codes_g, g, i, j, k);
            const int cxm = code_of(a.codes, a.codes_g, g, wrapx(g, i - 1), j, k) & 3;
            const int cxp = code_of(a.codes, a.codes_g, g, wrapx(g, i + 1), j, k) & 3;
            int jm = j - 1, jp = j + 1;
            if (!g.walls) { jm = wrapy(g, jm); jp = wrapy(g, jp); }
            const int cym = jm < 0 ? 3 : (code_of(a.codes, a.codes_g, g, i, jm, k) >> 2) & 3;
            const int cyp = jp > g.ny + 1 ? 3 : (code_of(a.codes, a.codes_g, g, i, jp, k) >> 2) & 3;
            const int isx = (cself & 3) + 1, isy = ((cself >> 2) & 3) + 1;
            const int hxm = hix(g, wrapx(g, i - 1), j, k), hxp = hix(g, wrapx(g, i + 1), j, k);
            // positions (-1 marks a zero beyond the ghost rows) of each face's 3 points
            int px[4][3], py[4][3];
            px[0][0] = h - 1; px[0][1] = h; px[0][2] = h + 1;        // pxm, nxp (own stencil)
            px[1][0] = hxp - 1; px[1][1] = hxp; px[1][2] = hxp + 1;  // pxp
            px[2][0] = hxm - 1; px[2][1] = hxm; px[2][2] = hxm + 1;  // nxm
            if (!g.walls) {
                const int oy = g.sx, hym = hix(g, i, jm, k), hyp = hix(g, i, jp, k);
                py[0][0] = h - oy; py[0][1] = h; py[0][2] = h + oy;             // pym, nyp
                py[1][0] = hyp - oy; py[1][1] = hyp; py[1][2] = hyp + oy;       // pyp
                py[2][0] = hym - oy; py[2][1] = hym; py[2][2] = hym + oy;       // nym
            } else {
                auto rowh = [&](int jj) { return (jj < 0 || jj > g.ny + 1) ? -1 : hix(g, i, jj, k); };
                py[0][0] = rowh(j - 1); py[0][1] = h; py[0][2] = rowh(j + 1);
                py[1][0] = h; py[1][1] = rowh(j + 1); py[1][2] = rowh(j + 2);
                py[2][0] = rowh(j - 2); py[2][1] = rowh(j - 1); py[2][2] = h;
            }
            double w[8][3];   // pxm, nxp, pxp, nxm, pym, nyp, pyp, nym
            fw_p(isx, w[0][0], w[0][1], w[0][2]);
            fw_n(isx, w[1][0], w[1][1], w[1][2]);
            fw_p(cxp + 1, w[2][0], w[2][1], w[2][2]);
            fw_n(cxm + 1, w[3][0], w[3][1], w[3][2]);
            fw_p(isy, w[4][0], w[4][1], w[4][2]);
            fw_n(isy, w[5][0], w[5][1], w[5][2]);
            fw_p(cyp + 1, w[6][0], w[6][1], w[6][2]);
            fw_n(cym + 1, w[7][0], w[7][1], w[7][2]);
            const int *pos[8] = {px[0], px[0], px[1], px[2], py[0], py[0], py[1], py[2]};
            const double sc[8] = {s3, s2, s1, s4, s7, s6, s5, s8};
            double ls[8];
            for (int q = 0; q < 8; ++q) {
                double face_mu = 0.0;   // sum_m mu_m face_q(m)
                for (int t = 0; t < 3; ++t) {
                    const int p = pos[q][t];
                    if (p < 0 || w[q][t] == 0.0) continue;
                    for (int m = 0; m < 3; ++m) {
                        face_mu += mu[m] * w[q][t] * a.C[m * cs + p];
                        scat(a.lC + m * cs, p, mu[m] * sc[q] * w[q][t]);
                    }
                }
                ls[q] = face_mu;
            }
            // s1..s8 (as ls order: s3 s2 s1 s4 s7 s6 s5 s8) -> u1, u2, v1, v2
            auto sg = [](double z) { return z > 0.0 ? 1.0 : (z < 0.0 ? -1.0 : 0.0); };
            const double lu2 = ls[2] * (-1 + sg(u2)) * hx + ls[1] * (-1 - sg(u2)) * hx;
            const double lu1 = ls[0] * (1 - sg(u1)) * hx + ls[3] * (1 + sg(u1)) * hx;
            const double lv2 = ls[6] * (-1 + sg(v2)) * hy + ls[5] * (-1 - sg(v2)) * hy;
            const double lv1 = ls[4] * (1 - sg(v1)) * hy + ls[7] * (1 + sg(v1)) * hy;
            scat(a.lU, h, lu2);
            scat(a.lU, hix(g, i - 1, j, k), lu1);
            scat(a.lV, h, lv2);
            sv(i, j - 1, lv1);
        }
    }
    block_atomic_add(gwi, a.grad + 0);
    block_atomic_add(gl2, a.grad + 2);
}

cudaError_t step_fp64_adjoint2(Dev &d, AdjState &A, const TapeStep &t, const double *drag_w, bool ab2_first,
                               bool polymer, cudaStream_t s) {
    const Geo &g = d.g;
    const int cs = d.cs;
    const size_t hb = (size_t)cs * sizeof(double);
    const double dt = d.ph.dt, re = d.ph.re, beta = d.ph.beta, wi = d.ph.wi;
    const double kap = dt * beta / re / 2.0;
    const unsigned nb = (unsigned)((cs + 255) / 256);
    dim3 blk(32, 8);
    AdjCoef<double> kc = adj_coef<double>(g);
    kc.id[2] = kc.id2[2] = kc.i4[2] = kc.dtd[2] = kc.dt2d[2] = kc.dt4d[2] = 0.0;   // no z terms
    F8_CUDA_RET(cudaMemsetAsync(A.lW, 0, hb, s));
    // 6. projection / pressure update
    k_march_adj<double><<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lP, A.lPhi, t.Phi, g, kap, dt / (2.0 * re), kc, A.grad); count_launch();
    F8_CUDA_RET(fold(fold_set<double>({{A.lPhi, BC_P}}), g, s));
    // 5. Poisson
    k_pack<double><<<adj_cells(g, blk), blk, 0, s>>>(A.lPhi, A.pack, g); count_launch();
    double *lq = A.lQ[0];
    if (A.sor) {
        F8_CUDA_RET(remove_mean_fp64(d, A.pack, d.ni, s));
        int it = 0;
        F8_CUDA_RET(sor_solve_fp64(d, A.pack, A.lsor, A.work, A.sor_omega, A.sor_eps, A.sor_itrmax, &it, s));
        if (it > A.sor_itrmax) ++A.sor_capped;
        lq = A.lsor;
    } else {
        F8_CUDA_RET(poisson_solve_fp64(d, A.pack, A.lQ[0], s));
    }
    k_div_adj<double><<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, lq, A.lUp[0], A.lUp[1], A.lUp[2], g); count_launch();
    F8_CUDA_RET(fold(fold_set<double>({{A.lUp[0], BC_U}, {A.lUp[1], BC_V}}), g, s));
    // 4. Helmholtz
    for (int c = 0; c < 2; ++c) {
        k_pack<double><<<adj_cells(g, blk), blk, 0, s>>>(A.lUp[c], A.pack, g); count_launch();
        F8_CUDA_RET(helmholtz_solve_fp64(d, c, A.pack, A.lQ[c], s));
    }
    // 3. IBM
    for (int c = 0; c < 2; ++c) F8_CUDA_RET(cudaMemsetAsync(A.lUa[c], 0, hb, s));
    if (d.nm > 0) {
        IbmAdjArgs<double> ia{};
        ia.mx = d.mx; ia.my = d.my; ia.mcyl = d.mcyl; ia.nm = d.nm; ia.ncyl = d.ncyl;
        ia.dvol = g.dx * g.dy; ia.dxn = g.dx * g.dx; ia.mvol = d.mvol; ia.cylvol = d.cylvol;
        for (int c = 0; c < 2; ++c) {
            ia.Ua[c] = t.Ua[c]; ia.Fc[c] = t.Fc[c]; ia.lQ[c] = A.lQ[c]; ia.lUa[c] = A.lUa[c];
        }
        ia.w = drag_w;
        ia.grad = A.grad;
        ia.d3 = 0;
        k_ibm_adj<double><<<dim3((d.nm + 127) / 128, 1, 2), 128, 0, s>>>(ia, g); count_launch();
        F8_CUDA_RET(fold(fold_set<double>({{A.lUa[0], BC_U}, {A.lUa[1], BC_V}}), g, s));
    }
    // 2. momentum right-hand side (the adjoint of U^n starts here; P^n keeps
    // the identity part from P^{n+1})
    F8_CUDA_RET(cudaMemsetAsync(A.lU, 0, hb, s));
    F8_CUDA_RET(cudaMemsetAsync(A.lV, 0, hb, s));
    F8_CUDA_RET(cudaMemsetAsync(A.work, 0, 3 * hb, s));
    {
        Mom2AdjArgs ma{};
        ma.U = t.U; ma.V = t.V; ma.C = t.Cn;
        for (int c = 0; c < 2; ++c) {
            ma.Up[c] = t.Up[c]; ma.lQ[c] = A.lQ[c]; ma.lUa[c] = A.lUa[c];
            ma.lA0[c] = A.lA0[c]; ma.lT0[c] = A.lT0[c];
        }
        ma.lU = A.lU; ma.lV = A.lV; ma.lP = A.lP; ma.lC0 = A.work;
        ma.cs = cs; ma.ab2_first = ab2_first ? 1 : 0; ma.polymer = polymer ? 1 : 0;
        ma.dt = dt; ma.vis = beta / re; ma.coef_t = (1.0 - beta) / (re * wi);
        ma.c_helm = dt / (2.0 * re); ma.inv_re = 1.0 / re; ma.lp2 = d.ph.lp2;
        ma.inv_1mb = polymer ? 1.0 / (1.0 - beta) : 0.0; ma.inv_wi = 1.0 / wi;
        ma.grad = A.grad;
        k_momadj2<<<adj_cells(g, blk), blk, 0, s>>>(ma, g); count_launch();
        if (polymer) { k_c0adj2<<<nb, 256, 0, s>>>(t.Cn, A.work, A.lC, cs, d.ph.lp2, A.grad); count_launch(); }
    }
    // 1. polymer
    if (polymer) {
        if (g.walls) F8_CUDA_RET(fold_xz(fold_c(A.lC, cs, 3), g, s));
        else F8_CUDA_RET(fold(fold_c(A.lC, cs, 3), g, s));
        F8_CUDA_RET(cudaMemsetAsync(A.lC2, 0, 3 * hb, s));
        Poly2AdjArgs pa{};
        pa.C = t.C; pa.Cn = t.Cn; pa.codes = t.codes; pa.codes_g = t.codes_g; pa.U = t.U; pa.V = t.V;
        pa.lX = A.lC; pa.lC = A.lC2; pa.lU = A.lU; pa.lV = A.lV;
        pa.cs = cs; pa.dt = dt; pa.wi = wi; pa.lp2 = d.ph.lp2; pa.grad = A.grad;
        dim3 pb(32, 4);
        const dim3 pgd((g.nx + pb.x - 1) / pb.x, (prows(g) + pb.y - 1) / pb.y, 1);
        k_polyadj2<<<pgd, pb, 0, s>>>(pa, g); count_launch();
        std::swap(A.lC, A.lC2);
    } else {
        F8_CUDA_RET(cudaMemsetAsync(A.lC, 0, 3 * hb, s));
    }
    return fold(fold_with_c(fold_set<double>({{A.lU, BC_U}, {A.lV, BC_V}, {A.lP, BC_P}}), A.lC, cs, 3), g, s);
}

}  // namespace f8
