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
    F8_CUDA_RET(fold(fold_set<double>({{A.lU, BC_U}, {A.lV, BC_V}, {A.lW, BC_W}, {A.lP, BC_P}}), g, s));
    return fold(fold_c(A.lC, d.cs), g, s);
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
        k_polyadj_src<double><<<pg, pb, 0, s>>>(pa, A.work, g); count_launch();
        PolyGatherArgs<double> pga{};
        pga.src = A.work; pga.lC = A.lC2; pga.lU = A.lU; pga.lV = A.lV; pga.lW = A.lW; pga.cs = cs;
        k_polyadj_gather<double><<<nb, 256, 0, s>>>(pga, g); count_launch();
        std::swap(A.lC, A.lC2);
    } else {
        F8_CUDA_RET(cudaMemsetAsync(A.lC, 0, 6 * hb, s));
    }
    return adjoint_fold_state(A, d, s);
}

}  // namespace f8
