// f8_adjoint_mixed.cu — discrete adjoint of the FP32-mixed 3D step (the
// gradient of f8_grad on an F8_MIXED context).
//
// The mixed step (f8_step_mixed.cu) computes the same discrete operator as
// the FP64 step; it differs in precision and in how it reaches the same
// solutions (increment-form Helmholtz solves, a Neumann / Sherman-Morrison
// Newton iteration converging to the same root, an FP32 pressure solve with a
// double-float defect correction).  Its adjoint is therefore the FP64 step's
// stage transposes (f8_adjoint_kernels.cuh), here in FP32 arithmetic on FP32
// adjoint fields, reading the tape the mixed step writes (MixTape): the
// velocity high parts, C before and after the update, the selection codes,
// the explicit IBM velocity, U* and Phi with the boundary values the forward
// kernels read, and the marker forces.  The parameter gradient is accumulated
// in FP64.  The solves are the mixed step's own FP32 transforms and
// tridiagonal sweeps (the operators are symmetric).
#include <algorithm>
#include <cstdio>
#include "f8_adjoint_kernels.cuh"
#include "f8_df64.cuh"
#include "f8_kernels.h"

namespace f8 {

cudaError_t adjoint_fold_state_f(AdjStateF &A, const Dev &d, cudaStream_t s) {
    const Geo &g = d.g;
    return fold(fold_with_c(fold_set<float>({{A.lU, BC_U}, {A.lV, BC_V}, {A.lW, BC_W}, {A.lP, BC_P}}), A.lC, d.cs, 6), g, s);
}

cudaError_t take_interior_f(const float *src, float *dst, const Geo &g, int n, cudaStream_t s) {
    k_take_interior<float><<<(n + 255) / 256, 256, 0, s>>>(src, dst, g, n); count_launch();
    return cudaGetLastError();
}

namespace {

cudaError_t poisson_solve_f(Dev &d, const float *src, float *dst, float *lo, int mode, cudaStream_t s) {
    return d.g.walls ? mixed_solve_walls(d, src, dst, lo, mode, 2, s)
                     : mixed_solve_periodic(d, src, dst, lo, mode, 0.0, -1.0, s);
}

// k_div_adj with the pressure adjoint q as a double-float pair (qh, ql): the
// adjoint projection lUp = lU + (q - q(+e))/(d dt) cancels the gradient part of
// lU, so the difference and its scaling are formed in df64 and only the
// result is rounded to FP32
__global__ void k_div_adj_df(const float *__restrict__ lU, const float *__restrict__ lV, const float *__restrict__ lW,
                             const float *__restrict__ qh, const float *__restrict__ ql, float *__restrict__ lUp,
                             float *__restrict__ lVp, float *__restrict__ lWp, Geo g, df cx, df cy, df cz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cs = g.sx * g.sy * g.sz;
    if (t >= cs) return;
    const int i = t % g.sx, j = (t / g.sx) % g.sy, k = t / (g.sx * g.sy);
    auto q = [&](int ii, int jj, int kk) {
        if (!adj_inner(g, ii, jj, kk)) return df{0.0f, 0.0f};
        const int h = hix(g, ii, jj, kk);
        return df{qh[h], ql[h]};
    };
    const df q0 = q(i, j, k);
    lUp[t] = df_to_f(df_add_f(df_mul(df_sub(q0, q(i + 1, j, k)), cx), lin(lU, g, i, j, k)));
    lVp[t] = df_to_f(df_add_f(df_mul(df_sub(q0, q(i, j + 1, k)), cy), lin(lV, g, i, j, k)));
    lWp[t] = df_to_f(df_add_f(df_mul(df_sub(q0, q(i, j, k + 1)), cz), lin(lW, g, i, j, k)));
}

}  // namespace

cudaError_t step_mixed_adjoint(Dev &d, AdjStateF &A, const MixTape &t, const double *drag_w, bool ab2_first,
                               bool polymer, cudaStream_t s) {
    const Geo &g = d.g;
    const int cs = d.cs;
    const size_t hb = (size_t)cs * sizeof(float);
    const double dt = d.ph.dt, re = d.ph.re, beta = d.ph.beta, wi = d.ph.wi;
    const double kap = dt * beta / re / 2.0;
    const unsigned nb = (unsigned)((cs + 255) / 256);
    dim3 blk(32, 8);
    const AdjCoef<float> kc = adj_coef<float>(g);
    // 6. projection / pressure update
    k_march_adj<float><<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lP, A.lPhi, t.Phi, g, (float)kap, (float)(dt / (2.0 * re)),
                                          kc, A.grad); count_launch();
    F8_CUDA_RET(fold(fold_set<float>({{A.lPhi, BC_P}}), g, s));
    // 5. Poisson, refined as the forward's pressure solve: q0 = L^-1 r in FP32,
    // the defect r - L_h q0 in df64, q = q0 + L^-1 (defect) as a df64 pair
    k_pack<float><<<adj_cells(g, blk), blk, 0, s>>>(A.lPhi, A.pack, g); count_launch();
    F8_CUDA_RET(poisson_solve_f(d, A.pack, A.lQ[0], nullptr, 0, s));
    F8_CUDA_RET(mixed_defect(d, A.lQ[0], A.pack, A.zero, A.rdef, s));
    F8_CUDA_RET(poisson_solve_f(d, A.rdef, A.lQ[0], A.qlo, 2, s));
    k_div_adj_df<<<nb, 256, 0, s>>>(A.lU, A.lV, A.lW, A.lQ[0], A.qlo, A.lUp[0], A.lUp[1], A.lUp[2], g,
                                    df_from_d(1.0 / (g.dx * dt)), df_from_d(1.0 / (g.dy * dt)),
                                    df_from_d(1.0 / (g.dz * dt))); count_launch();
    F8_CUDA_RET(fold(fold_set<float>({{A.lUp[0], BC_U}, {A.lUp[1], BC_V}, {A.lUp[2], BC_W}}), g, s));
    // 4. Helmholtz: the three solves as the forward's parallel branches
    {
        float *pk[3];
        for (int c = 0; c < 3; ++c) pk[c] = A.pack + (size_t)c * d.ni;
        k_pack3<float><<<adj_cells(g, blk), blk, 0, s>>>(A.lUp[0], A.lUp[1], A.lUp[2], pk[0], pk[1], pk[2], g);
        count_launch();
        const float *src[3] = {pk[0], pk[1], pk[2]};
        F8_CUDA_RET(mixed_helmholtz3(d, src, A.lQ, s));
    }
    // 3. IBM
    for (int c = 0; c < 3; ++c) F8_CUDA_RET(cudaMemsetAsync(A.lUa[c], 0, hb, s));
    if (d.nm > 0) {
        IbmAdjArgs<float> ia{};
        ia.mx = d.mx; ia.my = d.my; ia.mcyl = d.mcyl; ia.nm = d.nm; ia.ncyl = d.ncyl;
        ia.dvol = (g.dx * g.dy) * g.dz; ia.dxn = g.dx * g.dx * g.dx; ia.mvol = d.mvol; ia.cylvol = d.cylvol;
        for (int c = 0; c < 3; ++c) {
            ia.Ua[c] = t.Ua[c]; ia.Fc[c] = t.Fc[c]; ia.lQ[c] = A.lQ[c]; ia.lUa[c] = A.lUa[c];
        }
        ia.w = drag_w;
        ia.grad = A.grad;
        ia.d3 = 1;
        k_ibm_adj<float><<<dim3((d.nm + 127) / 128, g.nz, 3), 128, 0, s>>>(ia, g); count_launch();
        // the markers' stencils reach the ghost planes in z; where they reach
        // no ghost column or row (nor row NY, which the V wall rule zeroes)
        // the y and x passes have nothing to do
        const FoldSet<float> fa = fold_set<float>({{A.lUa[0], BC_U}, {A.lUa[1], BC_V}, {A.lUa[2], BC_W}});
        F8_CUDA_RET(d.ibm_edge ? fold(fa, g, s) : fold_z_only(fa, g, s));
    }
    // 2. momentum right-hand side: per-cell sources, then the gather of the
    // velocity, pressure and (with the polymer) C0 / C adjoints
    {
        MomAdjArgs<float> ma{};
        ma.U = t.U; ma.V = t.V; ma.W = t.W;
        for (int c = 0; c < 3; ++c) {
            ma.Up[c] = t.Up[c]; ma.lQ[c] = A.lQ[c]; ma.lUa[c] = A.lUa[c];
            ma.lA0[c] = A.lA0[c]; ma.lT0[c] = A.lT0[c];
        }
        ma.cs = cs; ma.ab2_first = ab2_first ? 1 : 0; ma.polymer = polymer ? 1 : 0;
        ma.vis = (float)(beta / re); ma.coef_t = (float)((1.0 - beta) / (re * wi));
        ma.c_helm = (float)(dt / (2.0 * re)); ma.inv_re = (float)(1.0 / re);
        ma.grad = A.grad;
        ma.kc = kc;
        k_momadj_src<float><<<adj_cells(g, blk), blk, 0, s>>>(ma, A.work, g); count_launch();
        MomGatherArgs<float> mg{};
        mg.U = t.U; mg.V = t.V; mg.W = t.W; mg.src = A.work;
        mg.lU = A.lU; mg.lV = A.lV; mg.lW = A.lW; mg.lP = A.lP; mg.C = t.Cn; mg.lC = A.lC;
        mg.cs = cs; mg.polymer = polymer ? 1 : 0;
        mg.lp2 = (float)(d.ph.lp2); mg.inv_1mb = (float)(1.0 / (1.0 - beta)); mg.inv_wi = (float)(1.0 / wi);
        mg.grad = A.grad;
        mg.kc = kc;
        k_momadj_gather<float><<<nb, 256, 0, s>>>(mg, g); count_launch();
    }
    // 1. polymer: per-cell implicit-function adjoint and Cstar weights, then
    // the gather of the adjoint of C^n and of the velocity
    if (polymer) {
        // with walls the stress read the updated ghost rows and their x/z
        // copies; the state's C (wall-extrapolated) adjoint is interior already
        if (g.walls) F8_CUDA_RET(fold_xz(fold_c(A.lC, cs), g, s));
        else F8_CUDA_RET(fold(fold_c(A.lC, cs), g, s));
        PolyAdjArgs<float> pa{};
        pa.C = t.C; pa.Cn = t.Cn; pa.codes = t.codes; pa.codes_g = t.codes_g; pa.U = t.U; pa.V = t.V; pa.W = t.W;
        pa.lX = A.lC;
        pa.cs = cs; pa.dt = (float)(dt); pa.wi = (float)(wi); pa.lp2 = (float)(d.ph.lp2); pa.grad = A.grad;
        pa.kc = kc; pa.dtwi = (float)(dt / wi); pa.dtwi2 = (float)(dt / (wi * wi));
        dim3 pb(32, 4);
        const dim3 pg((g.nx + pb.x - 1) / pb.x, (prows(g) + pb.y - 1) / pb.y, g.nz);
        k_polyadj_mu<float><<<pg, pb, 0, s>>>(pa, A.work, g); count_launch();
        const dim3 pb2(32, 8), pg2((g.nx + pb2.x - 1) / pb2.x, (prows(g) + pb2.y - 1) / pb2.y, g.nz);
        k_polyadj_cstar<float><<<pg2, pb2, 0, s>>>(pa, A.work, g); count_launch();
        PolyGatherArgs<float> pga{};
        pga.src = A.work; pga.lC = A.lC2; pga.lU = A.lU; pga.lV = A.lV; pga.lW = A.lW; pga.cs = cs;
        k_polyadj_gather<float><<<nb, 256, 0, s>>>(pga, g); count_launch();
        std::swap(A.lC, A.lC2);
    } else {
        F8_CUDA_RET(cudaMemsetAsync(A.lC, 0, 6 * hb, s));
    }
    return adjoint_fold_state_f(A, d, s);
}

}  // namespace f8
