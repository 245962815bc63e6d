// f8_kernels.h — device state and kernel launchers of the step (host-visible).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "f8_common.cuh"

namespace f8 {

// Device pointers of one context.  Field layouts are described in f8_common.cuh.
struct Dev {
    Geo g;
    Phys ph;
    int ncomp;           // 6 (3D) or 3 (2D)
    int cs;              // elements of one halo field, SX*SY*SZ
    int ni;              // interior cells NX*NY*NZ
    // state (FP64)
    double *U, *V, *W, *P, *Phi;
    double *C, *Cn;      // ncomp SoA halo fields each
    double *fpet;        // Peterlin factor f(C) on every halo cell
    uint8_t *codes;      // interior: 2 bits per direction, chosen candidate - 1
    uint8_t *codes_g;    // the same for the ghost rows of a wall channel (gcix)
    double *Ax0, *Ay0, *Az0, *Tx0, *Ty0, *Tz0, *Fx, *Fy, *Fz;
    // work
    double *Up, *Vp, *Wp, *Ua, *Va, *Wa;   // halo
    double *Bx, *By, *Bz;                  // interior
    double *Q[3];                          // interior right-hand sides
    double *E;                             // interior SOR residual
    double *H, *H2;                        // spectral scratch
    double *twx_r, *twx_i, *twy_r, *twy_i, *twz_r, *twz_i;
    double *kx2, *ky2, *kz2;
    // IBM
    int nm;                                // markers per plane
    int ncyl;
    double *mx, *my, *mu, *mv;
    int *mcyl;
    double *Fc[3];                         // nm * nz each
    int *csr_off[3], *csr_idx[3];          // per component over (SX*SY) columns
    int *mperm, *moff;                     // markers grouped by cylinder (drag reduction)
    double *dragpart;                      // ncyl * nz * 3 partial sums
    double *mvol;                          // per marker: the volume its force is spread with
    double *cylvol;                        // per cylinder: the marker volume of its drag
    int ibm_repeats;                       // direct-forcing iterations per step (NS)
    int ibm_edge;                          // some marker stencil reaches a ghost column, a ghost row or row NY
    float *Qpre[3];                        // mixed, NS > 1: the right-hand sides before spreading
    float *Fcf[3];                         // mixed: FP32 copies of the marker forces (the spreading's)
    // mixed-precision state and work (F8_MIXED): the state as df64 pairs
    // (hi, lo) of FP32 halo fields
    float *Uf, *Vf, *Wf, *Ul, *Vl, *Wl;    // velocity hi / lo
    float *Pf, *Pl;                        // pressure hi / lo
    float *Phif, *Phil;                    // pressure correction hi / lo
    float *dUf[3];                         // Helmholtz increments dU, dV, dW (halo)
    float *Cf, *Cnf, *fpetf;               // FP32 conformation tensor (SoA halo) and f(C)
    int *fixlist, *fixcnt;                 // cells queued for the exact Newton re-solve
    float *A0f[3], *T0f[3], *Ff[3];        // FP32 history and body force (interior)
    int Funi[3];                           // body force component uniform (value Fval)
    float Fval[3];
    float *Qf[3];                          // FP32 right-hand sides dt*(R + f)
    float *Rhf, *Rlf;                      // df64 Poisson right-hand side (interior)
    float *Rdf;                            // Poisson defect (interior)
    float *Hf, *H2f;                       // FP32 spectra
    float *HfB[2];                         // spectra of the V and W Helmholtz solves when they run
                                           // beside the U solve (fused spectral path)
    cudaStream_t aux[2];                   // the side streams of those two solves (0: none)
    cudaEvent_t ev_fork, ev_join[2];
    cudaEvent_t ev_g[4];                   // wall ghost-row branch: start, codes ready, update done, momentum done
    float *twxf_r, *twxf_i, *twyf_r, *twyf_i, *twzf_r, *twzf_i;
    float *kx2f, *ky2f, *kz2f;             // FP32 copies of the modified wavenumbers
    int fused_planes;                      // 1: (z, y) plane of one kx fits in shared memory
    int plane_cl;                          // walls: CTAs per cluster holding one (z, y) plane (0: none)
    WallLayout plane_wl;                   // its shared-memory layout (wall_layout)
    int march_runs, march_ctas;            // staged projection: z runs per y tile, persistent CTAs (0: direct loads)
    int march_depth;                       // its steps of copies in flight
    float2 *twz2;                          // stage-major twiddles of the warp z transforms (NZ entries)
    float2 *twx2;                          // and of the warp x transforms (NX entries)
    float *wtR[3];                         // Thomas 1/den tables of the U, V, P wall systems
    float *mwx[3], *mwy[3];                // per-marker 1D kernel weights (3 each)
    float *csr_w[3];                       // per column-list entry: the marker's x weight times y weight there
    int *mi0[3], *mj0[3];                  // per-marker stencil origins
    double *mwxd[3], *mwyd[3];             // FP64: per-marker x / y kernel weights (3 each)
    double *mwzd[3];                       // FP64: per-plane z weights of planes n-1, n, n+1 (3 each)
    int *mi0d[3], *mj0d[3];                // FP64: per-marker stencil origins
    int *act_cols[3];                      // interior (i,j) columns that receive spreading
    int nact[3];
    // reductions
    double *red;                           // scratch partial sums (>= 4096)
    double *scal;                          // small scalar results
    int *flag;                             // SOR convergence flag / iteration
    StepCounters *cnt;
};

// Fields of one FP32-mixed step that the reverse of that step reads (the
// tape), written by step_mixed when StepOpts::tape is set.  Halo fields
// carry the boundary values the forward kernels read there.
struct MixTape {
    float *U, *V, *W;        // velocity (hi parts) at the start of the step
    float *C;                // C at the start of the step (6 SoA halo fields)
    float *Cn;               // C after the update as the stress read it (6 fields)
    uint8_t *codes, *codes_g;
    float *Ua[3];            // explicit velocity U^n + dt R (halo, boundary values)
    float *Up[3];            // Helmholtz solutions U^n + dU (halo)
    float *Phi;              // pressure correction (hi part, halo)
    double *Fc[3];           // marker forces (nm * nz each)
};

struct StepOpts {
    bool polymer;      // beta != 1
    bool ab2_first;    // this step copies A->A0, T->T0 first
    bool ibm;
    int poisson;       // F8_POISSON_FFT / SOR
    double sor_omega, sor_eps;
    int sor_itrmax;
    cudaEvent_t *ev;   // NSTAGE+1 events recorded at the stage boundaries, or null
    cudaEvent_t *kev;  // 2*NKERNEL events bracketing the single-launch kernels (f8_kernel), or null
    double *c_mid;     // FP64: receives C as the momentum stage read it (6 halo fields), or null
    const MixTape *tape;   // FP32-mixed: tape of this step, or null
};
constexpr int NSTAGE = 7;
constexpr int NKERNEL = 6;   // enum f8_kernel

// FP64 step (f8_step_fp64.cu).  Returns a cudaError_t of the launches; SOR
// iteration count in *sor_iters.
cudaError_t step_fp64(Dev &d, const StepOpts &o, double *drag_out_dev, int *sor_iters, cudaStream_t s);
cudaError_t bc_all_state_fp64(Dev &d, cudaStream_t s);
cudaError_t init_kernels_fp64();
cudaError_t aos_to_soa(const double *aos, double *soa, int ncomp, int cs, cudaStream_t s);
cudaError_t soa_to_aos(const double *soa, double *aos, int ncomp, int cs, cudaStream_t s);
cudaError_t count_nonfinite(const double *a, int n, unsigned long long *out, cudaStream_t s);
// FP64 helpers shared with the mixed path (f8_step_fp64.cu)
cudaError_t bc_field(double *A, const Geo &g, int kind, cudaStream_t s);
cudaError_t launch_poisson_rhs(Dev &d, double *out, cudaStream_t s);
cudaError_t launch_march(Dev &d, cudaStream_t s);
cudaError_t launch_drag(Dev &d, double *out, cudaStream_t s);
// the FP64 IBM weight tables (mwxd, mwyd, mwzd, mi0d, mj0d) from the marker positions
cudaError_t marker_weights_fp64(Dev &d, cudaStream_t s);
// the linear solves of the step without their inhomogeneous boundary terms:
// Helmholtz (I - dt beta/(2 Re) L) x = q of velocity component comp, and the
// pressure Poisson L x = q; src interior, dst halo layout (interior written)
cudaError_t helmholtz_solve_fp64(Dev &d, int comp, const double *src, double *dst, cudaStream_t s);
cudaError_t poisson_solve_fp64(Dev &d, const double *src, double *dst, cudaStream_t s);
// red-black SOR of Q (interior) into the halo field Phi (start value), residuals in E (interior)
cudaError_t sor_solve_fp64(Dev &d, const double *Q, double *Phi, double *E, double omega, double eps, int itrmax,
                           int *iters, cudaStream_t s);
cudaError_t remove_mean_fp64(Dev &d, double *A, int n, cudaStream_t s);
// On-device diagnostics (f8_diag.cu)
struct DiagValues {
    double ke, cfl, trc_min, trc_max, trc_mean, trc_std, div_max;
    int nan_found;
};
// streaming multiprocessors of the current device (queried once per device)
int device_sm_count();
// blocks of the deterministic on-device reductions: 4 per SM of the device
inline int diag_blocks() { return 4 * device_sm_count(); }
size_t diag_partials();   // doubles of the partials buffer
// slice output (f8_diag.cu): the state of either precision, read as FP64
struct DiagSliceIn {
    const double *U, *V, *W;
    const float *Uh, *Ul, *Vh, *Vl, *Wh, *Wl;
    const double *C;
    const float *Cf;
    int cs, mixed;
};
int slice_points(const Geo &g, int axis);
// turbulence statistics and energy spectrum (f8_diag.cu)
struct TurbValues {
    double k_energy, k_staggered, lambda, re_lambda, epsilon, l_kolmogorov, t_kolmogorov, u_kolmogorov, ep_energy;
};
struct SpecWork {       // FP64 transform workspace of the spectrum (allocated on first use)
    double *pack;       // one interior field, packed
    double *H;          // half spectrum [k][j][kx] complex
    double *twr[3], *twi[3];
    double *hist;       // per-block histograms
};
size_t turb_partials(int nx);
cudaError_t device_turbulence(Dev &d, bool mixed, const double *const mean[3], double *part, double *out,
                              TurbValues *res, cudaStream_t s);
cudaError_t device_spectrum(Dev &d, bool mixed, const double *const mean[3], SpecWork &w, double *energy_dev,
                            cudaStream_t s);
cudaError_t spectrum_kernel_attrs();
cudaError_t device_stats_accum(Dev &d, bool mixed, int mode, const double *mean, double *sums, double *probes, int n,
                               int max_steps, cudaStream_t s);
cudaError_t device_slice(Dev &d, bool mixed, int axis, int variant, double *dev_out, cudaStream_t s);
cudaError_t device_diagnostics(Dev &d, bool mixed, double *part, double *out, DiagValues *res, cudaStream_t s);
// Discrete adjoint of the FP64 3D step (f8_adjoint.cu).  Adjoint fields are
// full halo arrays whose halo cells are zero between stages.
constexpr int ADJ_WORK_FIELDS = 34;   // the largest per-cell source set of the gather kernels
struct AdjState {
    double *lU, *lV, *lW, *lP, *lPhi;      // state U, V, W, P and the pressure correction
    double *lC, *lC2;                      // C and a second C buffer (6 fields each)
    double *lA0[3], *lT0[3];               // AB2 histories (interior)
    double *lUa[3], *lUp[3], *lQ[3];       // explicit velocity, Helmholtz solution, right-hand side
    double *pack;                          // one packed interior field
    double *work;                          // per-cell sources of the gather kernels (ADJ_WORK_FIELDS halo fields)
    double *grad;                          // dJ/d(Wi, beta, L^2, (xc, yc) per cylinder), accumulated
    // SOR variant: the adjoint pressure solve by the same red-black SOR, warm
    // started from the previous adjoint step's solution (lsor, halo)
    int sor;
    double sor_omega, sor_eps;
    int sor_itrmax;
    double *lsor;
    int sor_capped;                        // adjoint solves that reached sor_itrmax
};
// what the reverse of one step reads from its forward step
struct TapeStep {
    const double *U, *V, *W;               // velocity at the start of the step (halo)
    const double *C, *Cn;                  // C before the polymer update (the state) and after it as
                                           // the stress read it (with walls: updated ghost rows)
    const uint8_t *codes, *codes_g;        // face selection codes (interior, wall ghost rows)
    const double *Ua[3], *Up[3], *Phi;     // explicit velocity, Helmholtz solutions, Phi (halo)
    const double *Fc[3];                   // marker forces
};
cudaError_t step_fp64_adjoint(Dev &d, AdjState &A, const TapeStep &t, const double *drag_w, bool ab2_first,
                              bool polymer, cudaStream_t s);
cudaError_t step_fp64_adjoint2(Dev &d, AdjState &A, const TapeStep &t, const double *drag_w, bool ab2_first,
                              bool polymer, cudaStream_t s);
cudaError_t adjoint_fold_state(AdjState &A, const Dev &d, cudaStream_t s);
// dst[q] = src[q] on interior cells of n / cs stacked halo fields, 0 on halo cells
cudaError_t take_interior(const double *src, double *dst, const Geo &g, int n, cudaStream_t s);
// Discrete adjoint of the FP32-mixed 3D step (f8_adjoint_mixed.cu): the same
// stage transposes as the FP64 adjoint in FP32, reading a MixTape.
struct AdjStateF {
    float *lU, *lV, *lW, *lP, *lPhi;
    float *lC, *lC2;
    float *lA0[3], *lT0[3];
    float *lUa[3], *lUp[3], *lQ[3];
    float *pack;             // interior arrays of the solves' right-hand sides (3 * ni)
    float *qlo;              // low part of the refined pressure adjoint (halo, with lQ[0] its high part)
    float *zero, *rdef;      // interior: zeros (the right-hand side's low part), the defect
    float *work;             // per-cell sources of the gather kernels (ADJ_WORK_FIELDS halo fields)
    double *grad;
};
// FP32 solves of the mixed step (f8_step_mixed.cu); mode 0 writes dst, mode 2
// adds the solution to the pair (dst, lo) exactly; sys: 0 U/W, 1 V, 2 P
cudaError_t mixed_solve_periodic(Dev &d, const float *src, float *dst, float *lo, int mode, double lhs0, double lhs1,
                                 cudaStream_t s);
cudaError_t mixed_solve_walls(Dev &d, const float *src, float *dst, float *lo, int mode, int sys, cudaStream_t s);
cudaError_t mixed_helmholtz3(Dev &d, const float *const src[3], float *const dst[3], cudaStream_t s);
cudaError_t mixed_defect(Dev &d, const float *phi, const float *rh, const float *rl, float *rd, cudaStream_t s);
cudaError_t setup_staged_projection(Dev &d);
cudaError_t step_mixed_adjoint(Dev &d, AdjStateF &A, const MixTape &t, const double *drag_w, bool ab2_first,
                               bool polymer, cudaStream_t s);
cudaError_t adjoint_fold_state_f(AdjStateF &A, const Dev &d, cudaStream_t s);
cudaError_t take_interior_f(const float *src, float *dst, const Geo &g, int n, cudaStream_t s);
// Mixed path (f8_step_mixed.cu)
cudaError_t init_kernels_mixed();
cudaError_t step_mixed(Dev &d, const StepOpts &o, double *drag_out_dev, int *sor_iters, cudaStream_t s);
cudaError_t bc_all_state_mixed(Dev &d, cudaStream_t s);
cudaError_t mixed_state_to_fp64(Dev &d, cudaStream_t s);
cudaError_t count_nonfinite_f(const float *a, int n, unsigned long long *out, cudaStream_t s);
cudaError_t d2f(const double *a, float *b, int n, cudaStream_t s, int *varies = nullptr);
cudaError_t f2d(const float *a, double *b, int n, cudaStream_t s);
cudaError_t aos_to_soa_f(const double *aos, float *soa, int ncomp, int cs, cudaStream_t s);
cudaError_t soa_to_aos_f(const float *soa, double *aos, int ncomp, int cs, cudaStream_t s);

}  // namespace f8
