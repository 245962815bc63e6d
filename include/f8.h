/*
 * f8.h — C ABI of the GB300 SMAC + FENE-P + immersed-boundary time step.
 *
 * The reference (machapin/fortran8) has no library interface: its "API" is the
 * set of subroutines that each solver's main loop calls on whole grid arrays
 * (fenep.f90:2477-2527, fenep_2d.f90:1912-1966, fenep_mpi.f90:2929-2967).
 * This header replaces that loop body with one opaque context and a handful of
 * entry points that take the reference's own array layouts, so a Fortran main
 * program can bind them with iso_c_binding (fortran/f8_gpu.f90) and keep its
 * init / output code unchanged.
 *
 * Array layouts (all double precision, column-major as in the reference):
 *   U, V, W, P, Phi : (0:NX+1, 0:NY+1, 0:NZ+1), x fastest, one halo layer
 *                     (fenep.f90:2424, 2437-2438).  In 2D NZ = 1 and the z halo
 *                     planes are copies of plane 1.
 *   C               : (NC, 0:NX+1, 0:NY+1, 0:NZ+1), component fastest;
 *                     NC = 6 in 3D (xx,xy,xz,yy,yz,zz; fenep.f90:2425) and
 *                     NC = 3 in 2D (xx,xy,yy; fenep_2d.f90:1877).
 *   Ax0..Az0, Tx0..Tz0, Fx..Fz : (1:NX, 1:NY, 1:NZ), no halo (fenep.f90:2430-2439).
 *
 * Every call is synchronous on return.  A context is not thread-safe.  No call
 * aborts the host process: failures are reported by the returned status.
 *
 * The same entry points with the prefix f8o_ are exported by the CPU oracle
 * (oracle/liboracle_f8.so), so one harness drives both.
 */
#ifndef F8_H
#define F8_H

#ifdef __cplusplus
extern "C" {
#endif

#define F8_ABI_VERSION 2

/* Status codes.  F8_WARN_* are non-fatal: the step completed. */
enum f8_status {
    F8_OK = 0,
    F8_ERR_ARG = 1,         /* bad grid / parameter / pointer                     */
    F8_ERR_STATE = 2,       /* call out of order (step before load, ...)          */
    F8_ERR_NOMEM = 3,       /* device or host allocation failed                   */
    F8_ERR_CUDA = 4,        /* a CUDA runtime call failed                          */
    F8_ERR_NAN = 5,         /* NaN/Inf found in the velocity after a step
                               (reference: stop 'NaN value', fenep_2d.f90:1974)   */
    F8_ERR_UNSUPPORTED = 6, /* option combination not built                        */
    F8_ERR_NO_DEVICE = 7,   /* no CUDA device / extension not usable               */
    F8_ERR_TOO_LARGE = 8,   /* grid exceeds the fixed workspace of
                               f8_fft_solve_noalloc                                */
    F8_WARN_NEWTON = 16,    /* some cells reached newton_itrmax without meeting
                               newton_eps (reference continues silently,
                               fenep.f90:556-577)                                  */
    F8_WARN_SOR = 17        /* SOR reached sor_itrmax (fenep.f90:885-901)          */
};

enum f8_precision {
    F8_FP64 = 0,   /* every operation in FP64, same operation order as the oracle */
    F8_MIXED = 1   /* FP32 bulk stencils, FP64 state / Peterlin / reductions /
                      Poisson defect correction; 2D with the FFT solver only     */
};

enum f8_poisson {
    F8_POISSON_FFT = 0, /* periodic: 3D FFT (fenep.f90:1529-1560);
                           y-walls: FFT(x,z) + tridiagonal in y
                           (fenep_2d.f90:1294-1342)                            */
    F8_POISSON_SOR = 1  /* red-black SOR (fenep.f90:848-905, smac_kabe.f90:302-374) */
};

enum f8_bc_y {
    F8_BC_PERIODIC = 0, /* PBM (fenep.f90:147-166)                         */
    F8_BC_WALLS = 1,    /* no-slip walls at y = 0 and y = NY*dY
                           (fenep_2d.f90:1098-1143 with NA = 0, NB = NY)  */
    F8_BC_WALLS_Z = 2   /* no-slip walls at z = 0 and z = NZ*dZ, x and y
                           periodic: the channel of smac_kabe.f90
                           (U_kabe .. P_kabe, smac_kabe.f90:118-157; the
                           upper wall moves at uwall in x).  3D, no
                           cylinders; f8_slice, f8_spectrum, f8_turbulence,
                           f8_stats_* and f8_selection_codes return
                           F8_ERR_UNSUPPORTED.  Fields keep the caller's
                           (x, y, z) layouts; the library runs the y-walled
                           step with y and z exchanged                   */
};

typedef struct f8_grid {
    int dim;            /* 2 or 3                                         */
    int nx, ny, nz;     /* cell counts; powers of two for the FFT solver;
                           nz = 1 when dim == 2                           */
    double lx, ly, lz;  /* box lengths: dX = lx/nx ... (fenep.f90:13)     */
    int bc_y;           /* enum f8_bc_y: the box's boundary conditions    */
    double uwall;       /* upper-wall speed when bc_y == F8_BC_WALLS
                           (fenep_2d.f90:1084, 1103)                      */
} f8_grid;

typedef struct f8_phys {
    double re, wi, beta;    /* Re, Wi, beta (fenep.f90:23-25)                          */
    double lp2;             /* L^2 of the Peterlin factor; the reference's Lp**2
                               (fenep.f90:513)                                         */
    double dt;
    double newton_dc;       /* finite-difference step of the Jacobian (fenep.f90:526)  */
    double newton_eps;      /* relative step tolerance (fenep.f90:528)                 */
    int newton_itrmax;      /* fenep.f90:527                                           */
    double sor_omega;       /* SOR relaxation factor                                   */
    double sor_eps;         /* relative residual tolerance (fenep.f90:856)             */
    int sor_itrmax;         /* fenep.f90:857                                           */
    int ab2_start;          /* 1: the first step copies A->A0, T->T0 (input_type == 0,
                               fenep.f90:1445-1452)                                    */
    int ibm_volume;         /* volume a marker force is spread with: F8_IBM_CELL_VOLUME
                               (dX*dY*dZ, fenep.f90 / fenep_mpi.f90:1870-1898) or
                               F8_IBM_ARC_VOLUME (pi*DC/NL * dX*dX of the cylinder's
                               ring, smac.f90:1129, 1428-1446; 3D, surface rings)       */
    int ibm_repeats;        /* direct-forcing iterations per step, NS of smac.f90:20,
                               1607-1611 (interpolate from the last Helmholtz solution,
                               add to the marker force, spread, solve again); 1 = fenep */
    int eigen_test;         /* enum f8_eigen_test: the SPD test of the face candidates
                               (the reference's compile-time eigen_method,
                               fenep.f90:21, 187-212); 3D FP64 only, F8_EIGEN_VIETA
                               elsewhere                                              */
} f8_phys;

enum f8_eigen_test {
    F8_EIGEN_VIETA = 0,      /* eigen_method 3, the default: smallest eigenvalue by the
                                trigonometric cubic formula, -100 on repeated roots
                                (Vieta, fenep.f90:425-444)                            */
    F8_EIGEN_CARDANO = 1,    /* eigen_method 0: the three eigenvalues by Cardano's
                                complex cube roots, -1 when the discriminant is not
                                negative (Cardano, fenep.f90:384-423)                 */
    F8_EIGEN_SYLVESTER = 2,  /* eigen_method 1: +1 when Sylvester's leading minors are
                                positive, else -1 (Sylvester, fenep.f90:446-461)      */
    F8_EIGEN_SYMMETRIC = 3   /* eigen_method 2: the three eigenvalues of the symmetric
                                matrix, repeated roots included (LAPACK dsyev in the
                                reference, fenep.f90:197-212; here the closed form)   */
};

enum f8_ibm_volume {
    F8_IBM_CELL_VOLUME = 0,
    F8_IBM_ARC_VOLUME = 1
};

typedef struct f8_cyl {
    double xc, yc;  /* centre in the x-y plane; the cylinder spans z            */
    double r;       /* radius (the reference's DC/2, fenep.f90:19)             */
    double spin;    /* marker surface speed of a rotating cylinder; 0 = fixed
                       (fenep.f90:1847-1854, 1882-1889)                         */
    int filled;     /* 1: markers on concentric shells (ibm_type 2x,
                       fenep.f90:1791-1801); 0: surface ring (ibm_type 1x)      */
} f8_cyl;

typedef struct f8_fields {
    double *u, *v, *w, *p, *phi;    /* halo layout, see above                   */
    double *c;                      /* component-fastest halo layout            */
    double *ax0, *ay0, *az0;        /* AB2 history of the convection term       */
    double *tx0, *ty0, *tz0;        /* trapezoid history of the polymer stress  */
    double *fx, *fy, *fz;           /* body force (fenep.f90:96-120)            */
} f8_fields;

typedef struct f8_diag {
    int step;                   /* steps taken since f8_load's step0            */
    double ke;                  /* 0.5 <|u|^2> on cell centres (fenep.f90:2266-2300) */
    double cfl;                 /* max(|u|dt/dX + |v|dt/dY + |w|dt/dZ)           */
    double trc_min, trc_max, trc_mean;
    double div_max;             /* max |div u| after the projection             */
    long long newton_iters;     /* Newton iterations summed over cells and the
                                   steps of the last f8_step call               */
    long long newton_unconverged; /* cell-steps that hit newton_itrmax, same span */
    int poisson_iters;          /* SOR iterations of the last step (-1: FFT);
                                   sor_itrmax + 1 when the cap was reached, the
                                   value of the reference's loop counter after
                                   a DO loop that did not exit (fenep.f90:885-901) */
    int nan_found;
    long long kernel_launches;  /* CUDA kernels launched by this context's f8_step
                                   calls since f8_load or f8_timing_reset (0 for
                                   the CPU oracle)                                */
    double trc_std;             /* standard deviation of trC over the cells,
                                   mean first (fenep.f90:2316-2317)              */
} f8_diag;

/* Turbulence statistics of all_time_dif (fenep_mpi.f90:2200-2348), scales
 * U_C = L_C = 1, nu = 1/Re.  "rms" in the reference is a mean square. */
typedef struct f8_turb {
    double k_energy;            /* (<u'^2> + <v'^2> + <w'^2>)/2 on cell centres     */
    double k_staggered;         /* sum(U^2 + V^2 + W^2) / (2 N) of the state        */
    double lambda, re_lambda;   /* Taylor length sqrt(<u'^2>/<(du'/dx)^2>), Re_lambda */
    double epsilon;             /* nu/2 <S_ij S_ij>, S = D + D^T                     */
    double l_kolmogorov, t_kolmogorov, u_kolmogorov;
    double ep_energy;           /* <0.5 (1-beta)/(Re Wi) (L^2-3) log f(C)>           */
    double trc_mean, trc_std;
} f8_turb;

typedef struct f8_ctx f8_ctx;

/* Create a solver context.  cyls may be NULL when ncyl == 0 (no IBM; the
 * predictor is the plain CN/AB2 FFT step, fenep.f90:1430-1527).  precision is
 * enum f8_precision, poisson enum f8_poisson.
 * Replaces: fft_init + ibm_init (fenep.f90:2459-2462, 1374-1377, 1769-1900). */
int f8_create(f8_ctx **ctx, const f8_grid *grid, const f8_phys *phys,
              const f8_cyl *cyls, int ncyl, int precision, int poisson);

/* Copy a state in from host arrays in the reference layouts.  Any pointer of
 * the A0/T0/F/phi groups may be NULL (zeros).  step0 is the number of steps
 * already taken (0 = fresh start; the AB2 start rule applies when
 * step0 == 0 and phys->ab2_start).
 * Replaces: init / input (fenep.f90:52-145, 1186-1233). */
int f8_load(f8_ctx *ctx, const f8_fields *in, int step0);

/* Advance nsteps time steps.  drag may be NULL; otherwise it receives
 * nsteps * ncyl * 3 doubles: for each step and cylinder the force of the
 * fluid on the body, -sum_markers(Fc) * dV (x, y, z), dV the spreading volume
 * of a marker (dX*dY*dZ in 3D, dX*dY in 2D, or the ring's arc element with
 * F8_IBM_ARC_VOLUME), from the marker force after the last forcing iteration.
 * Returns the worst status of the steps.
 * Replaces: the body of the step loop (fenep.f90:2477-2527). */
int f8_step(f8_ctx *ctx, int nsteps, double *drag);

/* Copy the state out to host arrays (same layouts as f8_load).  NULL
 * pointers are skipped.  Replaces: output (fenep.f90:1186-1233). */
int f8_store(f8_ctx *ctx, f8_fields *out);

/* Advance nsteps steps like f8_step and return the gradient of
 *     J = sum_{n,l,c} drag_weights[n][l][c] * drag[n][l][c]
 *       + <seed, state after the nsteps> (interior values)
 * from the discrete adjoint of the step.  The reference has no adjoint; the
 * forward it differentiates is the step of f8_step (fenep.f90:2477-2527 with
 * the IBM of fenep_mpi.f90:1794-1929; 2D fenep_2d.f90:1912-1966).
 *   drag_weights : nsteps * ncyl * 3 doubles, or NULL for the time-averaged
 *                  total drag J = (1/nsteps) sum_n sum_l drag_x[n][l];
 *   seed         : adjoint of the final state (interior cells of u, v, w, p,
 *                  c, ax0..az0, tx0..tz0; NULL members are zero), or NULL;
 *   J            : the drag term of J (host, 1 double) or NULL;
 *   dJ_dparams   : 3 + 2*ncyl doubles: dJ/dWi, dJ/dbeta, dJ/dL^2, then
 *                  dJ/dxc, dJ/dyc of each cylinder (its markers move with it);
 *   dJ_dstate    : adjoint of the initial state (interior cells of u, v, w,
 *                  p, c, ax0..tz0; halo cells and the other members are set
 *                  to 0; NULL members skipped), or NULL;
 *   drag         : the drag history as f8_step returns it, or NULL.
 * The forward runs once, keeping a checkpoint of the state every
 * checkpoint_every steps (0: one segment); the reverse sweep recomputes each
 * segment with its intermediate fields stored, then runs the adjoint of its
 * steps.  The selection of the SPD face candidates is held fixed (its
 * derivative is zero almost everywhere); the Newton solution is
 * differentiated through the implicit-function theorem.  Requires one
 * forcing iteration per step and either an F8_FP64 context (2D or 3D, FFT or
 * SOR Poisson solver; the SOR variant's adjoint solve is the same SOR to the
 * same tolerance) or a 3D F8_MIXED context with the FFT solver
 * (F8_ERR_UNSUPPORTED otherwise).  The context's state advances by nsteps as
 * with f8_step. */
int f8_grad(f8_ctx *ctx, int nsteps, int checkpoint_every, const double *drag_weights,
            const f8_fields *seed, double *J, double *dJ_dparams, f8_fields *dJ_dstate, double *drag);

/* Diagnostics of the current state (log_progress, fenep.f90:2266-2342),
 * reduced on the device: kinetic energy, CFL, trC min / max / mean / std,
 * max |div u|, NaN flag, and the iteration counters of the last f8_step. */
int f8_diagnostics(f8_ctx *ctx, f8_diag *out);

/* Mid-plane slice of get_data_binary (fenep.f90:1108-1183; fenep_mpi.f90:
 * 811-937), computed on the device from the resident state: axis 2 is the
 * x-y plane k = NZ/2 (j outer, i inner), axis 1 the x-z plane j = NY/2 and
 * axis 0 the y-z plane i = NX/2 (k outer).  Per point 18 doubles: x, y, z,
 * E(3), KE (variant 0, fenep.f90) or Q (variant 1, fenep_mpi.f90), Omega(3),
 * |Omega|^2/2, trC, C(6); scales U_C = L_C = 1.  out holds 18 * points
 * doubles (host).  3D only (F8_ERR_UNSUPPORTED in 2D). */
int f8_slice(f8_ctx *ctx, int axis, int variant, double *out);

/* Turbulence statistics of the current state (all_time_dif).  mean_u/v/w are
 * host interior fields (1:NX,1:NY,1:NZ) subtracted from the velocity, or NULL
 * (the reference's 'same' key).  3D only. */
int f8_turbulence(f8_ctx *ctx, const double *mean_u, const double *mean_v, const double *mean_w,
                  f8_turb *out);

/* Shell-binned energy spectrum of energy_single (fenep.f90:1606-1672) /
 * fft_energy_dif (fenep_mpi.f90:2567-2667): energy[0..NX] (host, NX+1
 * doubles) from the FP64 3D transform of the (optionally mean-subtracted)
 * velocity on the device; the bins sum to the staggered kinetic energy
 * (Parseval).  3D only. */
int f8_spectrum(f8_ctx *ctx, const double *mean_u, const double *mean_v, const double *mean_w, double *energy);

/* Running statistics accumulated by f8_step after every step of the current
 * context (fenep_mpi.f90:2934-2941 first pass, 3054-3056 second pass).
 *   mode 1: sums of U, V, W over the steps, and the centre-line probes
 *           U_step(k, n) = (U(NX/2,NY/2,k) + U(NX/2-1,NY/2,k))/2, V alike in j,
 *           W alike in k, for k = 1..NZ and the first max_steps steps;
 *   mode 2: sums of (U - mean_u)^2 ... with the interior mean fields given;
 *   mode 0: stop.  Starting a mode clears the sums and the step count.  3D only. */
int f8_stats_begin(f8_ctx *ctx, int mode, const double *mean_u, const double *mean_v, const double *mean_w,
                   int max_steps);

/* Read the running statistics: three interior fields of sums (host, each may
 * be NULL), the probes as (component, step, k) doubles for the steps recorded
 * (NULL to skip), and the number of steps accumulated. */
int f8_stats_read(f8_ctx *ctx, double *sum_u, double *sum_v, double *sum_w, double *probes, int *nsteps);

/* SPD face-candidate choices of the last step's polymer update
 * (CpxCnx / CpyCny / CpzCnz, fenep.f90:220-230; 2D fenep_2d.f90:159-175),
 * one byte per updated cell, layout [k][row][i] with row 0..NY+1 (walls:
 * the ghost rows are updated too) or 1..NY (periodic): bits 2d..2d+1 hold
 * the chosen candidate - 1 (0..2), or 3 when the cell value was used, for
 * d = x, y, z.  For parity checks that count selection flips between two
 * runs.  F8_ERR_STATE before the first step after a load or when beta == 1. */
int f8_selection_codes(f8_ctx *ctx, unsigned char *codes);

/* Number of Lagrangian markers per z-plane and their host-side positions
 * (x, y interleaved; xy may be NULL).  Used by tests and tooling. */
int f8_markers(f8_ctx *ctx, int *n_per_plane, double *xy);

/* Device-side timing (the reference's cpu_time buckets, fenep.f90:2478-2527,
 * reported at 2561-2566).  With timing enabled, f8_step records CUDA events
 * around each stage of every step on the context's stream; f8_timing returns
 * the accumulated milliseconds per stage and the total device time of the
 * f8_step calls since the last reset (the total is recorded even when the
 * per-stage timing is off).  Stages: */
enum f8_stage {
    F8_STAGE_EIGEN = 0,      /* candidate selection by eigen test ("C+-")       */
    F8_STAGE_NEWTON = 1,     /* Cstar + implicit Newton ("Newton")              */
    F8_STAGE_MOMENTUM = 2,   /* stress, convection, viscous, predictor RHS      */
    F8_STAGE_IBM = 3,        /* marker interpolation, force, spreading           */
    F8_STAGE_HELMHOLTZ = 4,  /* CN viscous solves                                */
    F8_STAGE_POISSON = 5,    /* divergence and pressure Poisson solve            */
    F8_STAGE_PROJECT = 6,    /* projection, pressure update, boundary values     */
    F8_NSTAGE = 7
};
/* Kernels of the FP32-mixed step launched once per step, each bracketed by
 * its own pair of CUDA events on its stream while timing is enabled: */
enum f8_kernel {
    F8_KERNEL_CODES = 0,       /* k_codes3_f (2D: k_codes2_f): candidate faces + eigen test */
    F8_KERNEL_UPDATE = 1,      /* k_update3_f (k_update2_f): Cstar + Newton + f(C)          */
    F8_KERNEL_MOMENTUM = 2,    /* k_momentum3_f (k_momentum2_f): stress, convection, RHS   */
    F8_KERNEL_POISSON_RHS = 3, /* k_poisson_rhs_df: div(U + dU)/dt               */
    F8_KERNEL_DEFECT = 4,      /* k_defect_df: Poisson defect                    */
    F8_KERNEL_MARCH = 5,       /* k_march_df: projection + pressure update       */
    F8_NKERNEL = 6
};
int f8_set_timing(f8_ctx *ctx, int enable);
int f8_timing(f8_ctx *ctx, double *total_ms, double *stage_ms /* F8_NSTAGE or NULL */,
              long long *steps_timed);
int f8_timing_reset(f8_ctx *ctx);
/* Accumulated device milliseconds of each enum f8_kernel launch (F8_NKERNEL
 * doubles) and the number of steps they cover, since the last timing reset.
 * FP32-mixed contexts only (F8_ERR_UNSUPPORTED otherwise). */
int f8_kernel_timing(f8_ctx *ctx, double *kernel_ms, long long *steps_timed);

/* Stand-alone periodic spectral solve, the reference's fft_solve
 * (fenep.f90:1400-1428): phi = IFFT( FFT(q) / (nx ny nz) / LHS ) with
 * LHS = lhs0 + lhs1 * (k~x^2 + k~y^2 + k~z^2), k~^2 = 2(1 - cos(2 pi m/N))/d^2,
 * and modes with |LHS| < 1e-16 set to zero.  lhs0 = 1, lhs1 = dt beta/(2 Re)
 * is the CN Helmholtz solve of fft_navier (fenep.f90:1458-1479); lhs0 = 0,
 * lhs1 = -1 the Poisson solve of fft_poisson (fenep.f90:1539-1557).
 * q and phi are DEVICE pointers to dense nx*ny*nz arrays (x fastest, no halo;
 * nz = 1 for a 2D field).  Sizes are powers of two.  FP64.  Allocates its
 * workspace on the device for the duration of the call; runs on the default
 * stream and returns when the result is complete. */
int f8_fft_solve(int nx, int ny, int nz, double lx, double ly, double lz,
                 const double *q, double *phi, double lhs0, double lhs1);

/* The same solve as f8_fft_solve for callers that cannot let a library
 * allocate device memory (for example a driver that reserves all its device
 * memory at start-up, so an allocation during the run would fail or break its
 * budget).  No counterpart in the reference.  It calls no cudaMalloc, cudaFree
 * or other allocating routine: its workspace is a fixed device array of
 * 2.2 MB (plus 64 KB of tables) that every GPU which loads the library holds
 * until the process exits.  Limits and rules:
 *   - (nx/2+1)*ny*nz <= 135168 complex values (e.g. 64^3); larger grids return
 *     F8_ERR_TOO_LARGE;
 *   - every call shares that workspace and leaves its contents behind; each
 *     call overwrites what it reads, but calls that overlap on the GPU (from
 *     several threads or streams) race;
 *   - the first call on a device looks up the workspace address on that
 *     device (the device must be current); make it before any stream capture;
 *   - with CUDA's lazy module loading, the fixed arrays are placed in device
 *     memory when the library's device code is first used on that device,
 *     which may be that first call: make the first call (or any other f8
 *     call on that device) before the caller reserves the rest of the
 *     device memory for its own pool;
 *   - the looked-up address is kept for the life of the process; after a
 *     cudaDeviceReset the library must be unloaded and loaded again before
 *     this entry point is used on that device.
 * q and phi are caller-owned DEVICE buffers as for f8_fft_solve. */
int f8_fft_solve_noalloc(int nx, int ny, int nz, double lx, double ly, double lz,
                         const double *q, double *phi, double lhs0, double lhs1);

const char *f8_strerror(int status);
void f8_destroy(f8_ctx *ctx);

/* Fill a phys struct with the reference's defaults (fenep.f90:526-528, 855-857). */
void f8_default_phys(f8_phys *phys);

#ifdef __cplusplus
}
#endif
#endif /* F8_H */
