// f8_oracle.cpp — CPU FP64 restatement of the reference's SMAC + FENE-P + IBM
// time step.  TEST INFRASTRUCTURE ONLY: this file is the checker that the CUDA
// library in fortran8_gb300/csrc is compared against.  Only tests/, the smoke
// check and bench.py's CPU-baseline leg load it; the product path never does.
//
// It exports the ABI of include/f8.h with the prefix f8o_ so one harness can
// drive both implementations with the same host arrays.
//
// Every routine follows the reference loop by loop and keeps its operation
// order (left-to-right sums, the same divisions) so that an FP64 GPU build
// compiled without FMA contraction can be compared at the 1e-10 level.  Cited
// lines are in machapin/fortran8:
//   3D polymer   fenep.f90:169-643 (CpxCnx/CpyCny/CpzCnz, Vieta, Cstar, f,
//                Lyapunov, Lyapunov_func, gauss)
//   2D polymer   fenep_2d.f90:138-393
//   momentum     fenep.f90:645-770 (polymer_stress, convection, viscous)
//   predictor    fenep.f90:1430-1527 (fft_navier), 1970-2037 (ibm_preliminary)
//   IBM          fenep_mpi.f90:1776-1929 (no debug override), ibm_init
//                fenep.f90:1769-1900 / fenep_2d.f90:1450-1631
//   solvers      fenep.f90:1400-1428 (fft_solve), 1529-1560 (fft_poisson),
//                1562-1604 (fft_march), 848-905 (SOR);
//                walls fenep_2d.f90:1098-1383 (BCs, tdma, *_kabe)
// FFTW is not available here: the DFT is computed by the radix-2 Stockham
// transform below (FFTW's unnormalised sign convention), pinned in the tests
// against a naive DFT and numpy.fft.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off -fopenmp -shared).

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <new>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/f8.h"

namespace {

const double PI = 3.141592653589793238462643383279502884;  // acos(-1.0d0)

struct Marker2 { double x, y, u, v; int cyl; };

struct OCtx {
    f8_grid g{};
    f8_phys ph{};
    std::vector<f8_cyl> cyl;
    int prec = 0, poisson = 0;
    int NX = 0, NY = 0, NZ = 0, NC = 6, dim = 3;
    int SX = 0, SY = 0, SZ = 0;  // halo extents
    double dX = 0, dY = 0, dZ = 0;
    bool walls = false;
    bool loaded = false;
    int step = 0;
    // state
    std::vector<double> U, V, W, P, Phi, C;
    std::vector<double> Ax0, Ay0, Az0, Tx0, Ty0, Tz0, Fx, Fy, Fz;
    // work
    std::vector<double> Up, Vp, Wp, Ua, Va, Wa;
    std::vector<double> Ax, Ay, Az, Bx, By, Bz, Tx, Ty, Tz, Cx, C0;
    std::vector<double> Cpx, Cnx, Cpy, Cny, Cpz, Cnz;
    std::vector<double> Q, fint[3];
    // IBM
    std::vector<Marker2> mk;   // per-plane 2D marker set
    std::vector<double> Fc[3]; // per marker per plane
    // FFT tables: cos/sin(2 pi t / n), t < n/2, per length
    std::vector<double> twx_r, twx_i, twy_r, twy_i, twz_r, twz_i;
    std::vector<double> kx2, ky2, kz2;  // modified wavenumbers 2(1-cos(m d))/d^2
    // diagnostics of the last step
    long long newton_iters = 0, newton_unconv = 0;
    // SPD candidate choice of the last polymer update, one byte per updated
    // cell [k][row][i]: bits 2d..2d+1 = candidate - 1 (0..2) or 3 for the cell
    // value, direction d = x, y, z (fenep.f90:220-230, fenep_2d.f90:159-175)
    std::vector<unsigned char> codes;
    // running statistics (f8o_stats_begin): sums of U, V, W or of squared
    // fluctuations, centre-line probes (component, step, k)
    int stats_mode = 0, stats_n = 0, stats_max = 0;
    std::vector<double> stats_sum, stats_mean, stats_probe;
    int poisson_iters = -1;
    int sor_order = 0;  // 0: reference sweep order, 1: red-black
    bool timing = false;
    double total_ms = 0, stage_ms[7] = {};
    long long timed_steps = 0;
    std::chrono::steady_clock::time_point tmark;
    void mark(int q) {
        if (!timing) return;
        auto now = std::chrono::steady_clock::now();
        if (q > 0) stage_ms[q - 1] += std::chrono::duration<double, std::milli>(now - tmark).count();
        tmark = now;
    }

    size_t hidx(int i, int j, int k) const { return (size_t)i + (size_t)SX * ((size_t)j + (size_t)SY * (size_t)k); }
    size_t iidx(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)NX * ((size_t)(j - 1) + (size_t)NY * (size_t)(k - 1)); }
    size_t nh() const { return (size_t)SX * SY * SZ; }
    size_t ni() const { return (size_t)NX * NY * NZ; }
};

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// ---------------------------------------------------------------------------
// Boundary conditions.  Periodic: PBM / C_PBM (fenep.f90:147-166).
// y-walls (fenep_2d.f90:1098-1143 with NA = 0, NB = NY; the spanwise component
// W follows U with Uwall = 0, as smac_kabe.f90:118-127 treats the tangential
// components).
enum BcKind { BC_U, BC_V, BC_W, BC_P };

void bc_periodic_xz(OCtx &c, double *A, int ncomp) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    for (int k = 0; k <= NZ + 1; ++k)
        for (int j = 0; j <= NY + 1; ++j)
            for (int m = 0; m < ncomp; ++m) {
                A[m + ncomp * c.hidx(0, j, k)] = A[m + ncomp * c.hidx(NX, j, k)];
                A[m + ncomp * c.hidx(NX + 1, j, k)] = A[m + ncomp * c.hidx(1, j, k)];
            }
    (void)NY;
}

void bc_periodic_y(OCtx &c, double *A, int ncomp) {
    for (int k = 0; k <= c.NZ + 1; ++k)
        for (int i = 0; i <= c.NX + 1; ++i)
            for (int m = 0; m < ncomp; ++m) {
                A[m + ncomp * c.hidx(i, 0, k)] = A[m + ncomp * c.hidx(i, c.NY, k)];
                A[m + ncomp * c.hidx(i, c.NY + 1, k)] = A[m + ncomp * c.hidx(i, 1, k)];
            }
}

void bc_periodic_z(OCtx &c, double *A, int ncomp) {
    for (int j = 0; j <= c.NY + 1; ++j)
        for (int i = 0; i <= c.NX + 1; ++i)
            for (int m = 0; m < ncomp; ++m) {
                A[m + ncomp * c.hidx(i, j, 0)] = A[m + ncomp * c.hidx(i, j, c.NZ)];
                A[m + ncomp * c.hidx(i, j, c.NZ + 1)] = A[m + ncomp * c.hidx(i, j, 1)];
            }
}

void bc_scalar(OCtx &c, double *A, BcKind kind) {
    // x planes, then y, then z, as PBM does; the wall rules commute with the
    // periodic copies because each ghost depends on one line of interior cells.
    bc_periodic_xz(c, A, 1);
    if (!c.walls) {
        bc_periodic_y(c, A, 1);
    } else {
        const int NY = c.NY;
        for (int k = 0; k <= c.NZ + 1; ++k)
            for (int i = 0; i <= c.NX + 1; ++i) {
                double &g0 = A[c.hidx(i, 0, k)], &g1 = A[c.hidx(i, NY + 1, k)];
                switch (kind) {
                case BC_U:  // U_kabe: U(:,NA) = -U(:,NA+1); U(:,NB+1) = 2*Uwall - U(:,NB)
                    g0 = -A[c.hidx(i, 1, k)];
                    g1 = 2 * c.g.uwall - A[c.hidx(i, NY, k)];
                    break;
                case BC_W:
                    g0 = -A[c.hidx(i, 1, k)];
                    g1 = -A[c.hidx(i, NY, k)];
                    break;
                case BC_V:  // V_kabe: V(:,NA) = 0; V(:,NB) = 0 (+ beyond)
                    g0 = 0.0;
                    A[c.hidx(i, NY, k)] = 0.0;
                    g1 = 0.0;
                    break;
                case BC_P:  // P_kabe: Neumann copies
                    g0 = A[c.hidx(i, 1, k)];
                    g1 = A[c.hidx(i, NY, k)];
                    break;
                }
            }
    }
    // z periodic last (fenep.f90:153-154)
    for (int j = 0; j <= c.NY + 1; ++j)
        for (int i = 0; i <= c.NX + 1; ++i) {
            A[c.hidx(i, j, 0)] = A[c.hidx(i, j, c.NZ)];
            A[c.hidx(i, j, c.NZ + 1)] = A[c.hidx(i, j, 1)];
        }
}

// C: C_PBM or C_kabe (linear extrapolation 2C(NA+1) - C(NA+2), fenep_2d.f90:1131-1143)
void bc_c(OCtx &c, double *A) {
    const int nc = c.NC;
    bc_periodic_xz(c, A, nc);
    if (!c.walls) {
        bc_periodic_y(c, A, nc);
    } else {
        const int NY = c.NY;
        for (int k = 0; k <= c.NZ + 1; ++k)
            for (int i = 0; i <= c.NX + 1; ++i)
                for (int m = 0; m < nc; ++m) {
                    A[m + nc * c.hidx(i, 0, k)] = 2 * A[m + nc * c.hidx(i, 1, k)] - A[m + nc * c.hidx(i, 2, k)];
                    A[m + nc * c.hidx(i, NY + 1, k)] = 2 * A[m + nc * c.hidx(i, NY, k)] - A[m + nc * c.hidx(i, NY - 1, k)];
                }
    }
    bc_periodic_z(c, A, nc);
}

// ---------------------------------------------------------------------------
// Polymer: eigen tests, face reconstruction, Cstar, Peterlin f, Newton.

// fenep.f90:425-444 (eigen_method == 3, the default)
inline double vieta(const double *a) {
    double a2 = -(a[0] + a[3] + a[5]);
    double a1 = a[0] * a[3] + a[3] * a[5] + a[5] * a[0] - a[4] * a[4] - a[2] * a[2] - a[1] * a[1];
    double a0 = -(a[0] * a[3] * a[5] + a[1] * a[4] * a[2] + a[1] * a[4] * a[2] - a[0] * a[4] * a[4]
                  - a[1] * a[1] * a[5] - a[2] * a[3] * a[2]);
    double p = a1 - (a2 * a2) / 3.0;
    double q = a0 - a1 * a2 / 3.0 + 2.0 * (a2 * a2 * a2) / 27.0;
    double qh = q / 2.0, p3 = p / 3.0;
    double t = qh * qh + p3 * p3 * p3;
    if (t >= 0.0) return -100.0;
    const double two_pi_3 = 2.0 * PI / 3.0;
    return 2.0 * std::sqrt(-p / 3.0) * std::cos(std::acos(3.0 * q / (2.0 * p) * std::sqrt(-3.0 / p)) / 3.0 + two_pi_3)
           - a2 / 3.0;
}

// Fortran minval over two reals ignores NaN unless both are NaN.
inline double nanmin2(double a, double b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return b < a ? b : a;
}

// fenep.f90:384-423 (eigen_method == 0): the three roots of the cubic from
// the complex cube roots of u3 = -q/2 + i sqrt(-t) and of its conjugate v3,
// e_k = w_k u3^(1/3) + conj(w_k) v3^(1/3) - a2/3 with w_k the cube roots of
// unity (principal branch, as Fortran's complex power).  For t >= 0 the
// reference sets -1 and then reads u3, v3 unset; -1 is kept here.
inline void cardano(const double *a, double *e) {
    double a2 = -(a[0] + a[3] + a[5]);
    double a1 = a[0] * a[3] + a[3] * a[5] + a[5] * a[0] - a[4] * a[4] - a[2] * a[2] - a[1] * a[1];
    double a0 = -(a[0] * a[3] * a[5] + a[1] * a[4] * a[2] + a[1] * a[4] * a[2] - a[0] * a[4] * a[4]
                  - a[1] * a[1] * a[5] - a[2] * a[3] * a[2]);
    double p = a1 - (a2 * a2) / 3.0;
    double q = a0 - a1 * a2 / 3.0 + 2.0 * (a2 * a2 * a2) / 27.0;
    double qh = q / 2.0, p3 = p / 3.0;
    double t = qh * qh + p3 * p3 * p3;
    if (t >= 0.0) { e[0] = e[1] = e[2] = -1.0; return; }
    const std::complex<double> u3(-qh, std::sqrt(-t)), v3(-qh, -std::sqrt(-t));
    const std::complex<double> cu = std::pow(u3, 1.0 / 3.0), cv = std::pow(v3, 1.0 / 3.0);
    const std::complex<double> w1(-0.5, std::sqrt(3.0) / 2.0), w2(-0.5, -std::sqrt(3.0) / 2.0);
    e[0] = (cu + cv).real() - a2 / 3.0;
    e[1] = (w1 * cu + w2 * cv).real() - a2 / 3.0;
    e[2] = (w2 * cu + w1 * cv).real() - a2 / 3.0;
}

// fenep.f90:446-461 (eigen_method == 1): 1 when the leading minors are positive
inline double sylvester(const double *a) {
    if (a[0] > 0 && a[3] > 0 && a[5] > 0)
        if (a[0] * a[3] - a[1] * a[1] > 0)
            if (a[0] * a[3] * a[5] + a[1] * a[4] * a[2] + a[1] * a[4] * a[2] - a[0] * a[4] * a[4]
                - a[1] * a[1] * a[5] - a[2] * a[3] * a[2] > 0)
                return 1.0;
    return -1.0;
}

// eigen_method == 2 (LAPACK dsyev, fenep.f90:197-212): the three eigenvalues
// of the symmetric matrix by Jacobi rotations (the oracle's own method; the
// library evaluates the closed form), ascending
inline void symmetric_eig(const double *a, double *e) {
    double A[3][3] = {{a[0], a[1], a[2]}, {a[1], a[3], a[4]}, {a[2], a[4], a[5]}};
    for (int sweep = 0; sweep < 50; ++sweep) {
        const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (A[p][q] == 0.0) continue;
                const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double tt = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double cc = 1.0 / std::sqrt(tt * tt + 1.0), ss = tt * cc;
                for (int k = 0; k < 3; ++k) {   // columns p, q
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = cc * akp - ss * akq;
                    A[k][q] = ss * akp + cc * akq;
                }
                for (int k = 0; k < 3; ++k) {   // rows p, q
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = cc * apk - ss * aqk;
                    A[q][k] = ss * apk + cc * aqk;
                }
            }
    }
    e[0] = A[0][0]; e[1] = A[1][1]; e[2] = A[2][2];
    std::sort(e, e + 3);
}

// minval over the values of one candidate's two faces (fenep.f90:186-241)
inline double face_test(int method, const double *pt, const double *nt) {
    if (method == F8_EIGEN_CARDANO) {
        double e[6];
        cardano(pt, e);
        cardano(nt, e + 3);
        double v = e[0];
        for (int q = 1; q < 6; ++q) v = nanmin2(v, e[q]);
        return v;
    }
    if (method == F8_EIGEN_SYLVESTER) return nanmin2(sylvester(pt), sylvester(nt));
    if (method == F8_EIGEN_SYMMETRIC) {
        double e[6];
        symmetric_eig(pt, e);
        symmetric_eig(nt, e + 3);
        double v = e[0];
        for (int q = 1; q < 6; ++q) v = nanmin2(v, e[q]);
        return v;
    }
    return nanmin2(vieta(pt), vieta(nt));
}

// Fortran maxloc(minlist(1:4), 1): first position of the largest non-NaN value.
inline int maxloc4(const double *m) {
    int idx = 0; double best = 0; bool found = false;
    for (int l = 0; l < 4; ++l) {
        if (std::isnan(m[l])) continue;
        if (!found || m[l] > best) { best = m[l]; idx = l; found = true; }
    }
    return found ? idx + 1 : 1;
}

// Candidates of fenep.f90:179-184 for one direction.
inline void candidates3(const double *cm, const double *c0, const double *cp, double pt[3][6], double nt[3][6]) {
    for (int m = 0; m < 6; ++m) {
        pt[0][m] = c0[m] * 3 / 2 - cp[m] / 2;
        nt[0][m] = c0[m] / 2 + cp[m] / 2;
        pt[1][m] = cm[m] / 2 + c0[m] / 2;
        nt[1][m] = -cm[m] / 2 + c0[m] * 3 / 2;
        pt[2][m] = cm[m] / 4 + c0[m] - cp[m] / 4;
        nt[2][m] = -cm[m] / 4 + c0[m] + cp[m] / 4;
    }
}

// One direction of CpxCnx (fenep.f90:169-242): fills the two face values of
// cell (i,j,k) in direction d.  Returns the chosen index (1..4).
int reconstruct3(const double *cm, const double *c0, const double *cp, double *fp, double *fn, int method) {
    double pt[3][6], nt[3][6], minlist[4];
    candidates3(cm, c0, cp, pt, nt);
    for (int l = 0; l < 3; ++l) minlist[l] = face_test(method, pt[l], nt[l]);
    minlist[3] = 0.0;
    int index = maxloc4(minlist);
    if (index == 4) {
        for (int m = 0; m < 6; ++m) { fp[m] = c0[m]; fn[m] = c0[m]; }
    } else {
        for (int m = 0; m < 6; ++m) { fp[m] = pt[index - 1][m]; fn[m] = nt[index - 1][m]; }
    }
    return index;
}

// Rows of the polymer update.  Periodic: 1..NY.  With y walls also the ghost
// rows 0 and NY+1: the reference's wall mode runs the polymer update on every
// row of its box (CpxCnx .. Lyapunov, fenep_2d.f90:138-348, 1912-1929), where
// the rows beyond the walls hold zero C and velocity (C_kabe, U_kabe, V_kabe,
// fenep_2d.f90:1097-1143), so the ghost rows evolve with the step and the
// stress reads them; they are re-extrapolated only at the end of the step
// (fft_march_kabe, fenep_2d.f90:1371-1374).  The reference's published
// wall-channel accuracy table (_theory.py:44-49) is reproduced this way.
inline int prow_lo(const OCtx &c) { return c.walls ? 0 : 1; }
inline int prow_hi(const OCtx &c) { return c.walls ? c.NY + 1 : c.NY; }

// C of cell (i, j, k), zero beyond the ghost rows (the wall mode's outside rows)
inline const double *cval(const OCtx &c, const double *C, int nc, int i, int j, int k) {
    static const double zero[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return (j < 0 || j > c.NY + 1) ? zero : C + (size_t)nc * c.hidx(i, j, k);
}
inline double vval(const OCtx &c, const double *A, int i, int j, int k) {
    return (j < 0 || j > c.NY + 1) ? 0.0 : A[c.hidx(i, j, k)];
}

// Face arrays: Cpd holds the faces of each line, face f is between cell f and
// f+1; cell n writes Cp(n-1) and Cn(n).  Lines along y cover faces jlo-1 .. jhi.
struct FaceIdx {
    int NX, NY, NZ, jlo, nr;
    size_t x(int f, int j, int k) const { return (size_t)6 * ((size_t)f + (size_t)(NX + 1) * ((size_t)(j - jlo) + (size_t)nr * (k - 1))); }
    size_t y(int i, int f, int k) const { return (size_t)6 * ((size_t)(i - 1) + (size_t)NX * ((size_t)(f - jlo + 1) + (size_t)(nr + 1) * (k - 1))); }
    size_t z(int i, int j, int f) const { return (size_t)6 * ((size_t)(i - 1) + (size_t)NX * ((size_t)(j - jlo) + (size_t)nr * f)); }
    size_t cell(int i, int j, int k) const { return (size_t)6 * ((size_t)(i - 1) + (size_t)NX * ((size_t)(j - jlo) + (size_t)nr * (k - 1))); }
};
inline FaceIdx face_idx(const OCtx &c) {
    return FaceIdx{c.NX, c.NY, c.NZ, prow_lo(c), prow_hi(c) - prow_lo(c) + 1};
}

void polymer_faces3(OCtx &c) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ, jlo = prow_lo(c), jhi = prow_hi(c);
    const FaceIdx F = face_idx(c);
    c.codes.assign((size_t)NX * F.nr * NZ, 0);
    const double *C = c.C.data();
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
        for (int j = jlo; j <= jhi; ++j)
            for (int i = 1; i <= NX; ++i) {
                const double *c0 = cval(c, C, 6, i, j, k);
                const int ix = reconstruct3(cval(c, C, 6, i - 1, j, k), c0, cval(c, C, 6, i + 1, j, k),
                                            &c.Cpx[F.x(i - 1, j, k)], &c.Cnx[F.x(i, j, k)], c.ph.eigen_test);
                const int iy = reconstruct3(cval(c, C, 6, i, j - 1, k), c0, cval(c, C, 6, i, j + 1, k),
                                            &c.Cpy[F.y(i, j - 1, k)], &c.Cny[F.y(i, j, k)], c.ph.eigen_test);
                const int iz = reconstruct3(cval(c, C, 6, i, j, k - 1), c0, cval(c, C, 6, i, j, k + 1),
                                            &c.Cpz[F.z(i, j, k - 1)], &c.Cnz[F.z(i, j, k)], c.ph.eigen_test);
                c.codes[(size_t)(i - 1) + (size_t)NX * ((size_t)(j - jlo) + (size_t)F.nr * (k - 1))] =
                    (unsigned char)((ix - 1) | ((iy - 1) << 2) | ((iz - 1) << 4));
            }
    // Periodic face copies (fenep.f90:240-241, 310-311, 380-381).  With walls
    // the faces beyond the ghost rows belong to the outside cells; Cstar
    // multiplies them by exactly zero (the wall-normal velocity vanishes there).
    for (int k = 1; k <= NZ; ++k)
        for (int j = jlo; j <= jhi; ++j)
            for (int m = 0; m < 6; ++m) {
                c.Cpx[F.x(NX, j, k) + m] = c.Cpx[F.x(0, j, k) + m];
                c.Cnx[F.x(0, j, k) + m] = c.Cnx[F.x(NX, j, k) + m];
            }
    for (int k = 1; k <= NZ; ++k)
        for (int i = 1; i <= NX; ++i)
            for (int m = 0; m < 6; ++m) {
                if (!c.walls) {
                    c.Cpy[F.y(i, NY, k) + m] = c.Cpy[F.y(i, 0, k) + m];
                    c.Cny[F.y(i, 0, k) + m] = c.Cny[F.y(i, NY, k) + m];
                } else {
                    c.Cpy[F.y(i, jhi, k) + m] = 0.0;
                    c.Cny[F.y(i, jlo - 1, k) + m] = 0.0;
                }
            }
    for (int j = jlo; j <= jhi; ++j)
        for (int i = 1; i <= NX; ++i)
            for (int m = 0; m < 6; ++m) {
                c.Cpz[F.z(i, j, NZ) + m] = c.Cpz[F.z(i, j, 0) + m];
                c.Cnz[F.z(i, j, 0) + m] = c.Cnz[F.z(i, j, NZ) + m];
            }
}

// fenep.f90:464-507
void cstar3(OCtx &c) {
    const int NX = c.NX, NZ = c.NZ, jlo = prow_lo(c), jhi = prow_hi(c);
    const FaceIdx F = face_idx(c);
    const double dt = c.ph.dt, dX = c.dX, dY = c.dY, dZ = c.dZ;
    const double *U = c.U.data(), *V = c.V.data(), *W = c.W.data();
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
        for (int j = jlo; j <= jhi; ++j)
            for (int i = 1; i <= NX; ++i) {
                double u1 = vval(c, U, i - 1, j, k), u2 = vval(c, U, i, j, k);
                double v1 = vval(c, V, i, j - 1, k), v2 = vval(c, V, i, j, k);
                double w1 = vval(c, W, i, j, k - 1), w2 = vval(c, W, i, j, k);
                double s1 = (-u2 + std::fabs(u2)) * dt / (2 * dX);
                double s2 = 1.0 / 6 + (-u2 - std::fabs(u2)) * dt / (2 * dX);
                double s3 = 1.0 / 6 + (u1 - std::fabs(u1)) * dt / (2 * dX);
                double s4 = (u1 + std::fabs(u1)) * dt / (2 * dX);
                double s5 = (-v2 + std::fabs(v2)) * dt / (2 * dY);
                double s6 = 1.0 / 6 + (-v2 - std::fabs(v2)) * dt / (2 * dY);
                double s7 = 1.0 / 6 + (v1 - std::fabs(v1)) * dt / (2 * dY);
                double s8 = (v1 + std::fabs(v1)) * dt / (2 * dY);
                double s9 = (-w2 + std::fabs(w2)) * dt / (2 * dZ);
                double s10 = 1.0 / 6 + (-w2 - std::fabs(w2)) * dt / (2 * dZ);
                double s11 = 1.0 / 6 + (w1 - std::fabs(w1)) * dt / (2 * dZ);
                double s12 = (w1 + std::fabs(w1)) * dt / (2 * dZ);
                const double *pxm = &c.Cpx[F.x(i - 1, j, k)], *pxp = &c.Cpx[F.x(i, j, k)];
                const double *nxm = &c.Cnx[F.x(i - 1, j, k)], *nxp = &c.Cnx[F.x(i, j, k)];
                const double *pym = &c.Cpy[F.y(i, j - 1, k)], *pyp = &c.Cpy[F.y(i, j, k)];
                const double *nym = &c.Cny[F.y(i, j - 1, k)], *nyp = &c.Cny[F.y(i, j, k)];
                const double *pzm = &c.Cpz[F.z(i, j, k - 1)], *pzp = &c.Cpz[F.z(i, j, k)];
                const double *nzm = &c.Cnz[F.z(i, j, k - 1)], *nzp = &c.Cnz[F.z(i, j, k)];
                double *out = &c.Cx[F.cell(i, j, k)];
                for (int m = 0; m < 6; ++m)
                    out[m] = s3 * pxm[m] + s1 * pxp[m] + s4 * nxm[m] + s2 * nxp[m]
                             + s7 * pym[m] + s5 * pyp[m] + s8 * nym[m] + s6 * nyp[m]
                             + s11 * pzm[m] + s9 * pzp[m] + s12 * nzm[m] + s10 * nzp[m];
            }
}

// Peterlin factor, fenep.f90:510-515
inline double peterlin3(const double *x, double lp2) { return (lp2 - 3) / (lp2 - x[0] - x[3] - x[5]); }

// fenep.f90:588-605; A is the transposed velocity-gradient matrix, A[r][c].
inline void lyap_func3(const double A0[3][3], const double *b, const double *x, double *l, double lp2, double dt, double wi) {
    double A[3][3];
    for (int r = 0; r < 3; ++r) for (int q = 0; q < 3; ++q) A[r][q] = A0[r][q];
    double fx = peterlin3(x, lp2);
    double dd = (1.0 + fx * dt / wi) / 2.0;
    A[0][0] = A[0][0] + dd;
    A[1][1] = A[1][1] + dd;
    A[2][2] = A[2][2] + dd;
    l[0] = (A[0][0] + A[0][0]) * x[0] + A[0][1] * x[1] + A[0][2] * x[2] + A[0][1] * x[1] + A[0][2] * x[2] - b[0];
    l[1] = A[1][0] * x[0] + (A[1][1] + A[0][0]) * x[1] + A[1][2] * x[2] + A[0][1] * x[3] + A[0][2] * x[4] - b[1];
    l[2] = A[2][0] * x[0] + A[2][1] * x[1] + (A[2][2] + A[0][0]) * x[2] + A[0][1] * x[4] + A[0][2] * x[5] - b[2];
    l[3] = A[1][0] * x[1] + A[1][0] * x[1] + (A[1][1] + A[1][1]) * x[3] + A[1][2] * x[4] + A[1][2] * x[4] - b[3];
    l[4] = A[1][0] * x[2] + A[2][0] * x[1] + A[2][1] * x[3] + (A[2][2] + A[1][1]) * x[4] + A[1][2] * x[5] - b[4];
    l[5] = A[2][0] * x[2] + A[2][1] * x[4] + A[2][0] * x[2] + A[2][1] * x[4] + (A[2][2] + A[2][2]) * x[5] - b[5];
}

// Gauss-Jordan elimination with partial pivoting, fenep.f90:608-643 (n = 6)
// and fenep_2d.f90:358-393 (n = 3).  Ah is row-major n x (n+1).
template <int N>
void gauss(double Ah[N][N + 1], double *x) {
    for (int k = 0; k < N; ++k) {
        int maxidx = k; double maxabs = std::fabs(Ah[k][k]);
        for (int r = k + 1; r < N; ++r) {
            double a = std::fabs(Ah[r][k]);
            if (a > maxabs) { maxabs = a; maxidx = r; }
        }
        if (maxabs == 0.0) {
            for (int r = 0; r < N; ++r) Ah[r][N] = 0.0;
            break;
        }
        if (k != maxidx)
            for (int q = k; q <= N; ++q) std::swap(Ah[k][q], Ah[maxidx][q]);
        double piv = Ah[k][k];
        for (int q = k + 1; q <= N; ++q) Ah[k][q] = Ah[k][q] / piv;
        Ah[k][k] = 1.0;
        for (int r = 0; r < N; ++r) {
            if (r == k) continue;
            double f = Ah[r][k];
            for (int q = k + 1; q <= N; ++q) Ah[r][q] = Ah[r][q] - f * Ah[k][q];
            Ah[r][k] = 0.0;
        }
    }
    for (int r = 0; r < N; ++r) x[r] = Ah[r][N];
}

// fenep.f90:518-585, one cell.  Returns the iteration count (itrmax+1 when the
// loop ran out, as the Fortran do-variable does).
int newton_cell3(const double A0T[3][3], const double *b, double *x, const f8_phys &ph) {
    const double dc = ph.newton_dc, eps = ph.newton_eps;
    int itr;
    for (itr = 1; itr <= ph.newton_itrmax; ++itr) {
        double Ah[6][7], x1[6], x2[6], l1[6], l2[6], l[6], r[6];
        for (int col = 0; col < 6; ++col) {
            for (int m = 0; m < 6; ++m) { x1[m] = x[m]; x2[m] = x[m]; }
            x1[col] = x1[col] + dc;
            x2[col] = x2[col] - dc;
            lyap_func3(A0T, b, x1, l1, ph.lp2, ph.dt, ph.wi);
            lyap_func3(A0T, b, x2, l2, ph.lp2, ph.dt, ph.wi);
            for (int row = 0; row < 6; ++row) Ah[row][col] = (l1[row] - l2[row]) / (2.0 * dc);
        }
        lyap_func3(A0T, b, x, l, ph.lp2, ph.dt, ph.wi);
        for (int row = 0; row < 6; ++row) Ah[row][6] = l[row];
        gauss<6>(Ah, r);
        for (int m = 0; m < 6; ++m) x[m] = x[m] - r[m];
        double sr = 0, sx = 0;
        for (int m = 0; m < 6; ++m) sr = sr + r[m] * r[m];
        for (int m = 0; m < 6; ++m) sx = sx + x[m] * x[m];
        if (std::sqrt(sr / sx) < eps) break;
    }
    return itr;
}

// fenep.f90:518-585
void lyapunov3(OCtx &c) {
    const int NX = c.NX, NZ = c.NZ, jlo = prow_lo(c), jhi = prow_hi(c);
    const FaceIdx F = face_idx(c);
    const double dt = c.ph.dt, wi = c.ph.wi, dX = c.dX, dY = c.dY, dZ = c.dZ;
    const double *U = c.U.data(), *V = c.V.data(), *W = c.W.data();
    long long iters = 0, unconv = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : iters, unconv)
    for (int k = 1; k <= NZ; ++k)
        for (int j = jlo; j <= jhi; ++j)
            for (int i = 1; i <= NX; ++i) {
                double b[6];
                const double *cx = &c.Cx[F.cell(i, j, k)];
                for (int m = 0; m < 6; ++m) b[m] = cx[m];
                b[0] = b[0] + dt / wi;
                b[3] = b[3] + dt / wi;
                b[5] = b[5] + dt / wi;
                auto u = [&](int a, int bb, int cc) { return vval(c, U, a, bb, cc); };
                auto v = [&](int a, int bb, int cc) { return vval(c, V, a, bb, cc); };
                auto w = [&](int a, int bb, int cc) { return vval(c, W, a, bb, cc); };
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
                double AT[3][3];
                for (int r = 0; r < 3; ++r) for (int q = 0; q < 3; ++q) AT[r][q] = A0[q][r];
                double x[6];
                double *cc = &c.C[6 * c.hidx(i, j, k)];
                for (int m = 0; m < 6; ++m) x[m] = cc[m];
                int itr = newton_cell3(AT, b, x, c.ph);
                iters += itr;
                if (itr > c.ph.newton_itrmax) unconv += 1;
                double *outp = &c.C0[6 * c.hidx(i, j, k)];  // new C goes to a side buffer
                for (int m = 0; m < 6; ++m) outp[m] = x[m];
            }
    // copy the new values back (the reference overwrites C in place; each cell
    // reads only its own old value, so the result is the same)
    for (int k = 1; k <= NZ; ++k)
        for (int j = jlo; j <= jhi; ++j)
            for (int i = 1; i <= NX; ++i)
                for (int m = 0; m < 6; ++m) c.C[6 * c.hidx(i, j, k) + m] = c.C0[6 * c.hidx(i, j, k) + m];
    // C_PBM after Lyapunov (fenep_2d.f90:348): with walls only the periodic
    // x and z copies (the ghost rows keep their updated values)
    if (c.walls) {
        bc_periodic_xz(c, c.C.data(), 6);
        bc_periodic_z(c, c.C.data(), 6);
    } else {
        bc_c(c, c.C.data());
    }
    c.newton_iters += iters;
    c.newton_unconv += unconv;
}

// fenep.f90:645-691.  C0 = f(C) C - I on every cell (interior and halo: the
// halo of C already holds the boundary values, so this equals C_PBM(C0) on
// periodic sides and evaluates the stress from the extrapolated ghost C at
// walls).
void polymer_stress3(OCtx &c) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double E[6] = {1.0, 0.0, 0.0, 1.0, 0.0, 1.0};
    double *C0 = c.C0.data();
    const double *C = c.C.data();
    for (size_t n = 0; n < c.nh(); ++n) {
        double f = peterlin3(C + 6 * n, c.ph.lp2);
        for (int m = 0; m < 6; ++m) C0[6 * n + m] = f * C[6 * n + m] - E[m];
    }
    const double dX = c.dX, dY = c.dY, dZ = c.dZ;
    const double coef = (1.0 - c.ph.beta) / (c.ph.re * c.ph.wi);
    auto c0 = [&](int m, int i, int j, int k) { return C0[(m - 1) + 6 * c.hidx(i, j, k)]; };
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) {
                size_t o = c.iidx(i, j, k);
                double tx = (-c0(1, i, j, k) + c0(1, i + 1, j, k)) / dX
                          + (-c0(2, i, j - 1, k) - c0(2, i + 1, j - 1, k) + c0(2, i, j + 1, k) + c0(2, i + 1, j + 1, k)) / (4 * dY)
                          + (-c0(3, i, j, k - 1) - c0(3, i + 1, j, k - 1) + c0(3, i, j, k + 1) + c0(3, i + 1, j, k + 1)) / (4 * dZ);
                double ty = (-c0(2, i - 1, j, k) + c0(2, i + 1, j, k) - c0(2, i - 1, j + 1, k) + c0(2, i + 1, j + 1, k)) / (4 * dX)
                          + (-c0(4, i, j, k) + c0(4, i, j + 1, k)) / dY
                          + (-c0(5, i, j, k - 1) - c0(5, i, j + 1, k - 1) + c0(5, i, j, k + 1) + c0(5, i, j + 1, k + 1)) / (4 * dZ);
                double tz = (-c0(3, i - 1, j, k) + c0(3, i + 1, j, k) - c0(3, i - 1, j, k + 1) + c0(3, i + 1, j, k + 1)) / (4 * dX)
                          + (-c0(5, i, j - 1, k) + c0(5, i, j + 1, k) - c0(5, i, j - 1, k + 1) + c0(5, i, j + 1, k + 1)) / (4 * dY)
                          + (-c0(6, i, j, k) + c0(6, i, j, k + 1)) / dZ;
                c.Tx[o] = coef * tx;
                c.Ty[o] = coef * ty;
                c.Tz[o] = coef * tz;
            }
}

// ---------------------------------------------------------------------------
// 2D polymer (fenep_2d.f90:138-393).  C has 3 components (xx, xy, yy).

inline void eig2(const double *a, double &re1, double &re2) {  // fenep_2d.f90:229-238
    double d = (a[0] - a[2]) * (a[0] - a[2]) + 4.0 * (a[1] * a[1]);
    double s = std::sqrt(d);
    re1 = (a[0] + a[2] + s) * 0.5;
    re2 = (a[0] + a[2] - s) * 0.5;
}

// fenep_2d.f90:145-176 for one direction.  The 2D selection keeps the LAST
// candidate whose smallest eigenvalue is >= the running best (starting at 0);
// index 0 means none qualified and the cell value is used.
int reconstruct2(const double *cm, const double *c0, const double *cp, double *fp, double *fn) {
    double pt[3][3], nt[3][3];
    for (int m = 0; m < 3; ++m) {
        pt[0][m] = c0[m] * 3 / 2 - cp[m] / 2;
        nt[0][m] = c0[m] / 2 + cp[m] / 2;
        pt[1][m] = cm[m] / 2 + c0[m] / 2;
        nt[1][m] = -cm[m] / 2 + c0[m] * 3 / 2;
        pt[2][m] = cm[m] / 4 + c0[m] - cp[m] / 4;
        nt[2][m] = -cm[m] / 4 + c0[m] + cp[m] / 4;
    }
    int index = 0; double mintemp = 0.0;
    for (int l = 0; l < 3; ++l) {
        double e[4];
        eig2(pt[l], e[0], e[1]);
        eig2(nt[l], e[2], e[3]);
        // minval over 4 values, NaN ignored
        double mv = e[0];
        bool found = !std::isnan(mv);
        for (int q = 1; q < 4; ++q) {
            if (std::isnan(e[q])) continue;
            if (!found || e[q] < mv) { mv = e[q]; found = true; }
        }
        if (found && mv >= mintemp) { index = l + 1; mintemp = mv; }
    }
    if (index > 0) {
        for (int m = 0; m < 3; ++m) { fp[m] = pt[index - 1][m]; fn[m] = nt[index - 1][m]; }
    } else {
        for (int m = 0; m < 3; ++m) { fp[m] = c0[m]; fn[m] = c0[m]; }
    }
    return index;
}

inline double peterlin2(const double *x, double lp2) { return (lp2 - 2) / (lp2 - x[0] - x[2]); }

inline void lyap_func2(const double A0[2][2], const double *b, const double *x, double *l, double lp2, double dt, double wi) {
    double A[2][2] = {{A0[0][0], A0[0][1]}, {A0[1][0], A0[1][1]}};
    double fx = peterlin2(x, lp2);
    double dd = (1.0 + fx * dt / wi) / 2.0;
    A[0][0] = A[0][0] + dd;
    A[1][1] = A[1][1] + dd;
    l[0] = (A[0][0] + A[0][0]) * x[0] + A[0][1] * x[1] + A[0][1] * x[1] - b[0];
    l[1] = A[1][0] * x[0] + (A[1][1] + A[0][0]) * x[1] + A[0][1] * x[2] - b[1];
    l[2] = A[1][0] * x[1] + A[1][0] * x[1] + (A[1][1] + A[1][1]) * x[2] - b[2];
}

int newton_cell2(const double A0T[2][2], const double *b, double *x, const f8_phys &ph) {
    const double dc = ph.newton_dc, eps = ph.newton_eps;
    int itr;
    for (itr = 1; itr <= ph.newton_itrmax; ++itr) {
        double Ah[3][4], x1[3], x2[3], l1[3], l2[3], l[3], r[3];
        for (int col = 0; col < 3; ++col) {
            for (int m = 0; m < 3; ++m) { x1[m] = x[m]; x2[m] = x[m]; }
            x1[col] = x1[col] + dc;
            x2[col] = x2[col] - dc;
            lyap_func2(A0T, b, x1, l1, ph.lp2, ph.dt, ph.wi);
            lyap_func2(A0T, b, x2, l2, ph.lp2, ph.dt, ph.wi);
            for (int row = 0; row < 3; ++row) Ah[row][col] = (l1[row] - l2[row]) / (2.0 * dc);
        }
        lyap_func2(A0T, b, x, l, ph.lp2, ph.dt, ph.wi);
        for (int row = 0; row < 3; ++row) Ah[row][3] = l[row];
        gauss<3>(Ah, r);
        for (int m = 0; m < 3; ++m) x[m] = x[m] - r[m];
        double sr = 0, sx = 0;
        for (int m = 0; m < 3; ++m) sr = sr + r[m] * r[m];
        for (int m = 0; m < 3; ++m) sx = sx + x[m] * x[m];
        if (std::sqrt(sr / sx) < eps) break;
    }
    return itr;
}

// 2D polymer update: CpxCnx, CpyCny, Cstar (1/4 weights), Lyapunov.
void polymer2(OCtx &c) {
    const int NX = c.NX, NY = c.NY;
    const int k = 1;
    const bool ext = c.walls;   // ghost rows updated too (see prow_lo)
    const int jlo = prow_lo(c), jhi = prow_hi(c);
    const double *C = c.C.data();
    auto cp_ = [&](int i, int j) { return cval(c, C, 3, i, j, k); };
    const int nr = jhi - jlo + 1;
    std::vector<double> Cpx(3 * (NX + 1) * nr), Cnx(3 * (NX + 1) * nr), Cpy(3 * NX * (nr + 1), 0.0), Cny(3 * NX * (nr + 1), 0.0);
    auto fx = [&](int f, int j) { return (size_t)3 * ((size_t)f + (size_t)(NX + 1) * (j - jlo)); };
    auto fy = [&](int i, int f) { return (size_t)3 * ((size_t)(i - 1) + (size_t)NX * (f - (jlo - 1))); };
    c.codes.assign((size_t)NX * nr, 0);
    for (int j = jlo; j <= jhi; ++j)
        for (int i = 1; i <= NX; ++i) {
            const double *c0 = cp_(i, j);
            const int ix = reconstruct2(cp_(i - 1, j), c0, cp_(i + 1, j), &Cpx[fx(i - 1, j)], &Cnx[fx(i, j)]);
            const int iy = reconstruct2(cp_(i, j - 1), c0, cp_(i, j + 1), &Cpy[fy(i, j - 1)], &Cny[fy(i, j)]);
            // index 0 (no candidate qualified: the cell value) is stored as 3
            c.codes[(size_t)(i - 1) + (size_t)NX * (j - jlo)] =
                (unsigned char)((ix == 0 ? 3 : ix - 1) | ((iy == 0 ? 3 : iy - 1) << 2));
        }
    for (int j = jlo; j <= jhi; ++j)
        for (int m = 0; m < 3; ++m) {
            Cpx[fx(NX, j) + m] = Cpx[fx(0, j) + m];
            Cnx[fx(0, j) + m] = Cnx[fx(NX, j) + m];
        }
    for (int i = 1; i <= NX; ++i)
        for (int m = 0; m < 3; ++m) {
            if (!c.walls) {
                Cpy[fy(i, NY) + m] = Cpy[fy(i, 0) + m];
                Cny[fy(i, 0) + m] = Cny[fy(i, NY) + m];
            } else {
                Cpy[fy(i, jhi) + m] = 0.0;
                Cny[fy(i, jlo - 1) + m] = 0.0;
            }
        }
    const double dt = c.ph.dt, wi = c.ph.wi, dX = c.dX, dY = c.dY;
    const double *U = c.U.data(), *V = c.V.data();
    long long iters = 0, unconv = 0;
    std::vector<double> Cn(3 * NX * nr);
    for (int j = jlo; j <= jhi; ++j)
        for (int i = 1; i <= NX; ++i) {
            auto u = [&](int a, int bb) { return vval(c, U, a, bb, k); };
            auto v = [&](int a, int bb) { return vval(c, V, a, bb, k); };
            double u1 = u(i - 1, j), u2 = u(i, j);
            double v1 = v(i, j - 1), v2 = v(i, j);
            double s1 = (-u2 + std::fabs(u2)) * dt / (2 * dX);
            double s2 = 1.0 / 4 + (-u2 - std::fabs(u2)) * dt / (2 * dX);
            double s3 = 1.0 / 4 + (u1 - std::fabs(u1)) * dt / (2 * dX);
            double s4 = (u1 + std::fabs(u1)) * dt / (2 * dX);
            double s5 = (-v2 + std::fabs(v2)) * dt / (2 * dY);
            double s6 = 1.0 / 4 + (-v2 - std::fabs(v2)) * dt / (2 * dY);
            double s7 = 1.0 / 4 + (v1 - std::fabs(v1)) * dt / (2 * dY);
            double s8 = (v1 + std::fabs(v1)) * dt / (2 * dY);
            double b[3];
            for (int m = 0; m < 3; ++m)
                b[m] = s3 * Cpx[fx(i - 1, j) + m] + s1 * Cpx[fx(i, j) + m] + s4 * Cnx[fx(i - 1, j) + m] + s2 * Cnx[fx(i, j) + m]
                       + s7 * Cpy[fy(i, j - 1) + m] + s5 * Cpy[fy(i, j) + m] + s8 * Cny[fy(i, j - 1) + m] + s6 * Cny[fy(i, j) + m];
            b[0] = b[0] + dt / wi;
            b[2] = b[2] + dt / wi;
            double A0[2][2];
            A0[0][0] = -dt * (-u(i - 1, j) + u(i, j)) / dX;
            A0[0][1] = -dt * (-v(i - 1, j - 1) + v(i + 1, j - 1) - v(i - 1, j) + v(i + 1, j)) / (4 * dX);
            A0[1][0] = -dt * (-u(i - 1, j - 1) - u(i, j - 1) + u(i - 1, j + 1) + u(i, j + 1)) / (4 * dY);
            A0[1][1] = -dt * (-v(i, j - 1) + v(i, j)) / dY;
            double AT[2][2] = {{A0[0][0], A0[1][0]}, {A0[0][1], A0[1][1]}};
            double x[3];
            for (int m = 0; m < 3; ++m) x[m] = C[3 * c.hidx(i, j, k) + m];
            int itr = newton_cell2(AT, b, x, c.ph);
            iters += itr;
            if (itr > c.ph.newton_itrmax) unconv += 1;
            for (int m = 0; m < 3; ++m) Cn[3 * ((i - 1) + NX * (j - jlo)) + m] = x[m];
        }
    for (int j = jlo; j <= jhi; ++j)
        for (int i = 1; i <= NX; ++i)
            for (int m = 0; m < 3; ++m) c.C[3 * c.hidx(i, j, k) + m] = Cn[3 * ((i - 1) + NX * (j - jlo)) + m];
    if (ext) bc_periodic_xz(c, c.C.data(), 3);
    else bc_c(c, c.C.data());
    c.newton_iters += iters;
    c.newton_unconv += unconv;
}

// fenep_2d.f90:396-427
void polymer_stress2(OCtx &c) {
    const int NX = c.NX, NY = c.NY, k = 1;
    const double E[3] = {1.0, 0.0, 1.0};
    double *C0 = c.C0.data();
    const double *C = c.C.data();
    for (size_t n = 0; n < c.nh(); ++n) {
        double f = peterlin2(C + 3 * n, c.ph.lp2);
        for (int m = 0; m < 3; ++m) C0[3 * n + m] = f * C[3 * n + m] - E[m];
    }
    const double dX = c.dX, dY = c.dY;
    const double coef = (1.0 - c.ph.beta) / (c.ph.re * c.ph.wi);
    auto c0 = [&](int m, int i, int j) { return C0[(m - 1) + 3 * c.hidx(i, j, k)]; };
    for (int j = 1; j <= NY; ++j)
        for (int i = 1; i <= NX; ++i) {
            size_t o = c.iidx(i, j, k);
            double tx = (-c0(1, i, j) + c0(1, i + 1, j)) / dX
                      + (-c0(2, i, j - 1) - c0(2, i + 1, j - 1) + c0(2, i, j + 1) + c0(2, i + 1, j + 1)) / (4 * dY);
            double ty = (-c0(2, i - 1, j) + c0(2, i + 1, j) - c0(2, i - 1, j + 1) + c0(2, i + 1, j + 1)) / (4 * dX)
                      + (-c0(3, i, j) + c0(3, i, j + 1)) / dY;
            c.Tx[o] = coef * tx;
            c.Ty[o] = coef * ty;
            c.Tz[o] = 0.0;
        }
}

// ---------------------------------------------------------------------------
// Momentum: convection (fenep.f90:694-734) and viscous (736-770).  In 2D the
// z terms are dropped (fenep_2d.f90:430-475).
void convection_viscous(OCtx &c) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double dX = c.dX, dY = c.dY, dZ = c.dZ;
    const double *U = c.U.data(), *V = c.V.data(), *W = c.W.data();
    const bool d3 = c.dim == 3;
    const double vis = c.ph.beta / c.ph.re;
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) {
                auto u = [&](int a, int b, int cc) { return U[c.hidx(a, b, cc)]; };
                auto v = [&](int a, int b, int cc) { return V[c.hidx(a, b, cc)]; };
                auto w = [&](int a, int b, int cc) { return W[c.hidx(a, b, cc)]; };
                size_t o = c.iidx(i, j, k);
                double t1 = (u(i - 1, j, k) + u(i, j, k)) / 2, t2 = (u(i, j, k) + u(i + 1, j, k)) / 2;
                double ax = (-(t1 * t1) + t2 * t2) / dX
                          + (-(v(i, j - 1, k) + v(i + 1, j - 1, k)) / 2 * (u(i, j - 1, k) + u(i, j, k)) / 2
                             + (v(i, j, k) + v(i + 1, j, k)) / 2 * (u(i, j, k) + u(i, j + 1, k)) / 2) / dY;
                double t3 = (v(i, j - 1, k) + v(i, j, k)) / 2, t4 = (v(i, j, k) + v(i, j + 1, k)) / 2;
                double ay = (-(u(i - 1, j, k) + u(i - 1, j + 1, k)) / 2 * (v(i - 1, j, k) + v(i, j, k)) / 2
                             + (u(i, j, k) + u(i, j + 1, k)) / 2 * (v(i, j, k) + v(i + 1, j, k)) / 2) / dX
                          + (-(t3 * t3) + t4 * t4) / dY;
                double bx = (u(i - 1, j, k) - 2 * u(i, j, k) + u(i + 1, j, k)) / (dX * dX)
                          + (u(i, j - 1, k) - 2 * u(i, j, k) + u(i, j + 1, k)) / (dY * dY);
                double by = (v(i - 1, j, k) - 2 * v(i, j, k) + v(i + 1, j, k)) / (dX * dX)
                          + (v(i, j - 1, k) - 2 * v(i, j, k) + v(i, j + 1, k)) / (dY * dY);
                double az = 0, bz = 0;
                if (d3) {
                    ax = ax + (-(w(i, j, k - 1) + w(i + 1, j, k - 1)) / 2 * (u(i, j, k - 1) + u(i, j, k)) / 2
                               + (w(i, j, k) + w(i + 1, j, k)) / 2 * (u(i, j, k) + u(i, j, k + 1)) / 2) / dZ;
                    ay = ay + (-(w(i, j, k - 1) + w(i, j + 1, k - 1)) / 2 * (v(i, j, k - 1) + v(i, j, k)) / 2
                               + (w(i, j, k) + w(i, j + 1, k)) / 2 * (v(i, j, k) + v(i, j, k + 1)) / 2) / dZ;
                    double t5 = (w(i, j, k - 1) + w(i, j, k)) / 2, t6 = (w(i, j, k) + w(i, j, k + 1)) / 2;
                    az = (-(u(i - 1, j, k) + u(i - 1, j, k + 1)) / 2 * (w(i - 1, j, k) + w(i, j, k)) / 2
                          + (u(i, j, k) + u(i, j, k + 1)) / 2 * (w(i, j, k) + w(i + 1, j, k)) / 2) / dX
                       + (-(v(i, j - 1, k) + v(i, j - 1, k + 1)) / 2 * (w(i, j - 1, k) + w(i, j, k)) / 2
                          + (v(i, j, k) + v(i, j, k + 1)) / 2 * (w(i, j, k) + w(i, j + 1, k)) / 2) / dY
                       + (-(t5 * t5) + t6 * t6) / dZ;
                    bx = bx + (u(i, j, k - 1) - 2 * u(i, j, k) + u(i, j, k + 1)) / (dZ * dZ);
                    by = by + (v(i, j, k - 1) - 2 * v(i, j, k) + v(i, j, k + 1)) / (dZ * dZ);
                    bz = (w(i - 1, j, k) - 2 * w(i, j, k) + w(i + 1, j, k)) / (dX * dX)
                       + (w(i, j - 1, k) - 2 * w(i, j, k) + w(i, j + 1, k)) / (dY * dY)
                       + (w(i, j, k - 1) - 2 * w(i, j, k) + w(i, j, k + 1)) / (dZ * dZ);
                }
                c.Ax[o] = -ax; c.Ay[o] = -ay; c.Az[o] = -az;
                c.Bx[o] = vis * bx; c.By[o] = vis * by; c.Bz[o] = vis * bz;
            }
}

// ---------------------------------------------------------------------------
// FFT: radix-2 Stockham, unnormalised, sign -1 forward / +1 backward.
struct Tw { const double *r, *i; };

// In-place transform of one line (re[n], im[n]) using scratch of the same size.
void fft_line(double *re, double *im, int n, Tw tw, int sign, double *sr, double *si) {
    double *xr = re, *xi = im, *yr = sr, *yi = si;
    const int half = n / 2;
    for (int ns = 1; ns < n; ns *= 2) {
        const int stride = n / (2 * ns);
        for (int j = 0; j < half; ++j) {
            int kk = j % ns;
            double wr = tw.r[kk * stride], wi = sign < 0 ? tw.i[kk * stride] : -tw.i[kk * stride];
            double ar = xr[j], ai = xi[j], br = xr[j + half], bi = xi[j + half];
            double tr = br * wr - bi * wi, ti = br * wi + bi * wr;
            int o = (j / ns) * 2 * ns + kk;
            yr[o] = ar + tr; yi[o] = ai + ti;
            yr[o + ns] = ar - tr; yi[o + ns] = ai - ti;
        }
        std::swap(xr, yr); std::swap(xi, yi);
    }
    if (xr != re) {
        std::memcpy(re, xr, sizeof(double) * n);
        std::memcpy(im, xi, sizeof(double) * n);
    }
}

// Forward twiddles exp(-2 pi i t/n) for t < n/2.
void make_tw(int n, std::vector<double> &r, std::vector<double> &i) {
    r.resize(std::max(1, n / 2)); i.resize(std::max(1, n / 2));
    for (int t = 0; t < n / 2; ++t) {
        double a = 2.0 * PI * t / n;
        r[t] = std::cos(a);
        i[t] = -std::sin(a);
    }
    if (n / 2 == 0) { r[0] = 1.0; i[0] = 0.0; }
}

// Spectral array: H[(kx + NXH*(j + nj*k)) * 2] complex, NXH = NX/2+1.
// Forward x transform of rows j in [j0, j0+nj) (interior x) for all k.
// Two real rows a, b are transformed as one complex row a + i b.
void fft_x_forward(OCtx &c, const std::vector<double> &src_int, int j0, int nj, std::vector<double> &H) {
    const int NX = c.NX, NXH = NX / 2 + 1, NZ = c.NZ;
    Tw tw{c.twx_r.data(), c.twx_i.data()};
    std::vector<double> zr(NX), zi(NX), sr(NX), si(NX);
    for (int k = 0; k < NZ; ++k)
        for (int jj = 0; jj < nj; jj += 2) {
            int ja = j0 + jj, jb = j0 + jj + 1;
            for (int i = 0; i < NX; ++i) {
                zr[i] = src_int[(size_t)i + NX * ((size_t)(ja - 1) + (size_t)c.NY * k)];
                zi[i] = src_int[(size_t)i + NX * ((size_t)(jb - 1) + (size_t)c.NY * k)];
            }
            fft_line(zr.data(), zi.data(), NX, tw, -1, sr.data(), si.data());
            for (int kx = 0; kx < NXH; ++kx) {
                int m = (NX - kx) % NX;
                double ar = (zr[kx] + zr[m]) * 0.5, ai = (zi[kx] - zi[m]) * 0.5;
                double br = (zi[kx] + zi[m]) * 0.5, bi = (zr[m] - zr[kx]) * 0.5;
                size_t oa = 2 * ((size_t)kx + NXH * ((size_t)jj + (size_t)nj * k));
                size_t ob = 2 * ((size_t)kx + NXH * ((size_t)(jj + 1) + (size_t)nj * k));
                H[oa] = ar; H[oa + 1] = ai; H[ob] = br; H[ob + 1] = bi;
            }
        }
}

// Inverse x transform of spectral rows [0, nj) into halo rows jdst0.. of dst.
void fft_x_inverse(OCtx &c, const std::vector<double> &H, int nj, double *dst, int jdst0) {
    const int NX = c.NX, NXH = NX / 2 + 1, NZ = c.NZ;
    Tw tw{c.twx_r.data(), c.twx_i.data()};
    std::vector<double> zr(NX), zi(NX), sr(NX), si(NX);
    for (int k = 0; k < NZ; ++k)
        for (int jj = 0; jj < nj; jj += 2) {
            size_t ra = 2 * (NXH * ((size_t)jj + (size_t)nj * k));
            size_t rb = 2 * (NXH * ((size_t)(jj + 1) + (size_t)nj * k));
            for (int kx = 0; kx < NX; ++kx) {
                if (kx <= NX / 2) {
                    double ar = H[ra + 2 * kx], ai = H[ra + 2 * kx + 1], br = H[rb + 2 * kx], bi = H[rb + 2 * kx + 1];
                    zr[kx] = ar - bi; zi[kx] = ai + br;
                } else {
                    int m = NX - kx;
                    double ar = H[ra + 2 * m], ai = H[ra + 2 * m + 1], br = H[rb + 2 * m], bi = H[rb + 2 * m + 1];
                    zr[kx] = ar + bi; zi[kx] = br - ai;
                }
            }
            fft_line(zr.data(), zi.data(), NX, tw, +1, sr.data(), si.data());
            for (int i = 0; i < NX; ++i) {
                dst[c.hidx(i + 1, jdst0 + jj, k + 1)] = zr[i];
                dst[c.hidx(i + 1, jdst0 + jj + 1, k + 1)] = zi[i];
            }
        }
}

// c2c transform along y (stride NXH) for all kx, k; rows [0, nj).
void fft_y(OCtx &c, std::vector<double> &H, int nj, int sign) {
    const int NXH = c.NX / 2 + 1, NZ = c.NZ, n = nj;
    Tw tw{c.twy_r.data(), c.twy_i.data()};
    std::vector<double> lr(n), li(n), sr(n), si(n);
    for (int k = 0; k < NZ; ++k)
        for (int kx = 0; kx < NXH; ++kx) {
            for (int j = 0; j < n; ++j) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)nj * k));
                lr[j] = H[o]; li[j] = H[o + 1];
            }
            fft_line(lr.data(), li.data(), n, tw, sign, sr.data(), si.data());
            for (int j = 0; j < n; ++j) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)nj * k));
                H[o] = lr[j]; H[o + 1] = li[j];
            }
        }
}

void fft_z(OCtx &c, std::vector<double> &H, int nj, int sign) {
    const int NXH = c.NX / 2 + 1, NZ = c.NZ;
    if (NZ == 1) return;
    Tw tw{c.twz_r.data(), c.twz_i.data()};
    std::vector<double> lr(NZ), li(NZ), sr(NZ), si(NZ);
    for (int j = 0; j < nj; ++j)
        for (int kx = 0; kx < NXH; ++kx) {
            for (int k = 0; k < NZ; ++k) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)nj * k));
                lr[k] = H[o]; li[k] = H[o + 1];
            }
            fft_line(lr.data(), li.data(), NZ, tw, sign, sr.data(), si.data());
            for (int k = 0; k < NZ; ++k) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)nj * k));
                H[o] = lr[k]; H[o + 1] = li[k];
            }
        }
}

// Periodic fft_solve (fenep.f90:1400-1428): Phi = IFFT( FFT(Q)/N / LHS ).
// LHS(i,j,k) = lhs0 + lhs1*((kx2(i) + ky2(j)) + kz2(k)).
// Q is interior-ordered; the result is written to the interior of dst.
void fft_solve_periodic(OCtx &c, const std::vector<double> &Qv, double lhs0, double lhs1, double *dst) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ, NXH = NX / 2 + 1;
    std::vector<double> H((size_t)2 * NXH * NY * NZ);
    fft_x_forward(c, Qv, 1, NY, H);
    fft_y(c, H, NY, -1);
    fft_z(c, H, NY, -1);
    const double ntot = (double)(NX * NY * NZ);
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int kx = 0; kx < NXH; ++kx) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)NY * k));
                double lhs = lhs0 + lhs1 * (c.kx2[kx] + c.ky2[j] + c.kz2[k]);
                double qr = H[o] / ntot, qi = H[o + 1] / ntot;
                if (std::fabs(lhs) < 1.0e-16) { H[o] = 0.0; H[o + 1] = 0.0; }
                else { H[o] = qr / lhs; H[o + 1] = qi / lhs; }
            }
    fft_z(c, H, NY, +1);
    fft_y(c, H, NY, +1);
    fft_x_inverse(c, H, NY, dst, 1);
}

// Thomas solve of fenep_2d.f90:1145-1177 for a system whose coefficients are
// real (a, b, c) and right-hand side complex (dr, di).  a x_i + b x_{i+1} +
// c x_{i-1} = d_i.  The near-zero-pivot guard is the reference's.
void tdma(int n, const double *a, const double *b, const double *cc, const double *dr, const double *di,
          double *xr, double *xi, double *P, double *Qr, double *Qi) {
    P[0] = -b[0] / a[0];
    Qr[0] = dr[0] / a[0];
    Qi[0] = di[0] / a[0];
    for (int i = 1; i < n; ++i) {
        double den = a[i] + cc[i] * P[i - 1];
        if (std::fabs(den) < 1.0e-16) {
            P[i] = 0.0; Qr[i] = 0.0; Qi[i] = 0.0;
        } else {
            P[i] = -b[i] / den;
            Qr[i] = (dr[i] - cc[i] * Qr[i - 1]) / den;
            Qi[i] = (di[i] - cc[i] * Qi[i - 1]) / den;
        }
    }
    xr[n - 1] = Qr[n - 1]; xi[n - 1] = Qi[n - 1];
    for (int i = n - 2; i >= 0; --i) {
        xr[i] = P[i] * xr[i + 1] + Qr[i];
        xi[i] = P[i] * xi[i + 1] + Qi[i];
    }
}

enum WallSys { SYS_U, SYS_V, SYS_P };

// Wall-bounded solve (fenep_2d.f90:1179-1342 generalised to x,z periodic):
// FFT in x and z of rows j = 1..NY, one tridiagonal system per (kx,kz) over
// the rows j = 0..NY+1 (ghosts included), inverse FFT of all NY+2 rows into
// dst (halo layout, rows 0..NY+1).
void wall_solve(OCtx &c, const std::vector<double> &Qv, WallSys sys, double uwall, double *dst) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ, NXH = NX / 2 + 1, n = NY + 2;
    std::vector<double> Hin((size_t)2 * NXH * NY * NZ), Hout((size_t)2 * NXH * n * NZ);
    fft_x_forward(c, Qv, 1, NY, Hin);
    fft_z(c, Hin, NY, -1);
    const double nxz = (double)(NX * NZ);
    const double dt = c.ph.dt, beta = c.ph.beta, re = c.ph.re, dY = c.dY;
    std::vector<double> a(n), b(n), cc(n), dr(n), di(n), xr(n), xi(n), P(n), Qr(n), Qi(n);
    for (int k = 0; k < NZ; ++k)
        for (int kx = 0; kx < NXH; ++kx) {
            double lam = c.kx2[kx] + c.kz2[k];
            for (int j = 1; j <= NY; ++j) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)(j - 1) + (size_t)NY * k));
                dr[j] = Hin[o] / nxz; di[j] = Hin[o + 1] / nxz;
            }
            if (sys == SYS_U) {
                for (int j = 1; j <= NY; ++j) {
                    a[j] = 1.0 + dt * beta / re / 2.0 * (lam + 2.0 / (dY * dY));
                    b[j] = -dt * beta / re / 2.0 / (dY * dY);
                    cc[j] = -dt * beta / re / 2.0 / (dY * dY);
                }
                a[0] = 1.0; b[0] = 1.0; cc[0] = 0.0; dr[0] = 0.0; di[0] = 0.0;
                a[n - 1] = 1.0; cc[n - 1] = 1.0; b[n - 1] = 0.0;
                dr[n - 1] = (kx == 0 && k == 0) ? 2 * uwall : 0.0; di[n - 1] = 0.0;
            } else if (sys == SYS_V) {
                for (int j = 1; j <= NY - 1; ++j) {
                    a[j] = 1.0 + dt * beta / re / 2.0 * (lam + 2.0 / (dY * dY));
                    b[j] = -dt * beta / re / 2.0 / (dY * dY);
                    cc[j] = -dt * beta / re / 2.0 / (dY * dY);
                }
                a[0] = 1.0; b[0] = 0.0; cc[0] = 0.0; dr[0] = 0.0; di[0] = 0.0;
                for (int j = NY; j <= NY + 1; ++j) { a[j] = 1.0; b[j] = 0.0; cc[j] = 0.0; dr[j] = 0.0; di[j] = 0.0; }
            } else {
                for (int j = 1; j <= NY; ++j) {
                    a[j] = -(lam + 2.0 / (dY * dY));
                    b[j] = 1.0 / (dY * dY);
                    cc[j] = 1.0 / (dY * dY);
                }
                a[0] = 1.0; b[0] = -1.0; cc[0] = 0.0; dr[0] = 0.0; di[0] = 0.0;
                a[n - 1] = 1.0; cc[n - 1] = -1.0; b[n - 1] = 0.0; dr[n - 1] = 0.0; di[n - 1] = 0.0;
            }
            tdma(n, a.data(), b.data(), cc.data(), dr.data(), di.data(), xr.data(), xi.data(), P.data(), Qr.data(), Qi.data());
            for (int j = 0; j < n; ++j) {
                size_t o = 2 * ((size_t)kx + NXH * ((size_t)j + (size_t)n * k));
                Hout[o] = xr[j]; Hout[o + 1] = xi[j];
            }
        }
    fft_z(c, Hout, n, +1);
    fft_x_inverse(c, Hout, n, dst, 0);
}

// ---------------------------------------------------------------------------
// IBM.  Marker set per z-plane built from the cylinder list following
// ibm_init (fenep.f90:1784-1899, fenep_2d.f90:1472-1629).  Markers are
// ordered marker-major, cylinder-minor, as the reference's (NC, NL, NZ) arrays
// are walked by do n / do m / do l.

std::vector<Marker2> build_markers(const std::vector<f8_cyl> &cyl, double dX, int dim) {
    std::vector<std::vector<Marker2>> per(cyl.size());
    for (size_t l = 0; l < cyl.size(); ++l) {
        const f8_cyl &cy = cyl[l];
        const double DC = 2.0 * cy.r;
        if (!cy.filled) {
            int NL = (int)std::lround(PI * DC / dX);
            if (NL < 1) NL = 1;
            for (int j = 1; j <= NL; ++j) {
                double ang = 2 * PI / NL * j;
                Marker2 m;
                m.x = cy.xc + DC / 2 * std::cos(ang);
                m.y = cy.yc + DC / 2 * std::sin(ang);
                m.u = cy.spin * std::sin(ang);
                m.v = -cy.spin * std::cos(ang);
                m.cyl = (int)l;
                per[l].push_back(m);
            }
        } else {
            int NL_lap = (int)(DC / (2 * dX));
            std::vector<int> shell(NL_lap + 1);
            for (int i = 0; i <= NL_lap; ++i) shell[i] = (int)std::lround(PI * (DC - 2 * i * dX) / dX);
            if (shell[NL_lap] == 0) shell[NL_lap] = 1;
            for (int i = 0; i <= NL_lap; ++i)
                for (int j = 1; j <= shell[i]; ++j) {
                    double ang = 2 * PI / shell[i] * j;
                    double rr = (DC - 2 * i * dX) / 2;
                    Marker2 m;
                    m.x = cy.xc + rr * std::cos(ang);
                    m.y = cy.yc + rr * std::sin(ang);
                    m.u = cy.spin * ((DC - 2 * i * dX) / DC * std::sin(ang));
                    m.v = -cy.spin * ((DC - 2 * i * dX) / DC * std::cos(ang));
                    m.cyl = (int)l;
                    per[l].push_back(m);
                }
        }
    }
    std::vector<Marker2> out;
    size_t maxn = 0;
    for (auto &p : per) maxn = std::max(maxn, p.size());
    for (size_t m = 0; m < maxn; ++m)
        for (size_t l = 0; l < per.size(); ++l)
            if (m < per[l].size()) out.push_back(per[l][m]);
    if (dim == 2)  // fenep_2d.f90:1628-1629
        for (auto &m : out) { m.x = m.x + 10e-10 * dX; m.y = m.y + 10e-10 * dX; }
    return out;
}

// fenep.f90:2045-2055
inline double roma(double r) {
    double ar = std::fabs(r);
    if (ar < 1.5 && ar >= 0.5) return (5.0 - 3.0 * ar - std::sqrt(-3.0 * ((1 - ar) * (1 - ar)) + 1.0)) / 6.0;
    if (ar < 0.5) return (1.0 + std::sqrt(-3.0 * (r * r) + 1.0)) / 3.0;
    return 0.0;
}

struct IbmGeom { double dX, dY, dZ, dx3; };

// Staggered stencil origins for component comp (0:u, 1:v, 2:w) of a marker at
// (xc, yc): fenep.f90:2081-2100.
inline void stencil_origin(int comp, double xc, double yc, double dX, double dY, int &i0, int &j0) {
    if (comp == 0) { j0 = (int)(yc / dY); i0 = (int)(xc / dX - 0.5); }
    else if (comp == 1) { j0 = (int)(yc / dY - 0.5); i0 = (int)(xc / dX); }
    else { j0 = (int)(yc / dY); i0 = (int)(xc / dX); }
}

// Grid point position of component comp at (i,j,k): X(i)+0.5dX etc.
inline void grid_pos(int comp, int i, int j, int k, double dX, double dY, double dZ, double &x, double &y, double &z) {
    x = (i - 0.5) * dX; y = (j - 0.5) * dY; z = (k - 0.5) * dZ;
    if (comp == 0) x = x + 0.5 * dX;
    else if (comp == 1) y = y + 0.5 * dY;
    else z = z + 0.5 * dZ;
}

// Spreading (and drag) volume of a marker of cylinder l: dX**3 (fenep.f90:
// 2166-2187; the drag uses dX*dY*dZ) or, with F8_IBM_ARC_VOLUME, the arc
// element dV = PI*DC/NL * dX * dX of the cylinder's ring (smac.f90:1128-1129).
double arc_volume(const OCtx &c, int l) {
    const double DC = 2.0 * c.cyl[l].r;
    const int NL = std::max(1, (int)std::lround(PI * DC / c.dX));
    return PI * DC / NL * c.dX * c.dX;
}

// ibm_Helmholtz of fenep_mpi.f90:1794-1929 (3D, no debug override),
// fenep_2d.f90:1726-1819 (2D) and smac.f90:1303-1488 (the arc-element
// spreading volume).  Interpolates Up/Vp/Wp (halo); writes fint and Fc; with
// accumulate (a further forcing iteration, smac.f90:1345-1353) adds to Fc.
void ibm_force(OCtx &c, bool accumulate) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double dX = c.dX, dY = c.dY, dZ = c.dZ, dt = c.ph.dt;
    const bool d3 = c.dim == 3;
    const size_t nm = c.mk.size();
    const double *Uf[3] = {c.Up.data(), c.Vp.data(), c.Wp.data()};
    const double dvol = d3 ? (dX * dY) * dZ : dX * dY;
    const double dxn = d3 ? dX * dX * dX : dX * dX;
    const int ncomp = d3 ? 3 : 2;
    // interpolation (do n / do m / do l, sums over the 3^3 stencil)
    for (int comp = 0; comp < ncomp; ++comp) {
        std::vector<double> &Fc = c.Fc[comp];
#pragma omp parallel for schedule(static)
        for (int n = 1; n <= NZ; ++n)
            for (size_t m = 0; m < nm; ++m) {
                const Marker2 &mk = c.mk[m];
                double zc = d3 ? (n - 0.25) * dZ : 0.0;
                int i0, j0;
                stencil_origin(comp, mk.x, mk.y, dX, dY, i0, j0);
                double ub = 0.0;
                int klo = d3 ? n - 1 : 1, khi = d3 ? n + 1 : 1;
                for (int k = klo; k <= khi; ++k)
                    for (int j = j0; j <= j0 + 2; ++j)
                        for (int i = i0; i <= i0 + 2; ++i) {
                            double x, y, z;
                            grid_pos(comp, i, j, k, dX, dY, dZ, x, y, z);
                            double del = d3 ? roma((x - mk.x) / dX) * roma((y - mk.y) / dY) * roma((z - zc) / dZ) / dvol
                                            : roma((x - mk.x) / dX) * roma((y - mk.y) / dY) / dvol;
                            ub = ub + Uf[comp][c.hidx(i, j, k)] * del * dxn;
                        }
                double uc = comp == 0 ? mk.u : (comp == 1 ? mk.v : 0.0);
                size_t o = m + nm * (size_t)(n - 1);
                // Fc reset in ibm_preliminary, then += (fenep.f90:2028, 2114)
                Fc[o] = (accumulate ? Fc[o] : 0.0) + (uc - ub) / dt;
            }
    }
    // spreading into a halo-extended temporary, then periodic fold (ibm_PBM)
    std::vector<double> mvol(c.cyl.size(), dxn);
    if (c.ph.ibm_volume == F8_IBM_ARC_VOLUME)
        for (size_t l = 0; l < c.cyl.size(); ++l) mvol[l] = arc_volume(c, (int)l);
    std::vector<double> ftmp(c.nh());
    for (int comp = 0; comp < ncomp; ++comp) {
        std::fill(ftmp.begin(), ftmp.end(), 0.0);
        const std::vector<double> &Fc = c.Fc[comp];
        for (int n = 1; n <= NZ; ++n)
            for (size_t m = 0; m < nm; ++m) {
                const Marker2 &mk = c.mk[m];
                double zc = d3 ? (n - 0.25) * dZ : 0.0;
                int i0, j0;
                stencil_origin(comp, mk.x, mk.y, dX, dY, i0, j0);
                double fcv = Fc[m + nm * (size_t)(n - 1)];
                int klo = d3 ? n - 1 : 1, khi = d3 ? n + 1 : 1;
                for (int k = klo; k <= khi; ++k)
                    for (int j = j0; j <= j0 + 2; ++j)
                        for (int i = i0; i <= i0 + 2; ++i) {
                            double x, y, z;
                            grid_pos(comp, i, j, k, dX, dY, dZ, x, y, z);
                            double del = d3 ? roma((x - mk.x) / dX) * roma((y - mk.y) / dY) * roma((z - zc) / dZ) / dvol
                                            : roma((x - mk.x) / dX) * roma((y - mk.y) / dY) / dvol;
                            ftmp[c.hidx(i, j, k)] = ftmp[c.hidx(i, j, k)] + fcv * del * mvol[mk.cyl];
                        }
            }
        // fold (fenep.f90:2195-2205); y is folded only when periodic
        for (int k = 0; k <= NZ + 1; ++k)
            for (int j = 0; j <= NY + 1; ++j) {
                ftmp[c.hidx(1, j, k)] = ftmp[c.hidx(1, j, k)] + ftmp[c.hidx(NX + 1, j, k)];
                ftmp[c.hidx(NX, j, k)] = ftmp[c.hidx(NX, j, k)] + ftmp[c.hidx(0, j, k)];
            }
        if (!c.walls)
            for (int k = 0; k <= NZ + 1; ++k)
                for (int i = 0; i <= NX + 1; ++i) {
                    ftmp[c.hidx(i, 1, k)] = ftmp[c.hidx(i, 1, k)] + ftmp[c.hidx(i, NY + 1, k)];
                    ftmp[c.hidx(i, NY, k)] = ftmp[c.hidx(i, NY, k)] + ftmp[c.hidx(i, 0, k)];
                }
        if (d3)
            for (int j = 0; j <= NY + 1; ++j)
                for (int i = 0; i <= NX + 1; ++i) {
                    ftmp[c.hidx(i, j, 1)] = ftmp[c.hidx(i, j, 1)] + ftmp[c.hidx(i, j, NZ + 1)];
                    ftmp[c.hidx(i, j, NZ)] = ftmp[c.hidx(i, j, NZ)] + ftmp[c.hidx(i, j, 0)];
                }
        for (int k = 1; k <= NZ; ++k)
            for (int j = 1; j <= NY; ++j)
                for (int i = 1; i <= NX; ++i) c.fint[comp][c.iidx(i, j, k)] = ftmp[c.hidx(i, j, k)];
    }
    if (!d3) std::fill(c.fint[2].begin(), c.fint[2].end(), 0.0);
}

// ---------------------------------------------------------------------------
// Step stages.

double lhs_helm1(const OCtx &c) { return c.ph.dt * c.ph.beta / c.ph.re / 2.0; }

// Predictor RHS (fft_navier Q, fenep.f90:1469-1474) or the explicit IBM
// velocity Ua (ibm_preliminary, fenep.f90:1997-2010 plus dt*F as in
// fenep_2d.f90:1678).  comp 0/1/2 = x/y/z.
void predictor(OCtx &c, bool ibm) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double dt = c.ph.dt;
    const double *P = c.P.data();
    const double *Us[3] = {c.U.data(), c.V.data(), c.W.data()};
    const std::vector<double> *A[3] = {&c.Ax, &c.Ay, &c.Az}, *A0[3] = {&c.Ax0, &c.Ay0, &c.Az0};
    const std::vector<double> *B[3] = {&c.Bx, &c.By, &c.Bz}, *T[3] = {&c.Tx, &c.Ty, &c.Tz}, *T0[3] = {&c.Tx0, &c.Ty0, &c.Tz0};
    const std::vector<double> *F[3] = {&c.Fx, &c.Fy, &c.Fz};
    double d[3] = {c.dX, c.dY, c.dZ};
    std::vector<double> *outs[3] = {&c.Ua, &c.Va, &c.Wa};
    int ncomp = c.dim == 3 ? 3 : 2;
    for (int comp = 0; comp < ncomp; ++comp) {
        for (int k = 1; k <= NZ; ++k)
            for (int j = 1; j <= NY; ++j)
                for (int i = 1; i <= NX; ++i) {
                    size_t o = c.iidx(i, j, k);
                    int ip = i + (comp == 0), jp = j + (comp == 1), kp = k + (comp == 2);
                    double u = Us[comp][c.hidx(i, j, k)];
                    double gp = -dt * (-P[c.hidx(i, j, k)] + P[c.hidx(ip, jp, kp)]) / d[comp];
                    double val;
                    if (!ibm) {
                        val = u + gp + dt * (3.0 * (*A[comp])[o] - (*A0[comp])[o]) / 2.0 + dt * (*B[comp])[o] / 2.0
                              + dt * ((*T[comp])[o] + (*T0[comp])[o]) / 2.0 + dt * (*F[comp])[o];
                    } else {
                        val = u + gp + dt * (3.0 * (*A[comp])[o] - (*A0[comp])[o]) / 2.0 + dt * (*B[comp])[o]
                              + dt * ((*T[comp])[o] + (*T0[comp])[o]) / 2.0 + dt * (*F[comp])[o];
                    }
                    (*outs[comp])[c.hidx(i, j, k)] = val;
                }
    }
}

// The reference writes "U - dt*(-P(i)+P(i+1))/dX + ...": the leading term is
// U - (dt*(..))/dX.  The helper above folds the sign into gp = -(dt*(..))/dX;
// U + (-x) == U - x exactly in IEEE arithmetic.

void save_history(OCtx &c) {
    c.Ax0 = c.Ax; c.Ay0 = c.Ay; c.Az0 = c.Az;
    c.Tx0 = c.Tx; c.Ty0 = c.Ty; c.Tz0 = c.Tz;
}

void interior_copy(const OCtx &c, const double *h, std::vector<double> &out) {
    out.resize(c.ni());
    for (int k = 1; k <= c.NZ; ++k)
        for (int j = 1; j <= c.NY; ++j)
            for (int i = 1; i <= c.NX; ++i) out[c.iidx(i, j, k)] = h[c.hidx(i, j, k)];
}

// Helmholtz solves of the predictor: Q (interior) -> Up (halo), for the three
// components.
void helmholtz(OCtx &c, std::vector<double> *Qs[3]) {
    std::vector<double> *outs[3] = {&c.Up, &c.Vp, &c.Wp};
    int ncomp = c.dim == 3 ? 3 : 2;
    for (int comp = 0; comp < ncomp; ++comp) {
        if (!c.walls) {
            fft_solve_periodic(c, *Qs[comp], 1.0, lhs_helm1(c), outs[comp]->data());
        } else {
            WallSys s = comp == 1 ? SYS_V : SYS_U;
            wall_solve(c, *Qs[comp], s, comp == 0 ? c.g.uwall : 0.0, outs[comp]->data());
        }
    }
    bc_scalar(c, c.Up.data(), BC_U);
    bc_scalar(c, c.Vp.data(), BC_V);
    if (c.dim == 3) bc_scalar(c, c.Wp.data(), BC_W);
}

// Divergence RHS (fenep.f90:1547-1555).
void poisson_rhs(OCtx &c, std::vector<double> &Qv) {
    Qv.resize(c.ni());
    const double dX = c.dX, dY = c.dY, dZ = c.dZ, dt = c.ph.dt;
    const double *Up = c.Up.data(), *Vp = c.Vp.data(), *Wp = c.Wp.data();
    const bool d3 = c.dim == 3;
    for (int k = 1; k <= c.NZ; ++k)
        for (int j = 1; j <= c.NY; ++j)
            for (int i = 1; i <= c.NX; ++i) {
                double s = (-Up[c.hidx(i - 1, j, k)] + Up[c.hidx(i, j, k)]) / dX + (-Vp[c.hidx(i, j - 1, k)] + Vp[c.hidx(i, j, k)]) / dY;
                if (d3) s = s + (-Wp[c.hidx(i, j, k - 1)] + Wp[c.hidx(i, j, k)]) / dZ;
                Qv[c.iidx(i, j, k)] = s / dt;
            }
}

// SOR (fenep.f90:848-905; walls smac_kabe.f90:302-374).  order 0: the
// reference's sweep (k, j lexicographic, odd then even i within a row);
// order 1: red-black by (i+j+k) parity, the GPU kernel's order.
int sor(OCtx &c, const std::vector<double> &Qv, int order) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const bool d3 = c.dim == 3;
    const double BXM = 1.0 / (c.dX * c.dX), BXP = BXM, BYM = 1.0 / (c.dY * c.dY), BYP = BYM;
    const double BZM = d3 ? 1.0 / (c.dZ * c.dZ) : 0.0, BZP = BZM;
    const double B0 = BXM + BXP + BYM + BYP + BZM + BZP;
    const double om = c.ph.sor_omega;
    double *Phi = c.Phi.data();
    double er0 = 0;
    for (size_t n = 0; n < c.ni(); ++n) er0 = er0 + Qv[n] * Qv[n];
    if (er0 == 0.0) er0 = 1.0e-16;
    std::vector<double> E(c.ni());
    int itr;
    auto upd = [&](int i, int j, int k) {
        double e = BZM * Phi[c.hidx(i, j, k - 1)] + BYM * Phi[c.hidx(i, j - 1, k)] + BXM * Phi[c.hidx(i - 1, j, k)]
                   - B0 * Phi[c.hidx(i, j, k)] + BXP * Phi[c.hidx(i + 1, j, k)] + BYP * Phi[c.hidx(i, j + 1, k)]
                   + BZP * Phi[c.hidx(i, j, k + 1)] - Qv[c.iidx(i, j, k)];
        E[c.iidx(i, j, k)] = e;
        Phi[c.hidx(i, j, k)] = Phi[c.hidx(i, j, k)] + om * e / B0;
    };
    for (itr = 1; itr <= c.ph.sor_itrmax; ++itr) {
        if (order == 0) {
            for (int k = 1; k <= NZ; ++k)
                for (int j = 1; j <= NY; ++j)
                    for (int l = 1; l <= 2; ++l)
                        for (int i = l; i <= NX; i += 2) upd(i, j, k);
        } else {
            for (int color = 0; color < 2; ++color) {
                for (int k = 1; k <= NZ; ++k)
                    for (int j = 1; j <= NY; ++j)
                        for (int i = 1; i <= NX; ++i)
                            if (((i + j + k) & 1) == color) upd(i, j, k);
                bc_scalar(c, Phi, BC_P);
            }
        }
        bc_scalar(c, Phi, BC_P);
        double er = 0;
        for (size_t n = 0; n < c.ni(); ++n) er = er + E[n] * E[n];
        if (std::sqrt(er / er0) < c.ph.sor_eps) break;
    }
    // zero-mean shift (fenep_2d.f90:577-579, smac_kabe.f90:346-348)
    double s = 0;
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) s = s + Phi[c.hidx(i, j, k)];
    double mean = s / (double)(NX * NY * NZ);
    for (size_t n = 0; n < c.nh(); ++n) Phi[n] = Phi[n] - mean;
    return itr;
}

// fft_march (fenep.f90:1562-1604), wall form fenep_2d.f90:1344-1383.
void march(OCtx &c) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double dt = c.ph.dt, dX = c.dX, dY = c.dY, dZ = c.dZ;
    const bool d3 = c.dim == 3;
    const double *Phi = c.Phi.data();
    const double pc = c.ph.dt * c.ph.beta / c.ph.re / 2.0;
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) {
                size_t h = c.hidx(i, j, k);
                double ph = Phi[h];
                c.U[h] = c.Up[h] - dt * (-ph + Phi[c.hidx(i + 1, j, k)]) / dX;
                c.V[h] = c.Vp[h] - dt * (-ph + Phi[c.hidx(i, j + 1, k)]) / dY;
                if (d3) c.W[h] = c.Wp[h] - dt * (-ph + Phi[c.hidx(i, j, k + 1)]) / dZ;
                double lap = (Phi[c.hidx(i - 1, j, k)] - 2 * ph + Phi[c.hidx(i + 1, j, k)]) / (dX * dX)
                           + (Phi[c.hidx(i, j - 1, k)] - 2 * ph + Phi[c.hidx(i, j + 1, k)]) / (dY * dY);
                if (d3) lap = lap + (Phi[c.hidx(i, j, k - 1)] - 2 * ph + Phi[c.hidx(i, j, k + 1)]) / (dZ * dZ);
                c.P[h] = c.P[h] + ph - pc * lap;
            }
    bc_scalar(c, c.U.data(), BC_U);
    bc_scalar(c, c.V.data(), BC_V);
    if (d3) bc_scalar(c, c.W.data(), BC_W);
    bc_scalar(c, c.P.data(), BC_P);
}

int do_step(OCtx &c, double *drag) {
    const int step_no = c.step + 1;
    const bool d3 = c.dim == 3;
    const bool ibm = !c.mk.empty();
    if (c.ph.beta == 1.0) {
        std::fill(c.C.begin(), c.C.end(), 0.0);
        std::fill(c.Tx.begin(), c.Tx.end(), 0.0);
        std::fill(c.Ty.begin(), c.Ty.end(), 0.0);
        std::fill(c.Tz.begin(), c.Tz.end(), 0.0);
    } else if (d3) {
        c.mark(0);
        polymer_faces3(c);
        c.mark(1);
        cstar3(c);
        lyapunov3(c);
        c.mark(2);
        polymer_stress3(c);
    } else {
        c.mark(0);
        c.mark(1);
        polymer2(c);
        c.mark(2);
        polymer_stress2(c);
    }
    if (c.ph.beta == 1.0) { c.mark(0); c.mark(1); c.mark(2); }
    convection_viscous(c);
    if (step_no == 1 && c.ph.ab2_start) save_history(c);
    predictor(c, ibm);
    save_history(c);
    c.mark(3);
    std::vector<double> Qx, Qy, Qz;
    std::vector<double> *Qs[3] = {&Qx, &Qy, &Qz};
    const double dt = c.ph.dt;
    if (!ibm) {
        interior_copy(c, c.Ua.data(), Qx);
        interior_copy(c, c.Va.data(), Qy);
        if (d3) interior_copy(c, c.Wa.data(), Qz);
    } else {
        // Up = Ua with boundary values (ibm_preliminary), force, then
        // Q = Ua + dt*f - dt*B/2 (ibm_predict, fenep.f90:2229); with NS > 1
        // (smac.f90:1607-1611) further iterations interpolate the last
        // Helmholtz solution, add to Fc, spread and solve again
        bc_scalar(c, c.Ua.data(), BC_U);
        bc_scalar(c, c.Va.data(), BC_V);
        if (d3) bc_scalar(c, c.Wa.data(), BC_W);
        c.Up = c.Ua; c.Vp = c.Va; c.Wp = c.Wa;
        const std::vector<double> *B[3] = {&c.Bx, &c.By, &c.Bz};
        const std::vector<double> *Ua[3] = {&c.Ua, &c.Va, &c.Wa};
        const int repeats = std::max(1, c.ph.ibm_repeats);
        for (int r = 0; r < repeats; ++r) {
            ibm_force(c, r > 0);
            for (int comp = 0; comp < (d3 ? 3 : 2); ++comp) {
                Qs[comp]->resize(c.ni());
                for (int k = 1; k <= c.NZ; ++k)
                    for (int j = 1; j <= c.NY; ++j)
                        for (int i = 1; i <= c.NX; ++i) {
                            size_t o = c.iidx(i, j, k);
                            (*Qs[comp])[o] = (*Ua[comp])[c.hidx(i, j, k)] + dt * c.fint[comp][o] - dt * (*B[comp])[o] / 2;
                        }
            }
            if (r < repeats - 1) helmholtz(c, Qs);
        }
        if (drag) {
            const size_t nm = c.mk.size();
            const double dv = d3 ? (c.dX * c.dY) * c.dZ : c.dX * c.dY;
            int ncyl = (int)c.cyl.size();
            for (int l = 0; l < ncyl * 3; ++l) drag[l] = 0.0;
            for (int comp = 0; comp < (d3 ? 3 : 2); ++comp) {
                std::vector<double> s(ncyl, 0.0);
                for (int n = 0; n < c.NZ; ++n)
                    for (size_t m = 0; m < nm; ++m) s[c.mk[m].cyl] = s[c.mk[m].cyl] + c.Fc[comp][m + nm * n];
                for (int l = 0; l < ncyl; ++l)
                    drag[3 * l + comp] = -s[l] * (c.ph.ibm_volume == F8_IBM_ARC_VOLUME ? arc_volume(c, l) : dv);
            }
        }
    }
    c.mark(4);
    helmholtz(c, Qs);
    c.mark(5);
    // Poisson
    std::vector<double> Qp;
    poisson_rhs(c, Qp);
    if (c.poisson == F8_POISSON_FFT) {
        if (!c.walls) fft_solve_periodic(c, Qp, 0.0, -1.0, c.Phi.data());
        else wall_solve(c, Qp, SYS_P, 0.0, c.Phi.data());
        bc_scalar(c, c.Phi.data(), BC_P);
        c.poisson_iters = -1;
    } else {
        c.poisson_iters = sor(c, Qp, c.sor_order);
    }
    c.mark(6);
    march(c);
    // C_kabe at the end of the step (fft_march_kabe, fenep_2d.f90:1374)
    if (c.walls && c.ph.beta != 1.0) bc_c(c, c.C.data());
    c.mark(7);
    c.step += 1;
    // NaN guard (fenep_2d.f90:1974)
    for (size_t n = 0; n < c.nh(); ++n)
        if (!std::isfinite(c.U[n])) return F8_ERR_NAN;
    if (c.newton_unconv > 0) return F8_WARN_NEWTON;
    if (c.poisson == F8_POISSON_SOR && c.poisson_iters > c.ph.sor_itrmax) return F8_WARN_SOR;
    return F8_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// ABI (include/f8.h with the f8o_ prefix)

namespace {

int validate(const f8_grid *g, const f8_phys *ph, int ncyl, const f8_cyl *cy, int prec, int poisson) {
    if (!g || !ph) return F8_ERR_ARG;
    if (g->dim != 2 && g->dim != 3) return F8_ERR_ARG;
    if (g->nx < 4 || g->ny < 4 || g->nz < 1) return F8_ERR_ARG;
    if (g->dim == 2 && g->nz != 1) return F8_ERR_ARG;
    if (g->dim == 3 && g->nz < 4) return F8_ERR_ARG;
    if (!(g->lx > 0 && g->ly > 0 && g->lz > 0)) return F8_ERR_ARG;
    if (g->bc_y != F8_BC_PERIODIC && g->bc_y != F8_BC_WALLS) return F8_ERR_ARG;
    if (poisson == F8_POISSON_FFT && (!is_pow2(g->nx) || !is_pow2(g->ny) || !is_pow2(g->nz))) return F8_ERR_ARG;
    if (poisson != F8_POISSON_FFT && poisson != F8_POISSON_SOR) return F8_ERR_ARG;
    if (prec != F8_FP64 && prec != F8_MIXED) return F8_ERR_ARG;
    if (!(ph->dt > 0) || !(ph->re > 0) || !(ph->wi > 0)) return F8_ERR_ARG;
    if (ph->newton_itrmax < 1 || ph->sor_itrmax < 1) return F8_ERR_ARG;
    if (ncyl < 0 || (ncyl > 0 && !cy)) return F8_ERR_ARG;
    if (ph->ibm_repeats < 1 || ph->ibm_repeats > 64) return F8_ERR_ARG;
    if (ph->ibm_volume != F8_IBM_CELL_VOLUME && ph->ibm_volume != F8_IBM_ARC_VOLUME) return F8_ERR_ARG;
    if (ph->eigen_test < F8_EIGEN_VIETA || ph->eigen_test > F8_EIGEN_SYMMETRIC) return F8_ERR_ARG;
    if (ph->eigen_test != F8_EIGEN_VIETA && g->dim != 3) return F8_ERR_UNSUPPORTED;
    if (ph->ibm_volume == F8_IBM_ARC_VOLUME) {
        // the arc element of a surface ring (smac.f90:1128-1129), 3D
        if (g->dim != 3) return F8_ERR_UNSUPPORTED;
        for (int l = 0; l < ncyl; ++l)
            if (cy[l].filled) return F8_ERR_UNSUPPORTED;
    }
    return F8_OK;
}

void copy_in_halo(OCtx &c, std::vector<double> &dst, const double *src, int ncomp) {
    if (src) std::memcpy(dst.data(), src, sizeof(double) * c.nh() * ncomp);
    else std::fill(dst.begin(), dst.end(), 0.0);
}
void copy_in_int(OCtx &c, std::vector<double> &dst, const double *src) {
    if (src) std::memcpy(dst.data(), src, sizeof(double) * c.ni());
    else std::fill(dst.begin(), dst.end(), 0.0);
}

}  // namespace

// fenep_mpi.f90:2934-2941 (mode 1) and 3054-3056 (mode 2), after each step
void stats_accumulate(OCtx &c) {
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const size_t ni = (size_t)NX * NY * NZ;
    const std::vector<double> *F[3] = {&c.U, &c.V, &c.W};
    for (int q = 0; q < 3; ++q)
        for (int k = 1; k <= NZ; ++k)
            for (int j = 1; j <= NY; ++j)
                for (int i = 1; i <= NX; ++i) {
                    const size_t o = (size_t)(i - 1) + NX * ((size_t)(j - 1) + (size_t)NY * (k - 1));
                    const double v = (*F[q])[c.hidx(i, j, k)];
                    if (c.stats_mode == 1) c.stats_sum[q * ni + o] += v;
                    else c.stats_sum[q * ni + o] += (v - c.stats_mean[q * ni + o]) * (v - c.stats_mean[q * ni + o]);
                }
    if (c.stats_mode == 1 && c.stats_n < c.stats_max) {
        const int i = NX / 2, j = NY / 2;
        for (int k = 1; k <= NZ; ++k) {
            const size_t base = (size_t)c.stats_n * NZ + (k - 1);
            c.stats_probe[0 * (size_t)c.stats_max * NZ + base] = (c.U[c.hidx(i, j, k)] + c.U[c.hidx(i - 1, j, k)]) / 2.0;
            c.stats_probe[1 * (size_t)c.stats_max * NZ + base] = (c.V[c.hidx(i, j, k)] + c.V[c.hidx(i, j - 1, k)]) / 2.0;
            c.stats_probe[2 * (size_t)c.stats_max * NZ + base] = (c.W[c.hidx(i, j, k)] + c.W[c.hidx(i, j, k - 1)]) / 2.0;
        }
    }
    c.stats_n += 1;
}

extern "C" {

void f8o_default_phys(f8_phys *ph) {
    std::memset(ph, 0, sizeof(*ph));
    ph->re = 1.0; ph->wi = 1.0; ph->beta = 1.0; ph->lp2 = 100.0; ph->dt = 1.0e-3;
    ph->newton_dc = 1.0e-5; ph->newton_eps = 1.0e-6; ph->newton_itrmax = 10000;
    ph->sor_omega = 1.8; ph->sor_eps = 1.0e-5; ph->sor_itrmax = 10000;
    ph->ab2_start = 1;
    ph->ibm_volume = F8_IBM_CELL_VOLUME;
    ph->ibm_repeats = 1;
}

int f8o_create(f8_ctx **out, const f8_grid *g, const f8_phys *ph, const f8_cyl *cy, int ncyl, int prec, int poisson) {
    if (!out) return F8_ERR_ARG;
    *out = nullptr;
    int st = validate(g, ph, ncyl, cy, prec, poisson);
    if (st) return st;
    OCtx *c = new (std::nothrow) OCtx();
    if (!c) return F8_ERR_NOMEM;
    c->g = *g; c->ph = *ph; c->prec = prec; c->poisson = poisson;
    if (ncyl > 0) c->cyl.assign(cy, cy + ncyl);
    c->dim = g->dim; c->NC = g->dim == 3 ? 6 : 3;
    c->NX = g->nx; c->NY = g->ny; c->NZ = g->nz;
    c->SX = c->NX + 2; c->SY = c->NY + 2; c->SZ = c->NZ + 2;
    c->dX = g->lx / g->nx; c->dY = g->ly / g->ny; c->dZ = g->dim == 3 ? g->lz / g->nz : c->dX;
    c->walls = g->bc_y == F8_BC_WALLS;
    try {
        size_t nh = c->nh(), ni = c->ni();
        for (auto *v : {&c->U, &c->V, &c->W, &c->P, &c->Phi, &c->Up, &c->Vp, &c->Wp, &c->Ua, &c->Va, &c->Wa}) v->assign(nh, 0.0);
        c->C.assign(nh * c->NC, 0.0);
        c->C0.assign(nh * c->NC, 0.0);
        for (auto *v : {&c->Ax0, &c->Ay0, &c->Az0, &c->Tx0, &c->Ty0, &c->Tz0, &c->Fx, &c->Fy, &c->Fz, &c->Ax, &c->Ay, &c->Az,
                        &c->Bx, &c->By, &c->Bz, &c->Tx, &c->Ty, &c->Tz, &c->fint[0], &c->fint[1], &c->fint[2]})
            v->assign(ni, 0.0);
        if (c->dim == 3) {
            const size_t nr = (size_t)(prow_hi(*c) - prow_lo(*c) + 1);   // rows of the polymer update
            c->Cx.assign((size_t)6 * c->NX * nr * c->NZ, 0.0);
            c->Cpx.assign((size_t)6 * (c->NX + 1) * nr * c->NZ, 0.0); c->Cnx = c->Cpx;
            c->Cpy.assign((size_t)6 * c->NX * (nr + 1) * c->NZ, 0.0); c->Cny = c->Cpy;
            c->Cpz.assign((size_t)6 * c->NX * nr * (c->NZ + 1), 0.0); c->Cnz = c->Cpz;
        }
    } catch (...) { delete c; return F8_ERR_NOMEM; }
    make_tw(c->NX, c->twx_r, c->twx_i);
    make_tw(c->NY, c->twy_r, c->twy_i);
    make_tw(c->NZ, c->twz_r, c->twz_i);
    // Modified wavenumbers 2(1 - cos(m theta))/d^2 (fenep.f90:1458-1460).  The
    // reference writes cos((i-1)*dX) for its 2 pi box; the angle step is
    // theta = 2 pi / N for any box length, which is the same double when
    // L = 2 pi.
    const double thx = 2 * PI / c->NX, thy = 2 * PI / c->NY, thz = 2 * PI / c->NZ;
    c->kx2.resize(c->NX / 2 + 1);
    for (int i = 1; i <= c->NX / 2 + 1; ++i) c->kx2[i - 1] = 2 * (1 - std::cos((i - 1) * thx)) / (c->dX * c->dX);
    c->ky2.resize(c->NY);
    for (int j = 1; j <= c->NY; ++j) c->ky2[j - 1] = 2 * (1 - std::cos((j - 1) * thy)) / (c->dY * c->dY);
    c->kz2.resize(c->NZ);
    for (int k = 1; k <= c->NZ; ++k) c->kz2[k - 1] = 2 * (1 - std::cos((k - 1) * thz)) / (c->dZ * c->dZ);
    if (!c->cyl.empty()) {
        if (std::fabs(c->dX - c->dY) > 1e-14 * c->dX || (c->dim == 3 && std::fabs(c->dX - c->dZ) > 1e-14 * c->dX)) {
            delete c;  // fenep.f90:1808-1810
            return F8_ERR_ARG;
        }
        c->mk = build_markers(c->cyl, c->dX, c->dim);
        for (int q = 0; q < 3; ++q) c->Fc[q].assign(c->mk.size() * c->NZ, 0.0);
    }
    *out = reinterpret_cast<f8_ctx *>(c);
    return F8_OK;
}

int f8o_load(f8_ctx *ctx, const f8_fields *in, int step0) {
    if (!ctx || !in || !in->u || !in->v || !in->p || !in->c) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.dim == 3 && !in->w) return F8_ERR_ARG;
    copy_in_halo(c, c.U, in->u, 1);
    copy_in_halo(c, c.V, in->v, 1);
    copy_in_halo(c, c.W, c.dim == 3 ? in->w : nullptr, 1);
    copy_in_halo(c, c.P, in->p, 1);
    copy_in_halo(c, c.Phi, in->phi, 1);
    copy_in_halo(c, c.C, in->c, c.NC);
    copy_in_int(c, c.Ax0, in->ax0); copy_in_int(c, c.Ay0, in->ay0); copy_in_int(c, c.Az0, in->az0);
    copy_in_int(c, c.Tx0, in->tx0); copy_in_int(c, c.Ty0, in->ty0); copy_in_int(c, c.Tz0, in->tz0);
    copy_in_int(c, c.Fx, in->fx); copy_in_int(c, c.Fy, in->fy); copy_in_int(c, c.Fz, in->fz);
    // boundary values of the loaded state (init calls PBM / *_kabe, fenep.f90:139-143)
    bc_scalar(c, c.U.data(), BC_U);
    bc_scalar(c, c.V.data(), BC_V);
    if (c.dim == 3) bc_scalar(c, c.W.data(), BC_W);
    bc_scalar(c, c.P.data(), BC_P);
    bc_c(c, c.C.data());
    c.step = step0;
    c.loaded = true;
    return F8_OK;
}

int f8o_step(f8_ctx *ctx, int nsteps, double *drag) {
    if (!ctx || nsteps < 0) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (!c.loaded) return F8_ERR_STATE;
    int worst = F8_OK;
    const int ncyl = (int)c.cyl.size();
    c.newton_iters = 0;
    c.newton_unconv = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < nsteps; ++s) {
        int st = do_step(c, drag ? drag + (size_t)s * ncyl * 3 : nullptr);
        if (c.stats_mode) stats_accumulate(c);
        c.total_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        t0 = std::chrono::steady_clock::now();
        c.timed_steps += 1;
        if (st == F8_ERR_NAN) return st;
        if (st > worst) worst = st;
    }
    return worst;
}

int f8o_store(f8_ctx *ctx, f8_fields *out) {
    if (!ctx || !out) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    auto put = [&](double *dst, const std::vector<double> &src) { if (dst) std::memcpy(dst, src.data(), sizeof(double) * src.size()); };
    put(out->u, c.U); put(out->v, c.V); if (c.dim == 3) put(out->w, c.W);
    put(out->p, c.P); put(out->phi, c.Phi); put(out->c, c.C);
    put(out->ax0, c.Ax0); put(out->ay0, c.Ay0); put(out->az0, c.Az0);
    put(out->tx0, c.Tx0); put(out->ty0, c.Ty0); put(out->tz0, c.Tz0);
    put(out->fx, c.Fx); put(out->fy, c.Fy); put(out->fz, c.Fz);
    return F8_OK;
}

int f8o_diagnostics(f8_ctx *ctx, f8_diag *d) {
    if (!ctx || !d) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    std::memset(d, 0, sizeof(*d));
    d->step = c.step;
    double ke = 0, umax = -1e300, vmax = -1e300, wmax = -1e300, tmin = 1e300, tmax = -1e300, tsum = 0, dmax = 0;
    const bool d3 = c.dim == 3;
    for (int k = 1; k <= c.NZ; ++k)
        for (int j = 1; j <= c.NY; ++j)
            for (int i = 1; i <= c.NX; ++i) {
                double ur = (c.U[c.hidx(i, j, k)] + c.U[c.hidx(i - 1, j, k)]) / 2.0;
                double vr = (c.V[c.hidx(i, j, k)] + c.V[c.hidx(i, j - 1, k)]) / 2.0;
                double wr = d3 ? (c.W[c.hidx(i, j, k)] + c.W[c.hidx(i, j, k - 1)]) / 2.0 : 0.0;
                ke += ur * ur + vr * vr + wr * wr;
                const double *cc = &c.C[c.NC * c.hidx(i, j, k)];
                double tr = d3 ? cc[0] + cc[3] + cc[5] : cc[0] + cc[2];
                tmin = std::min(tmin, tr); tmax = std::max(tmax, tr); tsum += tr;
                double dv = (c.U[c.hidx(i, j, k)] - c.U[c.hidx(i - 1, j, k)]) / c.dX + (c.V[c.hidx(i, j, k)] - c.V[c.hidx(i, j - 1, k)]) / c.dY;
                if (d3) dv += (c.W[c.hidx(i, j, k)] - c.W[c.hidx(i, j, k - 1)]) / c.dZ;
                dmax = std::max(dmax, std::fabs(dv));
                if (std::isnan(ur) || std::isnan(vr) || std::isnan(wr)) d->nan_found = 1;
            }
    for (size_t n = 0; n < c.nh(); ++n) {
        umax = std::max(umax, c.U[n]); vmax = std::max(vmax, c.V[n]); if (d3) wmax = std::max(wmax, c.W[n]);
    }
    const double N = (double)c.ni();
    d->ke = ke / 2.0 / N;
    double cfl = std::max(umax * c.ph.dt / c.dX, vmax * c.ph.dt / c.dY);
    if (d3) cfl = std::max(cfl, wmax * c.ph.dt / c.dZ);
    d->cfl = cfl * 6.0;
    d->trc_min = tmin; d->trc_max = tmax; d->trc_mean = tsum / N;
    // std = sqrt(sum((trC - mean)^2) / N), mean first (fenep.f90:2316-2317)
    {
        const double mean = tsum / N;
        double s2 = 0.0;
        for (int k = 1; k <= c.NZ; ++k)
            for (int j = 1; j <= c.NY; ++j)
                for (int i = 1; i <= c.NX; ++i) {
                    const double *cc = &c.C[c.NC * c.hidx(i, j, k)];
                    const double tr = d3 ? cc[0] + cc[3] + cc[5] : cc[0] + cc[2];
                    s2 += (tr - mean) * (tr - mean);
                }
        d->trc_std = std::sqrt(s2 / N);
    }
    d->div_max = dmax;
    d->newton_iters = c.newton_iters; d->newton_unconverged = c.newton_unconv;
    d->poisson_iters = c.poisson_iters;
    return F8_OK;
}

// get_data_binary's slice records (fenep.f90:1108-1183; fenep_mpi.f90:811-937)
// with U_C = L_C = 1: x, y, z, E(3), KE or Q, Omega(3), |Omega|^2/2, trC, C(6)
int f8o_slice(f8_ctx *ctx, int axis, int variant, double *out) {
    if (!ctx || !out || axis < 0 || axis > 2 || variant < 0 || variant > 1) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.dim != 3) return F8_ERR_UNSUPPORTED;
    const double dX = c.dX, dY = c.dY, dZ = c.dZ;
    auto U = [&](int i, int j, int k) { return c.U[c.hidx(i, j, k)]; };
    auto V = [&](int i, int j, int k) { return c.V[c.hidx(i, j, k)]; };
    auto W = [&](int i, int j, int k) { return c.W[c.hidx(i, j, k)]; };
    const int n1 = axis == 0 ? c.NY : c.NX, n2 = axis == 2 ? c.NY : c.NZ;
    for (int b = 0; b < n2; ++b)
        for (int a = 0; a < n1; ++a) {
            int i, j, k;
            if (axis == 2) { k = c.NZ / 2; j = 1 + b; i = 1 + a; }
            else if (axis == 1) { j = c.NY / 2; k = 1 + b; i = 1 + a; }
            else { i = c.NX / 2; k = 1 + b; j = 1 + a; }
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
            const double *cc = &c.C[6 * c.hidx(i, j, k)];
            double *o = out + 18 * ((size_t)b * n1 + a);
            o[0] = (i - 0.5) * dX; o[1] = (j - 0.5) * dY; o[2] = (k - 0.5) * dZ;
            o[3] = E0; o[4] = E1; o[5] = E2;
            o[6] = variant == 1 ? Q : (E0 * E0 + E1 * E1 + E2 * E2) / 2;
            o[7] = O0; o[8] = O1; o[9] = O2;
            o[10] = (O0 * O0 + O1 * O1 + O2 * O2) / 2;
            o[11] = cc[0] + cc[3] + cc[5];
            for (int m = 0; m < 6; ++m) o[12 + m] = cc[m];
        }
    return F8_OK;
}

// all_time_dif (fenep_mpi.f90:2200-2348) with U_C = L_C = 1, nu = 1/Re; the
// fluctuation gets the periodic boundary values of PBM
int f8o_turbulence(f8_ctx *ctx, const double *mu, const double *mv, const double *mw, f8_turb *out) {
    if (!ctx || !out) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.dim != 3) return F8_ERR_UNSUPPORTED;
    const int NX = c.NX, NY = c.NY, NZ = c.NZ;
    const double *mean[3] = {mu, mv, mw};
    const std::vector<double> *F[3] = {&c.U, &c.V, &c.W};
    auto wrap = [](int a, int n) { return a < 1 ? a + n : (a > n ? a - n : a); };
    auto fl = [&](int q, int i, int j, int k) {
        i = wrap(i, NX); j = wrap(j, NY); k = wrap(k, NZ);
        double v = (*F[q])[c.hidx(i, j, k)];
        if (mean[q]) v -= mean[q][(size_t)(i - 1) + NX * ((size_t)(j - 1) + (size_t)NY * (k - 1))];
        return v;
    };
    const double dX = c.dX, dY = c.dY, dZ = c.dZ, N = (double)NX * NY * NZ, nu = 1.0 / c.ph.re;
    double u2 = 0, v2 = 0, w2 = 0, gu2 = 0, gv2 = 0, gw2 = 0, s2 = 0, ks = 0, ep = 0, tsum = 0;
    const double dep = 0.5 * (1.0 - c.ph.beta) / c.ph.re / c.ph.wi * (c.ph.lp2 - 3.0);
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) {
                auto U = [&](int a, int b, int cc) { return fl(0, a, b, cc); };
                auto V = [&](int a, int b, int cc) { return fl(1, a, b, cc); };
                auto W = [&](int a, int b, int cc) { return fl(2, a, b, cc); };
                const double ur = (U(i, j, k) + U(i - 1, j, k)) / 2.0, vr = (V(i, j, k) + V(i, j - 1, k)) / 2.0,
                             wr = (W(i, j, k) + W(i, j, k - 1)) / 2.0;
                u2 += ur * ur; v2 += vr * vr; w2 += wr * wr;
                const double gu = (U(i, j, k) - U(i - 1, j, k)) / dX, gv = (V(i, j, k) - V(i, j - 1, k)) / dY,
                             gw = (W(i, j, k) - W(i, j, k - 1)) / dZ;
                gu2 += gu * gu; gv2 += gv * gv; gw2 += gw * gw;
                double D[3][3];
                D[0][0] = gu;
                D[0][1] = (U(i, j + 1, k) - U(i, j - 1, k) + U(i - 1, j + 1, k) - U(i - 1, j - 1, k)) / (4 * dY);
                D[0][2] = (U(i, j, k + 1) - U(i, j, k - 1) + U(i - 1, j, k + 1) - U(i - 1, j, k - 1)) / (4 * dZ);
                D[1][0] = (V(i + 1, j, k) - V(i - 1, j, k) + V(i + 1, j - 1, k) - V(i - 1, j - 1, k)) / (4 * dX);
                D[1][1] = gv;
                D[1][2] = (V(i, j, k + 1) - V(i, j, k - 1) + V(i, j - 1, k + 1) - V(i, j - 1, k - 1)) / (4 * dZ);
                D[2][0] = (W(i + 1, j, k) - W(i - 1, j, k) + W(i + 1, j, k - 1) - W(i - 1, j, k - 1)) / (4 * dX);
                D[2][1] = (W(i, j + 1, k) - W(i, j - 1, k) + W(i, j + 1, k - 1) - W(i, j - 1, k - 1)) / (4 * dY);
                D[2][2] = gw;
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) s2 += (D[p][q] + D[q][p]) * (D[p][q] + D[q][p]);
                const size_t h = c.hidx(i, j, k);
                ks += c.U[h] * c.U[h] + c.V[h] * c.V[h] + c.W[h] * c.W[h];
                const double *cc = &c.C[6 * h];
                const double tr = cc[0] + cc[3] + cc[5];
                ep += dep * std::log((c.ph.lp2 - 3.0) / (c.ph.lp2 - tr));
                tsum += tr;
            }
    const double urms = u2 / N, vrms = v2 / N, wrms = w2 / N;
    const double all_rms = (urms + vrms + wrms) / 3.0, all_grad = (gu2 / N + gv2 / N + gw2 / N) / 3.0;
    std::memset(out, 0, sizeof(*out));
    out->epsilon = nu / 2.0 * s2 / N;
    out->l_kolmogorov = std::pow(nu * nu * nu / out->epsilon, 0.25);
    out->t_kolmogorov = std::pow(nu / out->epsilon, 0.5);
    out->u_kolmogorov = std::pow(nu * out->epsilon, 0.25);
    out->lambda = std::sqrt(all_rms / all_grad);
    out->re_lambda = std::sqrt(all_rms) * out->lambda / nu;
    out->k_energy = (urms + vrms + wrms) / 2.0;
    out->k_staggered = ks / (2.0 * N);
    out->ep_energy = ep / N;
    out->trc_mean = tsum / N;
    double sd = 0;
    for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) {
                const double *cc = &c.C[6 * c.hidx(i, j, k)];
                const double d = cc[0] + cc[3] + cc[5] - out->trc_mean;
                sd += d * d;
            }
    out->trc_std = std::sqrt(sd / N);
    return F8_OK;
}

// energy_single (fenep.f90:1606-1672): shell-binned |u_hat|^2 / N^2 of the
// (optionally mean-subtracted) velocity, half-spectrum weights 1/2 at kx = 0
// and NX/2
int f8o_spectrum(f8_ctx *ctx, const double *mu, const double *mv, const double *mw, double *energy) {
    if (!ctx || !energy) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.dim != 3) return F8_ERR_UNSUPPORTED;
    const int NX = c.NX, NY = c.NY, NZ = c.NZ, NXH = NX / 2 + 1;
    const double *mean[3] = {mu, mv, mw};
    const std::vector<double> *F[3] = {&c.U, &c.V, &c.W};
    std::fill(energy, energy + NX + 1, 0.0);
    const double N = (double)NX * NY * NZ;
    for (int q = 0; q < 3; ++q) {
        std::vector<double> src((size_t)NX * NY * NZ), H(2 * (size_t)NXH * NY * NZ);
        for (int k = 1; k <= NZ; ++k)
            for (int j = 1; j <= NY; ++j)
                for (int i = 1; i <= NX; ++i) {
                    const size_t o = (size_t)(i - 1) + NX * ((size_t)(j - 1) + (size_t)NY * (k - 1));
                    src[o] = (*F[q])[c.hidx(i, j, k)] - (mean[q] ? mean[q][o] : 0.0);
                }
        fft_x_forward(c, src, 1, NY, H);
        fft_y(c, H, NY, -1);
        fft_z(c, H, NY, -1);
        for (int k = 0; k < NZ; ++k)
            for (int j = 0; j < NY; ++j)
                for (int i = 0; i < NXH; ++i) {
                    const double kx = i, ky = j <= NY / 2 ? j : j - NY, kz = k <= NZ / 2 ? k : k - NZ;
                    const int idx = std::min(NX, (int)std::lround(std::sqrt(kx * kx + ky * ky + kz * kz)));
                    const size_t o = 2 * ((size_t)i + NXH * ((size_t)j + (size_t)NY * k));
                    const double e = (H[o] * H[o] + H[o + 1] * H[o + 1]) / (N * N);
                    energy[idx] += (i == 0 || i == NX / 2) ? e / 2.0 : e / 2.0 * 2.0;
                }
    }
    return F8_OK;
}

int f8o_stats_begin(f8_ctx *ctx, int mode, const double *mu, const double *mv, const double *mw, int max_steps) {
    if (!ctx || mode < 0 || mode > 2 || max_steps < 0) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.dim != 3) return F8_ERR_UNSUPPORTED;
    if (mode == 2 && (!mu || !mv || !mw)) return F8_ERR_ARG;
    const size_t ni = (size_t)c.NX * c.NY * c.NZ;
    c.stats_mode = mode;
    c.stats_n = 0;
    c.stats_sum.assign(3 * ni, 0.0);
    if (mode == 1) {
        c.stats_max = max_steps;
        c.stats_probe.assign((size_t)3 * max_steps * c.NZ, 0.0);
    }
    if (mode == 2) {
        c.stats_mean.resize(3 * ni);
        std::copy(mu, mu + ni, c.stats_mean.begin());
        std::copy(mv, mv + ni, c.stats_mean.begin() + ni);
        std::copy(mw, mw + ni, c.stats_mean.begin() + 2 * ni);
    }
    return F8_OK;
}

int f8o_stats_read(f8_ctx *ctx, double *su, double *sv, double *sw, double *probes, int *nsteps) {
    if (!ctx) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    const size_t ni = (size_t)c.NX * c.NY * c.NZ;
    double *dst[3] = {su, sv, sw};
    for (int q = 0; q < 3; ++q)
        if (dst[q] && c.stats_sum.size() == 3 * ni) std::copy(c.stats_sum.begin() + q * ni, c.stats_sum.begin() + (q + 1) * ni, dst[q]);
    const int n = std::min(c.stats_n, c.stats_max);
    if (probes && !c.stats_probe.empty())
        for (int q = 0; q < 3; ++q)
            std::copy(c.stats_probe.begin() + (size_t)q * c.stats_max * c.NZ,
                      c.stats_probe.begin() + (size_t)q * c.stats_max * c.NZ + (size_t)n * c.NZ,
                      probes + (size_t)q * n * c.NZ);
    if (nsteps) *nsteps = c.stats_n;
    return F8_OK;
}

int f8o_kernel_timing(f8_ctx *ctx, double *kernel_ms, long long *steps_timed) {
    (void)kernel_ms; (void)steps_timed;
    return ctx ? F8_ERR_UNSUPPORTED : F8_ERR_ARG;   // no device kernels
}

int f8o_selection_codes(f8_ctx *ctx, unsigned char *codes) {
    if (!ctx || !codes) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (c.codes.empty()) return F8_ERR_STATE;
    std::memcpy(codes, c.codes.data(), c.codes.size());
    return F8_OK;
}

int f8o_markers(f8_ctx *ctx, int *n, double *xy) {
    if (!ctx) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (n) *n = (int)c.mk.size();
    if (xy)
        for (size_t m = 0; m < c.mk.size(); ++m) { xy[2 * m] = c.mk[m].x; xy[2 * m + 1] = c.mk[m].y; }
    return F8_OK;
}

const char *f8o_strerror(int st) {
    switch (st) {
    case F8_OK: return "ok";
    case F8_ERR_ARG: return "invalid argument";
    case F8_ERR_STATE: return "call out of order";
    case F8_ERR_NOMEM: return "out of memory";
    case F8_ERR_NAN: return "NaN in the velocity field";
    case F8_ERR_UNSUPPORTED: return "unsupported option";
    case F8_ERR_TOO_LARGE: return "grid exceeds the fixed workspace of the allocation-free solve";
    case F8_WARN_NEWTON: return "Newton iteration limit reached in some cells";
    case F8_WARN_SOR: return "SOR iteration limit reached";
    default: return "unknown status";
    }
}

void f8o_destroy(f8_ctx *ctx) { delete reinterpret_cast<OCtx *>(ctx); }

int f8o_set_timing(f8_ctx *ctx, int enable) {
    if (!ctx) return F8_ERR_ARG;
    reinterpret_cast<OCtx *>(ctx)->timing = enable != 0;
    return F8_OK;
}

int f8o_timing(f8_ctx *ctx, double *total_ms, double *stage_ms, long long *steps) {
    if (!ctx) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    if (total_ms) *total_ms = c.total_ms;
    if (stage_ms) for (int q = 0; q < 7; ++q) stage_ms[q] = c.stage_ms[q];
    if (steps) *steps = c.timed_steps;
    return F8_OK;
}

int f8o_timing_reset(f8_ctx *ctx) {
    if (!ctx) return F8_ERR_ARG;
    OCtx &c = *reinterpret_cast<OCtx *>(ctx);
    c.total_ms = 0; for (double &v : c.stage_ms) v = 0; c.timed_steps = 0;
    return F8_OK;
}

// --- oracle-only controls and kernel-level entry points (tests) ------------

void f8o_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int f8o_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int f8o_set_sor_order(f8_ctx *ctx, int order) {
    if (!ctx || (order != 0 && order != 1)) return F8_ERR_ARG;
    reinterpret_cast<OCtx *>(ctx)->sor_order = order;
    return F8_OK;
}

double f8o_vieta(const double *a) { return vieta(a); }
// the value the eigen test gives one symmetric matrix (face_test on a pair of equal faces)
double f8o_eigen_test(int method, const double *a) { return face_test(method, a, a); }
void f8o_eig2(const double *a, double *out) { eig2(a, out[0], out[1]); }
double f8o_roma(double r) { return roma(r); }

// Gauss-Jordan with pivoting; A row-major n x n (n = 3 or 6).
int f8o_gauss(int n, const double *A, const double *b, double *x) {
    if (n == 6) {
        double Ah[6][7];
        for (int r = 0; r < 6; ++r) { for (int q = 0; q < 6; ++q) Ah[r][q] = A[r * 6 + q]; Ah[r][6] = b[r]; }
        gauss<6>(Ah, x);
        return 0;
    }
    if (n == 3) {
        double Ah[3][4];
        for (int r = 0; r < 3; ++r) { for (int q = 0; q < 3; ++q) Ah[r][q] = A[r * 3 + q]; Ah[r][3] = b[r]; }
        gauss<3>(Ah, x);
        return 0;
    }
    return F8_ERR_ARG;
}

// Real Thomas solve with the reference's guard (sample6.f90 pins it).
void f8o_tdma(int n, const double *a, const double *b, const double *cc, const double *d, double *x) {
    std::vector<double> di(n, 0.0), xi(n), P(n), Qr(n), Qi(n);
    tdma(n, a, b, cc, d, di.data(), x, xi.data(), P.data(), Qr.data(), Qi.data());
}

// Forward unnormalised complex DFT of one line (re, im in place).
int f8o_fft_line(int n, double *re, double *im, int sign) {
    if (!is_pow2(n)) return F8_ERR_ARG;
    std::vector<double> tr, ti, sr(n), si(n);
    make_tw(n, tr, ti);
    fft_line(re, im, n, Tw{tr.data(), ti.data()}, sign, sr.data(), si.data());
    return 0;
}

// Periodic Helmholtz/Poisson solve on an interior-ordered field q (nx*ny*nz),
// LHS = lhs0 + lhs1 * k~^2; result (interior order) in phi.  Same argument
// order as the library's f8_fft_solve (host pointers here).
int f8o_fft_solve(int nx, int ny, int nz, double lx, double ly, double lz, const double *q, double *out, double lhs0, double lhs1) {
    f8_grid g{}; g.dim = nz == 1 ? 2 : 3; g.nx = nx; g.ny = ny; g.nz = nz; g.lx = lx; g.ly = ly; g.lz = lz;
    f8_phys ph; f8o_default_phys(&ph);
    f8_ctx *cx = nullptr;
    int st = f8o_create(&cx, &g, &ph, nullptr, 0, F8_FP64, F8_POISSON_FFT);
    if (st) return st;
    OCtx &c = *reinterpret_cast<OCtx *>(cx);
    std::vector<double> Q(q, q + c.ni()), H(c.nh(), 0.0);
    fft_solve_periodic(c, Q, lhs0, lhs1, H.data());
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) out[c.iidx(i, j, k)] = H[c.hidx(i, j, k)];
    f8o_destroy(cx);
    return 0;
}

// The oracle allocates freely; it exports the allocation-free name so that
// one harness can bind both libraries.
int f8o_fft_solve_noalloc(int nx, int ny, int nz, double lx, double ly, double lz, const double *q, double *out,
                          double lhs0, double lhs1) {
    return f8o_fft_solve(nx, ny, nz, lx, ly, lz, q, out, lhs0, lhs1);
}

}  // extern "C"
