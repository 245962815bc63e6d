// f8_fftsolve.cu — stand-alone periodic spectral solve, the reference's
// fft_solve (fenep.f90:1400-1428): Phi = IFFT( FFT(Q) / (NX NY NZ) / LHS )
// with LHS = lhs0 + lhs1 * (k~x^2 + k~y^2 + k~z^2) and the modified wavenumbers
// k~^2 = 2 (1 - cos(2 pi m / N)) / d^2 (fenep.f90:1458-1460, 1539-1541);
// modes with |LHS| < 1e-16 are set to zero.  lhs0 = 1, lhs1 = dt beta/(2 Re)
// is the CN Helmholtz solve of fft_navier; lhs0 = 0, lhs1 = -1 the pressure
// Poisson solve of fft_poisson.  FP64, compiled without FMA contraction, same
// transform as the time step's periodic solves.
#include <algorithm>
#include <cmath>
#include <vector>
#include "../../include/f8.h"
#include "f8_common.cuh"
#include "f8_fft.cuh"

namespace {

const double PI = 3.141592653589793238462643383279502884;

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Host-side tables of one grid: twiddles of the three axes and the modified
// wavenumbers, packed in one buffer (layout given by the offsets).
struct SolveTables {
    std::vector<double> buf;
    size_t twx_r, twx_i, twy_r, twy_i, twz_r, twz_i, kx2, ky2, kz2;
};

SolveTables make_tables(int nx, int ny, int nz, double lx, double ly, double lz) {
    SolveTables t;
    auto tw = [&](int n, size_t &ro, size_t &io) {
        const int h = std::max(1, n / 2);
        ro = t.buf.size();
        for (int q = 0; q < h; ++q) t.buf.push_back(q < n / 2 ? std::cos(2.0 * PI * q / n) : 1.0);
        io = t.buf.size();
        for (int q = 0; q < h; ++q) t.buf.push_back(q < n / 2 ? -std::sin(2.0 * PI * q / n) : 0.0);
    };
    tw(nx, t.twx_r, t.twx_i);
    tw(ny, t.twy_r, t.twy_i);
    tw(nz, t.twz_r, t.twz_i);
    const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
    t.kx2 = t.buf.size();
    for (int i = 1; i <= nx / 2 + 1; ++i) t.buf.push_back(2 * (1 - std::cos((i - 1) * (2 * PI / nx))) / (dx * dx));
    t.ky2 = t.buf.size();
    for (int j = 1; j <= ny; ++j) t.buf.push_back(2 * (1 - std::cos((j - 1) * (2 * PI / ny))) / (dy * dy));
    t.kz2 = t.buf.size();
    for (int k = 1; k <= nz; ++k) t.buf.push_back(2 * (1 - std::cos((k - 1) * (2 * PI / nz))) / (dz * dz));
    return t;
}

// The five passes of the periodic solve on device buffers: q (dense
// nx*ny*nz) -> phi (dense), spectrum workspace H of 2*(nx/2+1)*ny*nz doubles,
// tables as laid out by make_tables at dtab.
cudaError_t run_solve(const double *q, double *phi, double *H, const double *dtab, const SolveTables &t, int nx,
                      int ny, int nz, double lhs0, double lhs1, cudaStream_t s) {
    using namespace f8;
    const int nxh = nx / 2 + 1;
    const double *twx_r = dtab + t.twx_r, *twx_i = dtab + t.twx_i;
    const double *twy_r = dtab + t.twy_r, *twy_i = dtab + t.twy_i;
    const double *twz_r = dtab + t.twz_r, *twz_i = dtab + t.twz_i;
    const int tpp = std::max(nx / 2, 1), ppc = std::max(1, 256 / tpp);
    const int npp = ny / 2, total = npp * nz;
    const size_t smx = (size_t)ppc * 2 * nx * sizeof(Cx<double>);
    k_fft_x_fwd<double, double><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(q, H, nx, ny, 1, ny, npp, nz, twx_r, twx_i); count_launch();
    DivideSpec none{};
    const int txy = std::max(1, std::min(32, 2048 / ny));
    const size_t smy = (size_t)2 * ny * txy * sizeof(Cx<double>);
    k_fft_lines<double><<<dim3((nxh + txy - 1) / txy, nz), 256, smy, s>>>(H, ny, nxh, nxh, nxh * ny, txy, twy_r, twy_i, -1, 0, none); count_launch();
    DivideSpec dv{dtab + t.kx2, dtab + t.ky2, dtab + t.kz2, lhs0, lhs1, (double)nx * ny * nz, 1};
    const int txz = std::max(1, std::min(32, 2048 / nz));
    const size_t smz = (size_t)2 * nz * txz * sizeof(Cx<double>);
    k_fft_lines<double><<<dim3((nxh + txz - 1) / txz, ny), 256, smz, s>>>(H, nz, nxh * ny, nxh, nxh, txz, twz_r, twz_i, -1, 1, dv); count_launch();
    k_fft_lines<double><<<dim3((nxh + txy - 1) / txy, nz), 256, smy, s>>>(H, ny, nxh, nxh, nxh * ny, txy, twy_r, twy_i, +1, 0, none); count_launch();
    k_fft_x_inv<double, XOutD><<<(total + ppc - 1) / ppc, ppc * tpp, smx, s>>>(H, XOutD{phi, nullptr}, nx, ny, npp, nz, 0, nx, ny,
                                                                            twx_r, twx_i, 1); count_launch();
    return cudaGetLastError();
}

int check_args(int nx, int ny, int nz, double lx, double ly, double lz, const double *q, double *phi) {
    if (!q || !phi) return F8_ERR_ARG;
    if (!pow2(nx) || !pow2(ny) || !pow2(nz) || nx < 2 || ny < 2) return F8_ERR_ARG;
    if (nx > 1024 || ny > 1024 || nz > 1024) return F8_ERR_ARG;
    if (!(lx > 0 && ly > 0 && lz > 0)) return F8_ERR_ARG;
    return F8_OK;
}

cudaError_t set_smem_attrs() {
    using namespace f8;
    const int big = 200 * 1024;
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_lines<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_x_fwd<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    F8_CUDA_RET(cudaFuncSetAttribute(k_fft_x_inv<double, XOutD>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    return cudaSuccess;
}

}  // namespace

extern "C" int f8_fft_solve(int nx, int ny, int nz, double lx, double ly, double lz, const double *q, double *phi,
                            double lhs0, double lhs1) {
    if (int st = check_args(nx, ny, nz, lx, ly, lz, q, phi)) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return F8_ERR_NO_DEVICE;
    }
    if (set_smem_attrs() != cudaSuccess) return F8_ERR_CUDA;
    const SolveTables t = make_tables(nx, ny, nz, lx, ly, lz);
    double *H = nullptr, *dtab = nullptr;
    const size_t nspec = 2 * (size_t)(nx / 2 + 1) * ny * nz;
    int st = F8_OK;
    if (cudaMalloc(&H, nspec * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dtab, t.buf.size() * sizeof(double)) != cudaSuccess) {
        st = F8_ERR_NOMEM;
    } else if (cudaMemcpy(dtab, t.buf.data(), t.buf.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
               run_solve(q, phi, H, dtab, t, nx, ny, nz, lhs0, lhs1, 0) != cudaSuccess ||
               cudaStreamSynchronize(0) != cudaSuccess) {
        st = F8_ERR_CUDA;
    }
    if (H) cudaFree(H);
    if (dtab) cudaFree(dtab);
    cudaGetLastError();
    return st;
}

// ---------------------------------------------------------------------------
// Allocation-free variant.
//
// Some host programs cannot let a library call cudaMalloc: for example a
// solver driver that reserves all the device memory it may use at start-up
// (its own pool, or a budget shared with other jobs on the same GPU), so an
// allocation inside the time loop would fail or fragment that budget.  For
// them f8_fft_solve_noalloc runs the same periodic solve as f8_fft_solve with
// its workspace in fixed arrays of device memory, and calls no allocating
// routine.  With CUDA's lazy module loading the arrays are placed in device
// memory when this library's device code is first used on a device (which
// may be the first call of this entry point), so a caller makes that first
// call before it reserves the rest of the device memory for itself.
//
// Limits and rules (also stated in include/f8.h):
//  * the spectrum of the grid must fit in F8_NOALLOC_MAX_SPECTRUM complex
//    values, (nx/2+1)*ny*nz <= 135168 (for example 64^3, 128 x 64 x 32 or a
//    2D 512 x 256 field); larger grids get F8_ERR_TOO_LARGE;
//  * the arrays are shared by every call in the process on a device and keep
//    the last call's contents; each call overwrites all it reads (the forward
//    transform fills the whole spectrum and the tables are rewritten), so
//    nothing has to start at zero, but calls that overlap on the GPU (from
//    several host threads, or other streams) race on the arrays;
//  * the first call on a device looks up the device addresses of the arrays
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture on that device.  The addresses are kept for
//    the life of the process: after a cudaDeviceReset the library has to be
//    unloaded and loaded again before this entry point is used there.

#include <mutex>

#define F8_NOALLOC_MAX_SPECTRUM 135168   /* complex values: 65 * 64 * 32 = 33 * 64 * 64 */
#define F8_NOALLOC_MAX_TABLE 8192        /* doubles: twiddles and wavenumbers, N <= 1024 */

static __device__ __align__(256) double g_noalloc_spectrum[2 * F8_NOALLOC_MAX_SPECTRUM];
static __device__ __align__(256) double g_noalloc_table[F8_NOALLOC_MAX_TABLE];

namespace {

struct NoallocPtrs {
    double *spec = nullptr;
    double *tab = nullptr;
};

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoallocPtrs g_noalloc_ptrs[kMaxDevices];

// Device addresses of the fixed arrays on the current device (looked up once
// per device; the symbol names are host-side stand-ins, not device addresses).
int noalloc_setup(NoallocPtrs &out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return F8_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocPtrs &p = g_noalloc_ptrs[dev];
    if (!p.spec) {
        void *a = nullptr, *b = nullptr;
        if (cudaGetSymbolAddress(&a, g_noalloc_spectrum) != cudaSuccess ||
            cudaGetSymbolAddress(&b, g_noalloc_table) != cudaSuccess) {
            cudaGetLastError();
            return F8_ERR_CUDA;
        }
        if (set_smem_attrs() != cudaSuccess) {
            cudaGetLastError();
            return F8_ERR_CUDA;
        }
        p.spec = static_cast<double *>(a);
        p.tab = static_cast<double *>(b);
    }
    out = p;
    return F8_OK;
}

}  // namespace

extern "C" int f8_fft_solve_noalloc(int nx, int ny, int nz, double lx, double ly, double lz, const double *q,
                                    double *phi, double lhs0, double lhs1) {
    if (int st = check_args(nx, ny, nz, lx, ly, lz, q, phi)) return st;
    if ((size_t)(nx / 2 + 1) * ny * nz > (size_t)F8_NOALLOC_MAX_SPECTRUM) return F8_ERR_TOO_LARGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return F8_ERR_NO_DEVICE;
    }
    NoallocPtrs p;
    if (int st = noalloc_setup(p)) return st;
    const SolveTables t = make_tables(nx, ny, nz, lx, ly, lz);
    if (t.buf.size() > (size_t)F8_NOALLOC_MAX_TABLE) return F8_ERR_TOO_LARGE;
    if (cudaMemcpyAsync(p.tab, t.buf.data(), t.buf.size() * sizeof(double), cudaMemcpyHostToDevice, 0) != cudaSuccess ||
        run_solve(q, phi, p.spec, p.tab, t, nx, ny, nz, lhs0, lhs1, 0) != cudaSuccess ||
        cudaStreamSynchronize(0) != cudaSuccess) {
        cudaGetLastError();
        return F8_ERR_CUDA;
    }
    return F8_OK;
}
