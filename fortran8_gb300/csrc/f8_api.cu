// f8_api.cu — the C ABI of include/f8.h on one GB300.
//
// One context owns the device state of one solver instance (one CUDA stream).
// Host arrays cross the boundary only in f8_load / f8_store / f8_step's drag
// history; between calls the state stays resident in HBM.  The step loop body
// replaces the reference's main loop (fenep.f90:2477-2527).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <new>
#include <string>
#include <vector>
#include "../../include/f8.h"
#include "f8_kernels.h"

using namespace f8;

namespace {

const double PI = 3.141592653589793238462643383279502884;

struct Marker { double x, y, u, v; int cyl; };

// Marker set of one z-plane from the cylinder list, following ibm_init
// (fenep.f90:1784-1899, fenep_2d.f90:1472-1629): surface rings of
// nint(pi*DC/dX) points, or concentric shells i = 0..int(DC/(2dX)) of
// nint(pi*(DC-2 i dX)/dX) points with one centre point; ordered marker-major,
// cylinder-minor like the reference's (NC, NL, NZ) arrays.
std::vector<Marker> build_markers(const std::vector<f8_cyl> &cyl, double dX, int dim) {
    std::vector<std::vector<Marker>> per(cyl.size());
    for (size_t l = 0; l < cyl.size(); ++l) {
        const f8_cyl &cy = cyl[l];
        const double DC = 2.0 * cy.r;
        if (!cy.filled) {
            int NL = (int)std::lround(PI * DC / dX);
            if (NL < 1) NL = 1;
            for (int j = 1; j <= NL; ++j) {
                double ang = 2 * PI / NL * j;
                per[l].push_back({cy.xc + DC / 2 * std::cos(ang), cy.yc + DC / 2 * std::sin(ang),
                                  cy.spin * std::sin(ang), -cy.spin * std::cos(ang), (int)l});
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
                    per[l].push_back({cy.xc + rr * std::cos(ang), cy.yc + rr * std::sin(ang),
                                      cy.spin * ((DC - 2 * i * dX) / DC * std::sin(ang)),
                                      -cy.spin * ((DC - 2 * i * dX) / DC * std::cos(ang)), (int)l});
                }
        }
    }
    std::vector<Marker> out;
    size_t maxn = 0;
    for (auto &p : per) maxn = std::max(maxn, p.size());
    for (size_t m = 0; m < maxn; ++m)
        for (size_t l = 0; l < per.size(); ++l)
            if (m < per[l].size()) out.push_back(per[l][m]);
    if (dim == 2)  // fenep_2d.f90:1628-1629
        for (auto &m : out) { m.x = m.x + 10e-10 * dX; m.y = m.y + 10e-10 * dX; }
    return out;
}

void stencil_origin_h(int comp, double xc, double yc, double dX, double dY, int &i0, int &j0) {
    if (comp == 0) { j0 = (int)(yc / dY); i0 = (int)(xc / dX - 0.5); }
    else if (comp == 1) { j0 = (int)(yc / dY - 0.5); i0 = (int)(xc / dX); }
    else { j0 = (int)(yc / dY); i0 = (int)(xc / dX); }
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Device memory of f8_grad: the adjoint fields, the tape of one checkpoint
// segment (the fields the reverse of each step reads) and the checkpoints of
// the state.  Kept between calls; regrown when a call needs more.
struct GradMem {
    // four groups, each regrown on its own: the adjoint fields (grid), the
    // tape (segment length), the checkpoints (segments) and the drag weights
    std::vector<void *> mem[4];
    AdjState A{};
    int K = 0, nck = 0, nsteps = 0;
    int sor_capped = 0;                     // forward SOR solves of the call that reached sor_itrmax
    size_t ck_slot = 0;                     // doubles per checkpoint
    double *tU = nullptr, *tV = nullptr, *tW = nullptr, *tC = nullptr;
    double *tUa = nullptr, *tUp = nullptr, *tPhi = nullptr, *tFc = nullptr, *tCm = nullptr;
    uint8_t *tcodes = nullptr, *tcodes_g = nullptr;
    double *ck = nullptr, *dw = nullptr;
    // FP32-mixed contexts: adjoint fields, K tape slots of MIXED_TAPE_FIELDS
    // halo fields each (plus codes and marker forces), checkpoints of the
    // mixed state
    AdjStateF AF{};
    float *ftape = nullptr, *fck = nullptr;
    uint8_t *fcodes = nullptr, *fcodes_g = nullptr;
    double *fFc = nullptr;
    size_t fck_slot = 0;                    // floats per mixed checkpoint
    // CUDA graphs of the mixed gradient's steps, [2 * rec + parity]: the
    // forward step writing tape slot rec and the reverse step reading it
    // (parity: which buffer of the C pair, or of the adjoint C pair, is
    // current); kernels per replay of each kind
    std::vector<cudaGraphExec_t> gfwd, grev;
    long long gfwd_launches = 0, grev_launches = 0;
    double *dw_slot = nullptr;              // drag weights of the step a replayed reverse step reads
    float *lc_base = nullptr;               // the adjoint C buffer of parity 0
    void drop_graphs() {
        for (auto *v : {&gfwd, &grev}) {
            for (cudaGraphExec_t &ge : *v)
                if (ge) cudaGraphExecDestroy(ge);
            v->clear();
        }
    }
    template <typename T>
    cudaError_t get(int grp, T **p, size_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        mem[grp].push_back(q);
        *p = static_cast<T *>(q);
        return cudaSuccess;
    }
    void free_group(int grp) {
        for (void *p : mem[grp]) cudaFree(p);
        mem[grp].clear();
    }
    void free_all() {
        drop_graphs();
        for (int q = 0; q < 4; ++q) free_group(q);
        *this = GradMem{};
    }
};

}  // namespace

struct f8_ctx {
    f8_grid grid{};                   // the grid the step runs on (y and z exchanged for F8_BC_WALLS_Z)
    f8_grid user_grid{};              // the caller's grid
    bool zwalls = false;              // F8_BC_WALLS_Z: fields are exchanged at the boundary
    std::vector<double> zbuf[15];     // host staging of the exchanged fields
    std::vector<double> zbuf2[15];    // a second set (f8_grad: seed and state adjoint)
    f8_phys phys{};
    std::vector<f8_cyl> cyl;
    std::vector<double> cyl_vol;      // drag / spreading volume of each cylinder's markers
    std::vector<Marker> mk;
    int precision = 0, poisson = 0;
    Dev d{};
    cudaStream_t s = nullptr;
    bool loaded = false;
    int step = 0;            // steps taken (absolute, includes step0)
    int step0 = 0;
    std::vector<void *> allocs;
    double *drag_dev = nullptr;
    int drag_cap = 0;
    double *scratch_aos = nullptr;   // ncomp * cs doubles (C transposes)
    unsigned long long *nan_dev = nullptr;
    double *diag_part = nullptr;      // block partials of the on-device diagnostics
    double *slice_dev = nullptr;      // 18 doubles per point of the largest slice
    SpecWork spec{};                  // spectrum workspace (first f8_spectrum call)
    double *mean_dev = nullptr;       // mean velocity fields of f8_turbulence / f8_spectrum
    double *energy_dev = nullptr;
    // CUDA graphs of the mixed FFT step, one per parity of the C / C-new
    // buffer pair (the step swaps them), replayed when no stage timing,
    // AB2 start or SOR is requested
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    float *cf_base = nullptr;
    // one device block holds the step counters (cumulative since the load;
    // a call reports the difference from cnt_prev) followed by the drag slot
    // that the replayed step writes, so that a one-step call reads both back
    // with one copy into the same layout on the host (res_host)
    unsigned char *res_dev = nullptr;
    unsigned char *res_host = nullptr;
    size_t res_bytes = 0;
    double *drag_slot = nullptr;
    StepCounters cnt_prev{};
    int *load_flags = nullptr;        // device: non-uniform body force components (f8_load)
    // pinned host staging of the per-call results (counters, NaN count, drag),
    // so that their copies are asynchronous and end with one synchronisation
    unsigned long long *nan_host = nullptr;
    double *drag_host = nullptr;
    size_t drag_host_n = 0;
    long long graph_launches = 0;
    int stats_mode = 0, stats_n = 0, stats_max = 0;   // running statistics (f8_stats_begin)
    double *stats_sum = nullptr, *stats_probe = nullptr;
    GradMem gm;                        // f8_grad buffers
    int grad_kept_segments = 0;        // mixed f8_grad: segments of the last call kept from its first pass
    long long last_newton_iters = 0, last_newton_unconv = 0;
    int last_poisson_iters = -1;
    std::string last_error;
    // device timing
    bool timing = false;
    std::vector<cudaEvent_t> evpool;
    cudaEvent_t tot0 = nullptr, tot1 = nullptr;
    double total_ms = 0.0, stage_ms[NSTAGE] = {}, kernel_ms[NKERNEL] = {};
    long long timed_steps = 0;
    long long kernel_steps = 0;    // steps covered by kernel_ms
    long long step_launches = 0;   // kernels launched by f8_step since load / timing reset

    template <typename T>
    cudaError_t alloc(T **p, size_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        allocs.push_back(q);
        *p = static_cast<T *>(q);
        return cudaMemsetAsync(q, 0, std::max<size_t>(n, 1) * sizeof(T), s);
    }
    void drop_graphs() {
        for (cudaGraphExec_t &ge : gexec)
            if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
        gm.drop_graphs();
    }
    void release() {
        for (cudaEvent_t e : evpool) cudaEventDestroy(e);
        evpool.clear();
        if (tot0) cudaEventDestroy(tot0);
        if (tot1) cudaEventDestroy(tot1);
        tot0 = tot1 = nullptr;
        drop_graphs();
        for (void *p : allocs) cudaFree(p);
        allocs.clear();
        if (res_host) cudaFreeHost(res_host);
        res_host = nullptr;
        if (nan_host) cudaFreeHost(nan_host);
        if (drag_host) cudaFreeHost(drag_host);
        nan_host = nullptr; drag_host = nullptr; drag_host_n = 0;
        gm.free_all();
        if (stats_probe) cudaFree(stats_probe);   // resized outside the allocation list
        stats_probe = nullptr;
        for (int b = 0; b < 2; ++b) {
            if (d.aux[b]) cudaStreamDestroy(d.aux[b]);
            if (d.ev_join[b]) cudaEventDestroy(d.ev_join[b]);
            d.aux[b] = nullptr;
            d.ev_join[b] = nullptr;
        }
        if (d.ev_fork) cudaEventDestroy(d.ev_fork);
        d.ev_fork = nullptr;
        for (cudaEvent_t &ev : d.ev_g) {
            if (ev) cudaEventDestroy(ev);
            ev = nullptr;
        }
        if (s) cudaStreamDestroy(s);
        s = nullptr;
    }
};

namespace {

int fail(f8_ctx *c, cudaError_t e, const char *where) {
    if (c) c->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? F8_ERR_NOMEM : F8_ERR_CUDA;
}

#define API_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e__ = (call);                             \
        if (e__ != cudaSuccess) return fail(ctx, e__, #call); \
    } while (0)

// wall_plane_cluster searches a few thousand candidate layouts
// (milliseconds); contexts of the same grid reuse the result
int cached_wall_plane(int ny, int nz, int optin, WallLayout *wl) {
    struct Entry { int cl; WallLayout wl; };
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, Entry> memo;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(ny, nz, optin);
    auto it = memo.find(key);
    if (it == memo.end()) {
        Entry e{0, WallLayout{0, 0, 0}};
        e.cl = wall_plane_cluster(ny, nz, (size_t)optin, &e.wl);
        it = memo.emplace(key, e).first;
    }
    *wl = it->second.wl;
    return it->second.cl;
}

int validate(const f8_grid *g, const f8_phys *ph, int ncyl, const f8_cyl *cy, int prec, int poisson) {
    if (!g || !ph) return F8_ERR_ARG;
    if (g->dim != 2 && g->dim != 3) return F8_ERR_ARG;
    if (g->nx < 4 || g->ny < 4 || g->nz < 1) return F8_ERR_ARG;
    if (g->dim == 2 && g->nz != 1) return F8_ERR_ARG;
    if (g->dim == 3 && g->nz < 4) return F8_ERR_ARG;
    if (!(g->lx > 0 && g->ly > 0 && g->lz > 0)) return F8_ERR_ARG;
    if (g->bc_y != F8_BC_PERIODIC && g->bc_y != F8_BC_WALLS && g->bc_y != F8_BC_WALLS_Z) return F8_ERR_ARG;
    if (g->bc_y == F8_BC_WALLS_Z && (g->dim != 3 || ncyl > 0)) return F8_ERR_UNSUPPORTED;
    if (!is_pow2(g->nx) || !is_pow2(g->ny) || !is_pow2(g->nz)) return F8_ERR_ARG;  // spectral solves
    if (g->nx > 1024 || g->ny > 1024 || g->nz > 1024) return F8_ERR_ARG;
    if ((long)(g->nx + 2) * (g->ny + 2) * (g->nz + 2) > (1L << 31) / 8) return F8_ERR_ARG;
    if (poisson != F8_POISSON_FFT && poisson != F8_POISSON_SOR) return F8_ERR_ARG;
    if (prec != F8_FP64 && prec != F8_MIXED) return F8_ERR_ARG;
    if (!(ph->dt > 0) || !(ph->re > 0) || !(ph->wi > 0)) return F8_ERR_ARG;
    if (ph->newton_itrmax < 1 || ph->sor_itrmax < 1) return F8_ERR_ARG;
    if (ncyl < 0 || (ncyl > 0 && !cy)) return F8_ERR_ARG;
    if (ph->ibm_repeats < 1 || ph->ibm_repeats > 64) return F8_ERR_ARG;
    if (ph->eigen_test < F8_EIGEN_VIETA || ph->eigen_test > F8_EIGEN_SYMMETRIC) return F8_ERR_ARG;
    if (ph->eigen_test != F8_EIGEN_VIETA && (g->dim != 3 || prec != F8_FP64)) return F8_ERR_UNSUPPORTED;
    if (ph->ibm_volume != F8_IBM_CELL_VOLUME && ph->ibm_volume != F8_IBM_ARC_VOLUME) return F8_ERR_ARG;
    if (ph->ibm_volume == F8_IBM_ARC_VOLUME) {
        // the arc element of a surface ring (smac.f90:1128-1129), 3D
        if (g->dim != 3) return F8_ERR_UNSUPPORTED;
        for (int l = 0; l < ncyl; ++l)
            if (cy[l].filled) return F8_ERR_UNSUPPORTED;
    }
    return F8_OK;
}

void make_tw(int n, std::vector<double> &r, std::vector<double> &i) {
    int h = std::max(1, n / 2);
    r.assign(h, 1.0); i.assign(h, 0.0);
    for (int t = 0; t < n / 2; ++t) {
        double a = 2.0 * PI * t / n;
        r[t] = std::cos(a);
        i[t] = -std::sin(a);
    }
}

int upload(f8_ctx *c, double **dst, const std::vector<double> &v) {
    API_CUDA(c, c->alloc(dst, v.size()));
    API_CUDA(c, cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, c->s));
    return F8_OK;
}

int upload_f(f8_ctx *c, float **dst, const std::vector<double> &v) {
    std::vector<float> f(v.begin(), v.end());
    API_CUDA(c, c->alloc(dst, f.size()));
    API_CUDA(c, cudaMemcpyAsync(*dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

int upload_i(f8_ctx *c, int **dst, const std::vector<int> &v) {
    API_CUDA(c, c->alloc(dst, std::max<size_t>(v.size(), 1)));
    if (!v.empty()) API_CUDA(c, cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

// Kernel of the IBM delta function (fenep.f90:2045-2055), host copy.
double roma_h(double r) {
    double ar = std::fabs(r);
    if (ar < 1.5 && ar >= 0.5) return (5.0 - 3.0 * ar - std::sqrt(-3.0 * ((1 - ar) * (1 - ar)) + 1.0)) / 6.0;
    if (ar < 0.5) return (1.0 + std::sqrt(-3.0 * (r * r) + 1.0)) / 3.0;
    return 0.0;
}

int setup(f8_ctx *c) {
    const f8_grid &G = c->grid;
    Dev &d = c->d;
    Geo &g = d.g;
    g.nx = G.nx; g.ny = G.ny; g.nz = G.nz;
    g.sx = G.nx + 2; g.sy = G.ny + 2; g.sz = G.nz + 2;
    g.dim = G.dim; g.walls = G.bc_y == F8_BC_WALLS;
    g.dx = G.lx / G.nx; g.dy = G.ly / G.ny; g.dz = G.dim == 3 ? G.lz / G.nz : g.dx;
    g.dt = c->phys.dt; g.uwall = G.uwall;
    d.ph = Phys{c->phys.re, c->phys.wi, c->phys.beta, c->phys.lp2, c->phys.dt,
                c->phys.newton_dc, c->phys.newton_eps, c->phys.newton_itrmax, c->phys.eigen_test};
    d.ibm_repeats = c->phys.ibm_repeats;
    d.ncomp = G.dim == 3 ? 6 : 3;
    d.cs = g.sx * g.sy * g.sz;
    d.ni = g.nx * g.ny * g.nz;
    API_CUDA(c, cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
    API_CUDA(c, init_kernels_fp64());
    API_CUDA(c, cudaEventCreate(&c->tot0));
    API_CUDA(c, cudaEventCreate(&c->tot1));
    const size_t cs = d.cs, ni = d.ni;
    const bool mixed = c->precision == F8_MIXED;
    if (mixed) API_CUDA(c, init_kernels_mixed());
    for (double **p : {&d.U, &d.V, &d.W, &d.P, &d.Phi, &d.Up, &d.Vp, &d.Wp})
        API_CUDA(c, c->alloc(p, cs));
    API_CUDA(c, c->alloc(&c->scratch_aos, cs * d.ncomp));
    API_CUDA(c, c->alloc(&d.codes, ni));
    API_CUDA(c, c->alloc(&d.codes_g, 2 * (size_t)g.nx * g.nz));
    const size_t nxh = g.nx / 2 + 1;
    const size_t nspec = 2 * nxh * (size_t)(g.ny + 2) * g.nz;
    if (!mixed) {
        for (double **p : {&d.fpet, &d.Ua, &d.Va, &d.Wa}) API_CUDA(c, c->alloc(p, cs));
        API_CUDA(c, c->alloc(&d.C, cs * d.ncomp));
        API_CUDA(c, c->alloc(&d.Cn, cs * d.ncomp));
        for (double **p : {&d.Ax0, &d.Ay0, &d.Az0, &d.Tx0, &d.Ty0, &d.Tz0, &d.Fx, &d.Fy, &d.Fz, &d.Bx, &d.By, &d.Bz,
                           &d.Q[0], &d.Q[1], &d.Q[2], &d.E})
            API_CUDA(c, c->alloc(p, ni));
        API_CUDA(c, c->alloc(&d.H, nspec));
        API_CUDA(c, c->alloc(&d.H2, nspec));
    } else {
        API_CUDA(c, c->alloc(&d.Cf, cs * d.ncomp));
        for (float **p : {&d.Uf, &d.Vf, &d.Wf, &d.Ul, &d.Vl, &d.Wl, &d.Pf, &d.Pl, &d.Phif, &d.Phil,
                          &d.dUf[0], &d.dUf[1], &d.dUf[2]})
            API_CUDA(c, c->alloc(p, cs));
        if (c->phys.ibm_repeats > 1 && !c->cyl.empty())
            for (int q = 0; q < 3; ++q) API_CUDA(c, c->alloc(&d.Qpre[q], ni));
        API_CUDA(c, c->alloc(&d.Cnf, cs * d.ncomp));
        c->cf_base = d.Cf;
        API_CUDA(c, c->alloc(&d.fpetf, cs));
        API_CUDA(c, c->alloc(&d.fixlist, ni));
        API_CUDA(c, c->alloc(&d.fixcnt, 1));
        for (int q = 0; q < 3; ++q) {
            API_CUDA(c, c->alloc(&d.A0f[q], ni));
            API_CUDA(c, c->alloc(&d.T0f[q], ni));
            API_CUDA(c, c->alloc(&d.Ff[q], ni));
            API_CUDA(c, c->alloc(&d.Qf[q], ni));
        }
        API_CUDA(c, c->alloc(&d.Rhf, ni));
        API_CUDA(c, c->alloc(&d.Rlf, ni));
        API_CUDA(c, c->alloc(&d.Rdf, ni));
        API_CUDA(c, c->alloc(&d.Hf, nspec));
        API_CUDA(c, c->alloc(&d.H2f, nspec));
    }
    API_CUDA(c, c->alloc(&d.red, 4096));
    API_CUDA(c, c->alloc(&d.scal, 64));
    API_CUDA(c, c->alloc(&d.flag, 4));
    c->res_bytes = sizeof(StepCounters) + c->cyl.size() * 3 * sizeof(double);
    static_assert(sizeof(StepCounters) % sizeof(double) == 0, "drag slot alignment");
    API_CUDA(c, c->alloc(&c->res_dev, c->res_bytes));
    API_CUDA(c, cudaHostAlloc((void **)&c->res_host, c->res_bytes, cudaHostAllocDefault));
    d.cnt = reinterpret_cast<StepCounters *>(c->res_dev);
    if (c->cyl.size()) c->drag_slot = reinterpret_cast<double *>(c->res_dev + sizeof(StepCounters));
    API_CUDA(c, c->alloc(&c->load_flags, 3));
    API_CUDA(c, c->alloc(&c->nan_dev, 1));
    API_CUDA(c, cudaHostAlloc((void **)&c->nan_host, sizeof(unsigned long long), cudaHostAllocDefault));
    API_CUDA(c, c->alloc(&c->diag_part, std::max(diag_partials(), turb_partials(0))));
    if (g.dim == 3) {
        const size_t np = std::max({(size_t)g.nx * g.ny, (size_t)g.nx * g.nz, (size_t)g.ny * g.nz});
        API_CUDA(c, c->alloc(&c->slice_dev, 18 * np));
    }
    std::vector<double> tr, ti;
    double **twd[3][2] = {{&d.twx_r, &d.twx_i}, {&d.twy_r, &d.twy_i}, {&d.twz_r, &d.twz_i}};
    float **twf[3][2] = {{&d.twxf_r, &d.twxf_i}, {&d.twyf_r, &d.twyf_i}, {&d.twzf_r, &d.twzf_i}};
    const int nn[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a) {
        make_tw(nn[a], tr, ti);
        if (!mixed) {
            if (int st = upload(c, twd[a][0], tr)) return st;
            if (int st = upload(c, twd[a][1], ti)) return st;
        } else {
            if (int st = upload_f(c, twf[a][0], tr)) return st;
            if (int st = upload_f(c, twf[a][1], ti)) return st;
        }
    }
    // modified wavenumbers 2(1-cos(m 2pi/N))/d^2 (fenep.f90:1458-1460 with
    // the angle step 2 pi/N, identical to (i-1)*dX in the reference's 2 pi box)
    const double thx = 2 * PI / g.nx, thy = 2 * PI / g.ny, thz = 2 * PI / g.nz;
    std::vector<double> kx2(nxh), ky2(g.ny), kz2(g.nz);
    for (int i = 1; i <= (int)nxh; ++i) kx2[i - 1] = 2 * (1 - std::cos((i - 1) * thx)) / (g.dx * g.dx);
    for (int j = 1; j <= g.ny; ++j) ky2[j - 1] = 2 * (1 - std::cos((j - 1) * thy)) / (g.dy * g.dy);
    for (int k = 1; k <= g.nz; ++k) kz2[k - 1] = 2 * (1 - std::cos((k - 1) * thz)) / (g.dz * g.dz);
    if (int st = upload(c, &d.kx2, kx2)) return st;
    if (int st = upload(c, &d.ky2, ky2)) return st;
    if (int st = upload(c, &d.kz2, kz2)) return st;
    if (mixed) {
        if (int st = upload_f(c, &d.kx2f, kx2)) return st;
        if (int st = upload_f(c, &d.ky2f, ky2)) return st;
        if (int st = upload_f(c, &d.kz2f, kz2)) return st;
        // shared memory of one (z, y) plane: walls 12 B x (NY+2 | 1) x NZ,
        // periodic 8 B x (NY+1) x NZ; opt-in limit 227 KB
        int dev = 0, optin = 0;
        API_CUDA(c, cudaGetDevice(&dev));
        API_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        d.plane_cl = g.walls ? cached_wall_plane(g.ny, g.nz, optin, &d.plane_wl) : 0;
        API_CUDA(c, setup_staged_projection(d));
        if (g.walls) d.fused_planes = (d.plane_cl > 0 || (size_t)12 * ((g.ny + 2) | 1) * g.nz <= (size_t)optin) ? 1 : 0;
        else d.fused_planes = (size_t)8 * (g.ny + 1) * g.nz <= (size_t)optin ? 1 : 0;
        if (g.dim == 2) d.fused_planes = 0;   // 2D: the line transforms and tridiagonal sweeps
        if (d.fused_planes) {
            // side streams and spectra of the V and W Helmholtz solves
            for (int b = 0; b < 2; ++b) {
                API_CUDA(c, c->alloc(&d.HfB[b], nspec));
                API_CUDA(c, cudaStreamCreateWithFlags(&d.aux[b], cudaStreamNonBlocking));
                API_CUDA(c, cudaEventCreateWithFlags(&d.ev_join[b], cudaEventDisableTiming));
            }
            API_CUDA(c, cudaEventCreateWithFlags(&d.ev_fork, cudaEventDisableTiming));
            for (int q = 0; q < 4; ++q) API_CUDA(c, cudaEventCreateWithFlags(&d.ev_g[q], cudaEventDisableTiming));
        }
        {
            // stage-major twiddles of the warp transforms: stage span m holds
            // w^(p N / (2m)), p < m, at m - 1 + p (N entries, the last unused)
            auto stage_table = [](int n) {
                std::vector<float2> t(std::max(1, n));
                for (int m = 1; m < n; m <<= 1)
                    for (int p = 0; p < m; ++p) {
                        const int q = p * (n / (2 * m));
                        const double a = 2.0 * PI * q / n;
                        t[m - 1 + p] = make_float2((float)std::cos(a), (float)-std::sin(a));
                    }
                return t;
            };
            const std::vector<float2> t2 = stage_table(g.nz), tx = stage_table(g.nx);
            API_CUDA(c, c->alloc(&d.twz2, t2.size()));
            API_CUDA(c, cudaMemcpyAsync(d.twz2, t2.data(), t2.size() * sizeof(float2), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, c->alloc(&d.twx2, tx.size()));
            API_CUDA(c, cudaMemcpyAsync(d.twx2, tx.data(), tx.size() * sizeof(float2), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, cudaStreamSynchronize(c->s));
        }
        if (g.walls && d.plane_cl > 0) {
            // Thomas pivots of the increment Helmholtz systems (U, V) and of the
            // pressure system (fenep_2d.f90:1222-1238, 1262-1277, 1318-1332;
            // tdma's guard, 1157-1160), for every (kx, kz)
            const int lj = g.ny + 2;
            const size_t nt = nxh * (size_t)g.nz * lj;
            const double kap = c->phys.dt * c->phys.beta / c->phys.re / 2.0, idy2 = 1.0 / (g.dy * g.dy);
            std::vector<float> tr(nt);
            for (int sys = 0; sys < 3; ++sys) {
                for (size_t kx = 0; kx < nxh; ++kx)
                    for (int kz = 0; kz < g.nz; ++kz) {
                        const double lam = kx2[kx] + kz2[kz];
                        double p = 0.0;
                        for (int j = 0; j < lj; ++j) {
                            double a, b, cc;
                            if (sys == 2) {  // pressure, Neumann rows
                                if (j == 0) { a = 1; b = -1; cc = 0; }
                                else if (j == lj - 1) { a = 1; b = 0; cc = -1; }
                                else { a = -(lam + 2.0 * idy2); b = idy2; cc = idy2; }
                            } else if (sys == 0) {  // U, W
                                if (j == 0) { a = 1; b = 1; cc = 0; }
                                else if (j == lj - 1) { a = 1; b = 0; cc = 1; }
                                else { a = 1.0 + kap * (lam + 2.0 * idy2); b = -kap * idy2; cc = b; }
                            } else {  // V
                                if (j == 0 || j >= g.ny) { a = 1; b = 0; cc = 0; }
                                else { a = 1.0 + kap * (lam + 2.0 * idy2); b = -kap * idy2; cc = b; }
                            }
                            const double den = j == 0 ? a : a + cc * p;
                            double rd;
                            if (std::fabs(den) < 1.0e-16) { p = 0.0; rd = 0.0; }
                            else { p = -b / den; rd = 1.0 / den; }
                            tr[(kx * g.nz + kz) * (size_t)lj + j] = (float)rd;
                        }
                    }
                std::vector<double> trd(tr.begin(), tr.end());
                if (int st = upload_f(c, &d.wtR[sys], trd)) return st;
            }
        }
    }
    // IBM markers and the gather lists of the spreading kernel
    d.ncyl = (int)c->cyl.size();
    if (!c->cyl.empty()) {
        if (std::fabs(g.dx - g.dy) > 1e-14 * g.dx || (g.dim == 3 && std::fabs(g.dx - g.dz) > 1e-14 * g.dx))
            return F8_ERR_ARG;  // fenep.f90:1808-1810
        c->mk = build_markers(c->cyl, g.dx, g.dim);
        const int nm = (int)c->mk.size();
        d.nm = nm;
        std::vector<double> mx(nm), my(nm), mu(nm), mv(nm);
        std::vector<int> mc(nm);
        for (int m = 0; m < nm; ++m) { mx[m] = c->mk[m].x; my[m] = c->mk[m].y; mu[m] = c->mk[m].u; mv[m] = c->mk[m].v; mc[m] = c->mk[m].cyl; }
        if (int st = upload(c, &d.mx, mx)) return st;
        if (int st = upload(c, &d.my, my)) return st;
        if (int st = upload(c, &d.mu, mu)) return st;
        if (int st = upload(c, &d.mv, mv)) return st;
        {
            // spreading volume of each marker and the drag volume of each
            // cylinder: dX^3 (fenep.f90:2166-2187) with the cell volume as the
            // drag's, or the arc element pi*DC/NL * dX * dX of the cylinder's
            // ring (smac.f90:1128-1129, 1428-1446) for both
            const double dxn = g.dim == 3 ? g.dx * g.dx * g.dx : g.dx * g.dx;
            const double dvol = g.dim == 3 ? (g.dx * g.dy) * g.dz : g.dx * g.dy;
            std::vector<double> cv(c->cyl.size(), dvol), mvol(nm, dxn);
            if (c->phys.ibm_volume == F8_IBM_ARC_VOLUME)
                for (size_t l = 0; l < c->cyl.size(); ++l) {
                    const double DC = 2.0 * c->cyl[l].r;
                    const int NL = std::max(1, (int)std::lround(PI * DC / g.dx));
                    cv[l] = PI * DC / NL * g.dx * g.dx;
                }
            if (c->phys.ibm_volume == F8_IBM_ARC_VOLUME)
                for (int m = 0; m < nm; ++m) mvol[m] = cv[c->mk[m].cyl];
            c->cyl_vol = cv;
            if (int st = upload(c, &d.mvol, mvol)) return st;
            if (int st = upload(c, &d.cylvol, cv)) return st;
        }
        API_CUDA(c, c->alloc(&d.mcyl, nm));
        API_CUDA(c, cudaMemcpyAsync(d.mcyl, mc.data(), nm * sizeof(int), cudaMemcpyHostToDevice, c->s));
        {
            std::vector<int> perm, off(c->cyl.size() + 1, 0);
            for (size_t l = 0; l < c->cyl.size(); ++l) {
                for (int m = 0; m < nm; ++m)
                    if (mc[m] == (int)l) perm.push_back(m);
                off[l + 1] = (int)perm.size();
            }
            if (int st = upload_i(c, &d.mperm, perm)) return st;
            if (int st = upload_i(c, &d.moff, off)) return st;
            API_CUDA(c, c->alloc(&d.dragpart, c->cyl.size() * (size_t)g.nz * 3));
        }
        const int ncomp = g.dim == 3 ? 3 : 2;
        const int ncol = g.sx * g.sy;
        const double dvol_m = g.dim == 3 ? (g.dx * g.dy) * g.dz : g.dx * g.dy;   // cell volume
        for (int comp = 0; comp < 3; ++comp) {
            API_CUDA(c, c->alloc(&d.Fc[comp], (size_t)nm * g.nz));
            if (mixed) API_CUDA(c, c->alloc(&d.Fcf[comp], (size_t)nm * g.nz));
            std::vector<int> off(ncol + 1, 0), idx;
            std::vector<std::vector<int>> lists(ncol);
            if (comp < ncomp)
                for (int m = 0; m < nm; ++m) {
                    int i0, j0;
                    stencil_origin_h(comp, mx[m], my[m], g.dx, g.dy, i0, j0);
                    for (int jj = j0; jj <= j0 + 2; ++jj)
                        for (int ii = i0; ii <= i0 + 2; ++ii) {
                            if (ii < 0 || ii >= g.sx || jj < 0 || jj >= g.sy) return F8_ERR_ARG;  // marker too close to the edge
                            lists[ii + g.sx * jj].push_back(m);
                            if (ii == 0 || ii == g.sx - 1 || jj == 0 || jj >= g.ny) d.ibm_edge = 1;
                        }
                }
            for (int q = 0; q < ncol; ++q) off[q + 1] = off[q] + (int)lists[q].size();
            idx.reserve(off[ncol]);
            for (int q = 0; q < ncol; ++q) idx.insert(idx.end(), lists[q].begin(), lists[q].end());
            API_CUDA(c, c->alloc(&d.csr_off[comp], off.size()));
            API_CUDA(c, cudaMemcpyAsync(d.csr_off[comp], off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, c->alloc(&d.csr_idx[comp], std::max<size_t>(idx.size(), 1)));
            if (!idx.empty())
                API_CUDA(c, cudaMemcpyAsync(d.csr_idx[comp], idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, cudaStreamSynchronize(c->s));
            if (mixed && comp < ncomp) {
                // separable 1D kernel weights of each marker and the interior
                // columns that receive spreading (after the periodic fold)
                std::vector<double> wx(3 * (size_t)nm), wy(3 * (size_t)nm);
                std::vector<int> i0v(nm), j0v(nm);
                for (int m = 0; m < nm; ++m) {
                    int i0, j0;
                    stencil_origin_h(comp, mx[m], my[m], g.dx, g.dy, i0, j0);
                    i0v[m] = i0; j0v[m] = j0;
                    for (int a = 0; a < 3; ++a) {
                        double xg = (i0 + a - 0.5) * g.dx + (comp == 0 ? 0.5 * g.dx : 0.0);
                        double yg = (j0 + a - 0.5) * g.dy + (comp == 1 ? 0.5 * g.dy : 0.0);
                        wx[3 * m + a] = roma_h((xg - mx[m]) / g.dx);
                        wy[3 * m + a] = roma_h((yg - my[m]) / g.dy);
                    }
                }
                if (int st = upload_f(c, &d.mwx[comp], wx)) return st;
                if (int st = upload_f(c, &d.mwy[comp], wy)) return st;
                // the FP32 product wx * wy of each list entry (the spreading
                // multiplies it by the z weight), as the kernel would form it
                std::vector<double> cw(std::max<size_t>(idx.size(), 1), 0.0);
                for (int q = 0; q < ncol; ++q) {
                    const int ii = q % g.sx, jj = q / g.sx;
                    for (int e = off[q]; e < off[q + 1]; ++e) {
                        const int m = idx[e];
                        const float fx = (float)wx[3 * (size_t)m + (ii - i0v[m])];
                        const float fy = (float)wy[3 * (size_t)m + (jj - j0v[m])];
                        cw[e] = (double)(fx * fy);
                        if (c->phys.ibm_volume == F8_IBM_ARC_VOLUME)   // spreading volume / cell volume
                            cw[e] = (double)(fx * fy * (float)(c->cyl_vol[mc[m]] / dvol_m));
                    }
                }
                if (int st = upload_f(c, &d.csr_w[comp], cw)) return st;
                if (int st = upload_i(c, &d.mi0[comp], i0v)) return st;
                if (int st = upload_i(c, &d.mj0[comp], j0v)) return st;
                std::vector<int> act;
                for (int j = 1; j <= g.ny; ++j)
                    for (int i = 1; i <= g.nx; ++i) {
                        int xs[2] = {i, -1}, ys[2] = {j, -1};
                        if (i == 1) xs[1] = g.nx + 1; else if (i == g.nx) xs[1] = 0;
                        if (!g.walls) { if (j == 1) ys[1] = g.ny + 1; else if (j == g.ny) ys[1] = 0; }
                        bool any = false;
                        for (int a = 0; a < 2 && !any; ++a)
                            for (int b2 = 0; b2 < 2 && !any; ++b2)
                                if (xs[a] >= 0 && ys[b2] >= 0 && !lists[xs[a] + g.sx * ys[b2]].empty()) any = true;
                        if (any) act.push_back((i - 1) + g.nx * (j - 1));
                    }
                d.nact[comp] = (int)act.size();
                if (int st = upload_i(c, &d.act_cols[comp], act)) return st;
            }
        }
        if (!mixed) {
            for (int comp = 0; comp < 3; ++comp) {
                API_CUDA(c, c->alloc(&d.mwxd[comp], 3 * (size_t)nm));
                API_CUDA(c, c->alloc(&d.mwyd[comp], 3 * (size_t)nm));
                API_CUDA(c, c->alloc(&d.mwzd[comp], 3 * (size_t)g.nz));
                API_CUDA(c, c->alloc(&d.mi0d[comp], nm));
                API_CUDA(c, c->alloc(&d.mj0d[comp], nm));
            }
            API_CUDA(c, marker_weights_fp64(d, c->s));
        }
        // the interpolation stencil reads k = n-1 .. n+1 and marker columns
        // inside the halo box; validated above through the gather lists
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

int ensure_drag(f8_ctx *c, int nsteps) {
    if (c->cyl.empty() || nsteps <= c->drag_cap) return F8_OK;
    // grow geometrically and free the smaller buffer (no work on it is in
    // flight: every f8_step call ends with a synchronisation)
    int cap = std::max({nsteps, 64, 2 * c->drag_cap});
    if (c->drag_dev) {
        API_CUDA(c, cudaStreamSynchronize(c->s));
        auto it = std::find(c->allocs.begin(), c->allocs.end(), (void *)c->drag_dev);
        if (it != c->allocs.end()) c->allocs.erase(it);
        cudaFree(c->drag_dev);
        c->drag_dev = nullptr;
        c->drag_cap = 0;
    }
    double *p = nullptr;
    API_CUDA(c, c->alloc(&p, (size_t)cap * c->cyl.size() * 3));
    c->drag_dev = p;
    c->drag_cap = cap;
    if (c->drag_host) cudaFreeHost(c->drag_host);
    c->drag_host = nullptr;
    c->drag_host_n = 0;
    API_CUDA(c, cudaHostAlloc((void **)&c->drag_host, (size_t)cap * c->cyl.size() * 3 * sizeof(double),
                              cudaHostAllocDefault));
    c->drag_host_n = (size_t)cap * c->cyl.size() * 3;
    return F8_OK;
}

// ---- walls normal to z (smac_kabe.f90) --------------------------------------
// The caller's fields (x, y, z) are the step's fields (x, y', z') = (x, z, y):
// halo and interior arrays are transposed in (y, z), the velocity-like
// components exchange y and z (u' = u, v' = w, w' = v), and the tensor C
// (xx, xy, xz, yy, yz, zz) becomes (xx, xz, xy, zz, zy, yy).
struct ZSwap {
    int nx, ny, nz;   // the caller's extents
    // caller (i, j, k) <-> step (i, k, j); halo = 1 with the halo layers
    template <bool Back>
    void move(const double *src, double *dst, int halo, int ncomp, const int *perm) const {
        const int sx = nx + 2 * halo, sy = ny + 2 * halo, sz = nz + 2 * halo;
        for (int k = 0; k < sz; ++k)
            for (int j = 0; j < sy; ++j)
                for (int i = 0; i < sx; ++i) {
                    const size_t u = (size_t)i + (size_t)sx * (j + (size_t)sy * k);   // caller
                    const size_t t = (size_t)i + (size_t)sx * (k + (size_t)sz * j);   // step
                    for (int m = 0; m < ncomp; ++m) {
                        const int mu = perm ? perm[m] : m;   // caller component of step component m
                        if (Back) dst[u * ncomp + mu] = src[t * ncomp + m];
                        else dst[t * ncomp + m] = src[u * ncomp + mu];
                    }
                }
    }
};

constexpr int C_SWAP[6] = {0, 2, 1, 5, 4, 3};

// pointers of the fields in the order below, with the halo flag and the
// source field of each step field (velocity-like triples exchange y and z)
void zwall_slots(f8_fields *f, double **slot[15]) {
    double **p[15] = {&f->u, &f->v, &f->w, &f->p, &f->phi, &f->c, &f->ax0, &f->ay0, &f->az0,
                      &f->tx0, &f->ty0, &f->tz0, &f->fx, &f->fy, &f->fz};
    for (int q = 0; q < 15; ++q) slot[q] = p[q];
}
constexpr int Z_SRC[15] = {0, 2, 1, 3, 4, 5, 6, 8, 7, 9, 11, 10, 12, 14, 13};   // step field q <- caller field Z_SRC[q]

// caller fields -> step fields in the context's staging buffers
void zwall_in(f8_ctx *c, const f8_fields *in, f8_fields *out, std::vector<double> (&buf)[15]) {
    const ZSwap zs{c->user_grid.nx, c->user_grid.ny, c->user_grid.nz};
    f8_fields src = *in;
    *out = f8_fields{};
    double **ps[15], **pd[15];
    zwall_slots(&src, ps);
    zwall_slots(out, pd);
    const size_t cs = (size_t)(zs.nx + 2) * (zs.ny + 2) * (zs.nz + 2), ni = (size_t)zs.nx * zs.ny * zs.nz;
    for (int q = 0; q < 15; ++q) {
        const double *from = *ps[Z_SRC[q]];
        if (!from) continue;
        const bool halo = q < 6, tensor = q == 5;
        buf[q].resize((halo ? cs : ni) * (tensor ? 6 : 1));
        zs.move<false>(from, buf[q].data(), halo ? 1 : 0, tensor ? 6 : 1, tensor ? C_SWAP : nullptr);
        *pd[q] = buf[q].data();
    }
}

// step fields (in the staging buffers) -> the caller's non-null arrays
void zwall_out(f8_ctx *c, const f8_fields *stepf, f8_fields *user) {
    const ZSwap zs{c->user_grid.nx, c->user_grid.ny, c->user_grid.nz};
    f8_fields sf = *stepf;
    double **ps[15], **pu[15];
    zwall_slots(&sf, ps);
    zwall_slots(user, pu);
    for (int q = 0; q < 15; ++q) {
        double *to = *pu[Z_SRC[q]];
        if (!to || !*ps[q]) continue;
        const bool halo = q < 6, tensor = q == 5;
        zs.move<true>(*ps[q], to, halo ? 1 : 0, tensor ? 6 : 1, tensor ? C_SWAP : nullptr);
    }
}

// staging buffers of the step fields a caller asked for
void zwall_stage(f8_ctx *c, const f8_fields *user, f8_fields *stepf, std::vector<double> (&buf)[15]) {
    const ZSwap zs{c->user_grid.nx, c->user_grid.ny, c->user_grid.nz};
    f8_fields u = *user;
    *stepf = f8_fields{};
    double **pu[15], **pd[15];
    zwall_slots(&u, pu);
    zwall_slots(stepf, pd);
    const size_t cs = (size_t)(zs.nx + 2) * (zs.ny + 2) * (zs.nz + 2), ni = (size_t)zs.nx * zs.ny * zs.nz;
    for (int q = 0; q < 15; ++q) {
        if (!*pu[Z_SRC[q]]) continue;
        const bool halo = q < 6, tensor = q == 5;
        buf[q].resize((halo ? cs : ni) * (tensor ? 6 : 1));
        *pd[q] = buf[q].data();
    }
}

}  // namespace

extern "C" {

void f8_default_phys(f8_phys *ph) {
    std::memset(ph, 0, sizeof(*ph));
    ph->re = 1.0; ph->wi = 1.0; ph->beta = 1.0; ph->lp2 = 100.0; ph->dt = 1.0e-3;
    ph->newton_dc = 1.0e-5; ph->newton_eps = 1.0e-6; ph->newton_itrmax = 10000;
    ph->sor_omega = 1.8; ph->sor_eps = 1.0e-5; ph->sor_itrmax = 10000;
    ph->ab2_start = 1;
    ph->ibm_volume = F8_IBM_CELL_VOLUME;
    ph->ibm_repeats = 1;
}

int f8_create(f8_ctx **out, const f8_grid *g, const f8_phys *ph, const f8_cyl *cy, int ncyl, int prec, int poisson) {
    if (!out) return F8_ERR_ARG;
    *out = nullptr;
    int st = validate(g, ph, ncyl, cy, prec, poisson);
    if (st) return st;
    // the 2D mixed step solves its pressure with the FFT solvers only
    if (prec == F8_MIXED && g->dim == 2 && poisson != F8_POISSON_FFT) return F8_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return F8_ERR_NO_DEVICE;
    }
    f8_ctx *c = new (std::nothrow) f8_ctx();
    if (!c) return F8_ERR_NOMEM;
    c->grid = *g; c->user_grid = *g; c->phys = *ph; c->precision = prec; c->poisson = poisson;
    if (g->bc_y == F8_BC_WALLS_Z) {
        // the walls-normal-to-z box is the y-walled box with y and z exchanged
        c->zwalls = true;
        c->grid.ny = g->nz; c->grid.nz = g->ny;
        c->grid.ly = g->lz; c->grid.lz = g->ly;
        c->grid.bc_y = F8_BC_WALLS;
    }
    if (ncyl > 0) c->cyl.assign(cy, cy + ncyl);
    st = setup(c);
    if (st) {
        c->release();
        delete c;
        return st;
    }
    *out = c;
    return F8_OK;
}

static int load_impl(f8_ctx *c, const f8_fields *in, int step0) {
    if (!c || !in || !in->u || !in->v || !in->p || !in->c || step0 < 0) return F8_ERR_ARG;
    if (c->grid.dim == 3 && !in->w) return F8_ERR_ARG;
    Dev &d = c->d;
    const size_t cs = d.cs, ni = d.ni;
    auto put = [&](double *dst, const double *src, size_t n) -> cudaError_t {
        if (src) return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, c->s);
        return cudaMemsetAsync(dst, 0, n * sizeof(double), c->s);
    };
    API_CUDA(c, put(d.U, in->u, cs));
    API_CUDA(c, put(d.V, in->v, cs));
    API_CUDA(c, put(d.W, c->grid.dim == 3 ? in->w : nullptr, cs));
    API_CUDA(c, put(d.P, in->p, cs));
    API_CUDA(c, put(d.Phi, in->phi, cs));
    API_CUDA(c, put(c->scratch_aos, in->c, cs * d.ncomp));
    if (c->precision == F8_FP64) {
        API_CUDA(c, aos_to_soa(c->scratch_aos, d.C, d.ncomp, (int)cs, c->s));
        API_CUDA(c, put(d.Ax0, in->ax0, ni)); API_CUDA(c, put(d.Ay0, in->ay0, ni)); API_CUDA(c, put(d.Az0, in->az0, ni));
        API_CUDA(c, put(d.Tx0, in->tx0, ni)); API_CUDA(c, put(d.Ty0, in->ty0, ni)); API_CUDA(c, put(d.Tz0, in->tz0, ni));
        API_CUDA(c, put(d.Fx, in->fx, ni)); API_CUDA(c, put(d.Fy, in->fy, ni)); API_CUDA(c, put(d.Fz, in->fz, ni));
        // boundary values of the loaded state (init calls PBM, fenep.f90:139-143)
        API_CUDA(c, bc_all_state_fp64(d, c->s));
    } else {
        API_CUDA(c, aos_to_soa_f(c->scratch_aos, d.Cf, d.ncomp, (int)cs, c->s));
        const double *src[9] = {in->ax0, in->ay0, in->az0, in->tx0, in->ty0, in->tz0, in->fx, in->fy, in->fz};
        float *dst[9] = {d.A0f[0], d.A0f[1], d.A0f[2], d.T0f[0], d.T0f[1], d.T0f[2], d.Ff[0], d.Ff[1], d.Ff[2]};
        double *tmp = c->scratch_aos;  // ncomp*cs >= ni doubles
        // the force conversions also flag a component that is not uniform
        API_CUDA(c, cudaMemsetAsync(c->load_flags, 0, 3 * sizeof(int), c->s));
        for (int q = 0; q < 9; ++q) {
            if (src[q]) {
                API_CUDA(c, cudaMemcpyAsync(tmp, src[q], ni * sizeof(double), cudaMemcpyHostToDevice, c->s));
                API_CUDA(c, d2f(tmp, dst[q], (int)ni, c->s, q >= 6 ? c->load_flags + (q - 6) : nullptr));
            } else {
                API_CUDA(c, cudaMemsetAsync(dst[q], 0, ni * sizeof(float), c->s));
            }
        }
        API_CUDA(c, bc_all_state_mixed(d, c->s));
    }
    API_CUDA(c, cudaMemsetAsync(d.cnt, 0, sizeof(StepCounters), c->s));
    int varies[3] = {0, 0, 0};
    if (c->precision == F8_MIXED)
        API_CUDA(c, cudaMemcpyAsync(varies, c->load_flags, sizeof(varies), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    c->cnt_prev = StepCounters{};
    if (c->precision == F8_MIXED) {
        // a spatially uniform body force component (the channel's driving
        // force) is passed to the momentum kernel as a constant.  The
        // replayed step graphs hold those kernel arguments, so a load that
        // changes them drops the graphs (recaptured at the next step).
        const double *f[3] = {in->fx, in->fy, in->fz};
        bool force_changed = false;
        for (int q = 0; q < 3; ++q) {
            const int u = f[q] && varies[q] ? 0 : 1;
            const float v = f[q] ? (float)f[q][0] : 0.0f;
            if (u != d.Funi[q] || v != d.Fval[q]) force_changed = true;
            d.Funi[q] = u;
            d.Fval[q] = v;
        }
        if (force_changed) c->drop_graphs();
    }
    c->step = step0;
    c->step0 = step0;
    c->loaded = true;
    c->step_launches = 0;
    return F8_OK;
}

int f8_step(f8_ctx *c, int nsteps, double *drag) {
    if (!c || nsteps < 0) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    if (nsteps == 0) return F8_OK;
    if (int st = ensure_drag(c, nsteps)) return st;
    Dev &d = c->d;
    const int ncyl = (int)c->cyl.size();
    // a one-step call of the replayed step reads its drag from the result
    // block together with the counters (one copy)
    bool drag_in_slot = false;
    // the mixed step counts non-finite velocities in its counters instead
    if (c->precision != F8_MIXED) API_CUDA(c, cudaMemsetAsync(c->nan_dev, 0, sizeof(unsigned long long), c->s));
    // per step: the stage boundaries, then the pairs around the single-launch
    // kernels of the mixed step
    const size_t per = NSTAGE + 1 + 2 * NKERNEL;
    if (c->timing && c->evpool.size() < per * nsteps) {
        size_t have = c->evpool.size();
        c->evpool.resize(per * nsteps, nullptr);
        for (size_t q = have; q < c->evpool.size(); ++q) API_CUDA(c, cudaEventCreate(&c->evpool[q]));
    }
    API_CUDA(c, cudaEventRecord(c->tot0, c->s));
    const long long launches0 = g_kernel_launches.load();
    int worst = F8_OK;
    for (int s = 0; s < nsteps; ++s) {
        StepOpts o{};
        o.polymer = c->phys.beta != 1.0;
        o.ab2_first = (c->step + 1 == 1) && c->phys.ab2_start;
        o.ibm = ncyl > 0;
        o.poisson = c->poisson;
        o.sor_omega = c->phys.sor_omega; o.sor_eps = c->phys.sor_eps; o.sor_itrmax = c->phys.sor_itrmax;
        o.ev = c->timing ? &c->evpool[per * s] : nullptr;
        o.kev = (c->timing && c->precision == F8_MIXED) ? &c->evpool[per * s + NSTAGE + 1] : nullptr;
        const bool mixed = c->precision == F8_MIXED;
        if (!o.polymer && s == 0) {
            // beta == 1: C and T vanish (fenep.f90:2479-2485)
            if (mixed) API_CUDA(c, cudaMemsetAsync(d.Cf, 0, (size_t)d.cs * d.ncomp * sizeof(float), c->s));
            else API_CUDA(c, cudaMemsetAsync(d.C, 0, (size_t)d.cs * d.ncomp * sizeof(double), c->s));
        }
        int sor_iters = -1;
        double *dg = (ncyl && drag) ? c->drag_dev + (size_t)s * ncyl * 3 : nullptr;
        const bool graph = mixed && !o.ev && !o.ab2_first && c->poisson == F8_POISSON_FFT;
        cudaError_t e = cudaSuccess;
        if (graph) {
            const int p = d.Cf == c->cf_base ? 0 : 1;
            if (!c->gexec[p]) {
                // capture one step; the capture runs no work, so the host-side
                // buffer swap the step makes is undone afterwards
                float *cf0 = d.Cf, *cn0 = d.Cnf;
                const long long l0 = g_kernel_launches.load();
                cudaGraph_t gr = nullptr;
                API_CUDA(c, cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
                e = step_mixed(d, o, ncyl ? c->drag_slot : nullptr, &sor_iters, c->s);
                const cudaError_t e2 = cudaStreamEndCapture(c->s, &gr);
                d.Cf = cf0;
                d.Cnf = cn0;
                c->graph_launches = g_kernel_launches.load() - l0;
                g_kernel_launches -= c->graph_launches;
                if (e == cudaSuccess) e = e2;
                if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gexec[p], gr, 0);
                if (gr) cudaGraphDestroy(gr);
                if (e != cudaSuccess) return fail(c, e, "graph capture");
            }
            e = cudaGraphLaunch(c->gexec[p], c->s);
            if (o.polymer) std::swap(d.Cf, d.Cnf);
            g_kernel_launches += c->graph_launches;
            if (e == cudaSuccess && dg) {
                if (nsteps == 1) drag_in_slot = true;
                else e = cudaMemcpyAsync(dg, c->drag_slot, (size_t)ncyl * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                         c->s);
            }
        } else {
            e = mixed ? step_mixed(d, o, dg, &sor_iters, c->s) : step_fp64(d, o, dg, &sor_iters, c->s);
        }
        if (e != cudaSuccess) return fail(c, e, "step");
        if (c->stats_mode) {
            API_CUDA(c, device_stats_accum(d, mixed, c->stats_mode, c->mean_dev, c->stats_sum, c->stats_probe,
                                           c->stats_n, c->stats_max, c->s));
            c->stats_n += 1;
        }
        c->last_poisson_iters = sor_iters;
        if (c->poisson == F8_POISSON_SOR && sor_iters > c->phys.sor_itrmax) worst = std::max(worst, (int)F8_WARN_SOR);
        c->step += 1;
    }
    API_CUDA(c, cudaEventRecord(c->tot1, c->s));
    // the mixed step counts non-finite velocities inside its projection kernel
    if (c->precision != F8_MIXED) API_CUDA(c, count_nonfinite(d.U, d.cs, c->nan_dev, c->s));
    c->step_launches += g_kernel_launches.load() - launches0;
    const size_t ndrag = (size_t)nsteps * ncyl * 3;
    *c->nan_host = 0;
    API_CUDA(c, cudaMemcpyAsync(c->res_host, c->res_dev, drag_in_slot ? c->res_bytes : sizeof(StepCounters),
                                cudaMemcpyDeviceToHost, c->s));
    if (c->precision != F8_MIXED)
        API_CUDA(c, cudaMemcpyAsync(c->nan_host, c->nan_dev, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->s));
    if (drag && ncyl && !drag_in_slot)
        API_CUDA(c, cudaMemcpyAsync(c->drag_host, c->drag_dev, ndrag * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    StepCounters now;
    std::memcpy(&now, c->res_host, sizeof(now));
    const StepCounters cnt{now.newton_iters - c->cnt_prev.newton_iters,
                           now.newton_unconverged - c->cnt_prev.newton_unconverged,
                           now.nan_cells - c->cnt_prev.nan_cells, now.copy_timeouts - c->cnt_prev.copy_timeouts};
    c->cnt_prev = now;
    const unsigned long long nan = *c->nan_host;
    if (drag && ncyl)
        std::memcpy(drag, drag_in_slot ? c->res_host + sizeof(StepCounters) : (const unsigned char *)c->drag_host,
                    ndrag * sizeof(double));
    {
        float ms = 0.f;
        API_CUDA(c, cudaEventElapsedTime(&ms, c->tot0, c->tot1));
        c->total_ms += ms;
        c->timed_steps += nsteps;
        if (c->timing)
            for (int s2 = 0; s2 < nsteps; ++s2)
                for (int q = 0; q < NSTAGE; ++q) {
                    API_CUDA(c, cudaEventElapsedTime(&ms, c->evpool[per * s2 + q], c->evpool[per * s2 + q + 1]));
                    c->stage_ms[q] += ms;
                }
        if (c->timing && c->precision == F8_MIXED) c->kernel_steps += nsteps;
        if (c->timing && c->precision == F8_MIXED)
            for (int s2 = 0; s2 < nsteps; ++s2)
                for (int q = 0; q < NKERNEL; ++q) {
                    const size_t e0 = per * s2 + NSTAGE + 1 + 2 * q;
                    API_CUDA(c, cudaEventElapsedTime(&ms, c->evpool[e0], c->evpool[e0 + 1]));
                    c->kernel_ms[q] += ms;
                }
    }
    c->last_newton_iters = (long long)cnt.newton_iters;
    c->last_newton_unconv = (long long)cnt.newton_unconverged;
    if (cnt.copy_timeouts) {
        c->last_error = "a bulk-copy wait of the projection kernel ran out; the step is incomplete";
        return F8_ERR_CUDA;
    }
    if (nan || cnt.nan_cells) return F8_ERR_NAN;
    if (cnt.newton_unconverged) worst = std::max(worst, (int)F8_WARN_NEWTON);
    return worst;
}

static int store_impl(f8_ctx *c, f8_fields *out) {
    if (!c || !out) return F8_ERR_ARG;
    Dev &d = c->d;
    const size_t cs = d.cs, ni = d.ni;
    auto get = [&](double *dst, const double *src, size_t n) -> cudaError_t {
        if (!dst) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->s);
    };
    if (c->precision == F8_MIXED && c->loaded) API_CUDA(c, mixed_state_to_fp64(d, c->s));
    API_CUDA(c, get(out->u, d.U, cs));
    API_CUDA(c, get(out->v, d.V, cs));
    if (c->grid.dim == 3) API_CUDA(c, get(out->w, d.W, cs));
    API_CUDA(c, get(out->p, d.P, cs));
    API_CUDA(c, get(out->phi, d.Phi, cs));
    if (c->precision == F8_FP64) {
        if (out->c) {
            API_CUDA(c, soa_to_aos(d.C, c->scratch_aos, d.ncomp, (int)cs, c->s));
            API_CUDA(c, get(out->c, c->scratch_aos, cs * d.ncomp));
        }
        API_CUDA(c, get(out->ax0, d.Ax0, ni)); API_CUDA(c, get(out->ay0, d.Ay0, ni)); API_CUDA(c, get(out->az0, d.Az0, ni));
        API_CUDA(c, get(out->tx0, d.Tx0, ni)); API_CUDA(c, get(out->ty0, d.Ty0, ni)); API_CUDA(c, get(out->tz0, d.Tz0, ni));
        API_CUDA(c, get(out->fx, d.Fx, ni)); API_CUDA(c, get(out->fy, d.Fy, ni)); API_CUDA(c, get(out->fz, d.Fz, ni));
    } else {
        if (out->c) {
            API_CUDA(c, soa_to_aos_f(d.Cf, c->scratch_aos, d.ncomp, (int)cs, c->s));
            API_CUDA(c, get(out->c, c->scratch_aos, cs * d.ncomp));
        }
        // the FP32 histories go through the FP64 staging area; each copy is
        // ordered on the stream before the next conversion overwrites it
        double *dsts[9] = {out->ax0, out->ay0, out->az0, out->tx0, out->ty0, out->tz0, out->fx, out->fy, out->fz};
        const float *srcs[9] = {d.A0f[0], d.A0f[1], d.A0f[2], d.T0f[0], d.T0f[1], d.T0f[2], d.Ff[0], d.Ff[1], d.Ff[2]};
        for (int q = 0; q < 9; ++q) {
            if (!dsts[q]) continue;
            API_CUDA(c, f2d(srcs[q], c->scratch_aos, (int)ni, c->s));
            API_CUDA(c, get(dsts[q], c->scratch_aos, ni));
        }
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

int f8_load(f8_ctx *c, const f8_fields *in, int step0) {
    if (!c || !in) return F8_ERR_ARG;
    if (!c->zwalls) return load_impl(c, in, step0);
    if (!in->u || !in->v || !in->w || !in->p || !in->c || step0 < 0) return F8_ERR_ARG;
    f8_fields t;
    zwall_in(c, in, &t, c->zbuf);
    return load_impl(c, &t, step0);
}

int f8_store(f8_ctx *c, f8_fields *out) {
    if (!c || !out) return F8_ERR_ARG;
    if (!c->zwalls) return store_impl(c, out);
    f8_fields t;
    zwall_stage(c, out, &t, c->zbuf);
    const int st = store_impl(c, &t);
    if (st == F8_OK) zwall_out(c, &t, out);
    return st;
}


}  // extern "C"

namespace {

int grad_alloc(f8_ctx *c, int K, int nck, int nsteps) {
    GradMem &G = c->gm;
    Dev &d = c->d;
    const size_t cs = d.cs, ni = d.ni, ncyl = c->cyl.size(), nfc = (size_t)d.nm * d.g.nz;
    if (!G.A.grad) {
        AdjState &A = G.A;
        for (double **p : {&A.lU, &A.lV, &A.lW, &A.lP, &A.lPhi}) API_CUDA(c, G.get(0, p, cs));
        for (double **p : {&A.lC, &A.lC2}) API_CUDA(c, G.get(0, p, 6 * cs));
        for (int q = 0; q < 3; ++q) {
            API_CUDA(c, G.get(0, &A.lA0[q], ni));
            API_CUDA(c, G.get(0, &A.lT0[q], ni));
            API_CUDA(c, G.get(0, &A.lUa[q], cs));
            API_CUDA(c, G.get(0, &A.lUp[q], cs));
            API_CUDA(c, G.get(0, &A.lQ[q], cs));
        }
        API_CUDA(c, G.get(0, &A.pack, 3 * ni));   // one interior array per Helmholtz solve
        API_CUDA(c, G.get(0, &A.work, ADJ_WORK_FIELDS * cs));
        API_CUDA(c, G.get(0, &A.grad, 3 + 2 * ncyl));
    }
    if (K > G.K) {
        G.free_group(1);
        G.K = 0;
        API_CUDA(c, G.get(1, &G.tU, K * cs));
        API_CUDA(c, G.get(1, &G.tV, K * cs));
        API_CUDA(c, G.get(1, &G.tW, K * cs));
        API_CUDA(c, G.get(1, &G.tC, (K + 1) * 6 * cs));
        API_CUDA(c, G.get(1, &G.tCm, K * 6 * cs));
        API_CUDA(c, G.get(1, &G.tcodes, K * ni));
        API_CUDA(c, G.get(1, &G.tcodes_g, K * 2 * (size_t)d.g.nx * d.g.nz));
        API_CUDA(c, G.get(1, &G.tUa, 3 * K * cs));
        API_CUDA(c, G.get(1, &G.tUp, 3 * K * cs));
        API_CUDA(c, G.get(1, &G.tPhi, K * cs));
        API_CUDA(c, G.get(1, &G.tFc, 3 * K * nfc));
        G.K = K;
    }
    if (nck > G.nck) {
        G.free_group(2);
        G.nck = 0;
        G.ck_slot = 11 * cs + 6 * ni;
        API_CUDA(c, G.get(2, &G.ck, nck * G.ck_slot));
        G.nck = nck;
    }
    if (nsteps > G.nsteps) {
        G.free_group(3);
        G.nsteps = 0;
        API_CUDA(c, G.get(3, &G.dw, (size_t)nsteps * std::max<size_t>(ncyl, 1) * 3));
        G.nsteps = nsteps;
    }
    return F8_OK;
}

// state <-> checkpoint slot: U, V, W, P, C (halo) and the AB2 histories
cudaError_t ck_copy(f8_ctx *c, int slot, bool save) {
    Dev &d = c->d;
    GradMem &G = c->gm;
    const size_t cs = d.cs, ni = d.ni;
    double *base = G.ck + (size_t)slot * G.ck_slot;
    // Phi is the SOR variant's start value of the next solve, so a recomputed
    // segment repeats the SOR iterates exactly
    double *f[12] = {d.U, d.V, d.W, d.P, d.C, d.Ax0, d.Ay0, d.Az0, d.Tx0, d.Ty0, d.Tz0, d.Phi};
    const size_t n[12] = {cs, cs, cs, cs, (size_t)d.ncomp * cs, ni, ni, ni, ni, ni, ni, cs};
    size_t off = 0;
    for (int q = 0; q < 12; ++q) {
        const size_t b = n[q] * sizeof(double);
        cudaError_t e = save ? cudaMemcpyAsync(base + off, f[q], b, cudaMemcpyDeviceToDevice, c->s)
                             : cudaMemcpyAsync(f[q], base + off, b, cudaMemcpyDeviceToDevice, c->s);
        if (e != cudaSuccess) return e;
        off += n[q];
    }
    return cudaSuccess;
}

// one forward step of f8_grad (absolute step index s of the call); rec >= 0
// stores the tape of the step in segment slot rec
cudaError_t grad_forward_step(f8_ctx *c, int step0, int s, int rec) {
    Dev &d = c->d;
    GradMem &G = c->gm;
    const size_t cs = d.cs, ni = d.ni, nfc = (size_t)d.nm * d.g.nz, hb = cs * sizeof(double);
    const int ncyl = (int)c->cyl.size();
    StepOpts o{};
    o.polymer = c->phys.beta != 1.0;
    o.ab2_first = (step0 + s + 1 == 1) && c->phys.ab2_start;
    o.ibm = ncyl > 0;
    o.poisson = c->poisson;
    o.sor_omega = c->phys.sor_omega; o.sor_eps = c->phys.sor_eps; o.sor_itrmax = c->phys.sor_itrmax;
    if (!o.polymer) F8_CUDA_RET(cudaMemsetAsync(d.C, 0, d.ncomp * hb, c->s));
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c->s);
    };
    if (rec >= 0) {
        F8_CUDA_RET(cp(G.tU + rec * cs, d.U, hb));
        F8_CUDA_RET(cp(G.tV + rec * cs, d.V, hb));
        F8_CUDA_RET(cp(G.tW + rec * cs, d.W, hb));
        if (rec == 0) F8_CUDA_RET(cp(G.tC, d.C, d.ncomp * hb));
    }
    int sor = -1;
    if (rec >= 0) o.c_mid = G.tCm + (size_t)rec * 6 * cs;
    F8_CUDA_RET(step_fp64(d, o, ncyl ? c->drag_dev + (size_t)s * ncyl * 3 : nullptr, &sor, c->s));
    if (c->poisson == F8_POISSON_SOR && sor > c->phys.sor_itrmax) ++G.sor_capped;
    if (rec >= 0) {
        const size_t ng = 2 * (size_t)d.g.nx * d.g.nz;
        F8_CUDA_RET(cp(G.tC + (size_t)(rec + 1) * 6 * cs, d.C, d.ncomp * hb));
        F8_CUDA_RET(cp(G.tcodes + rec * ni, d.codes, ni));
        F8_CUDA_RET(cp(G.tcodes_g + rec * ng, d.codes_g, ng));
        const double *ua[3] = {d.Ua, d.Va, d.Wa}, *up[3] = {d.Up, d.Vp, d.Wp};
        for (int q = 0; q < 3; ++q) {
            F8_CUDA_RET(cp(G.tUa + (3 * rec + q) * cs, ua[q], hb));
            F8_CUDA_RET(cp(G.tUp + (3 * rec + q) * cs, up[q], hb));
            if (nfc) F8_CUDA_RET(cp(G.tFc + (3 * rec + q) * nfc, d.Fc[q], nfc * sizeof(double)));
        }
        F8_CUDA_RET(cp(G.tPhi + rec * cs, d.Phi, hb));
    }
    return cudaSuccess;
}

// ---- FP32-mixed contexts --------------------------------------------------

constexpr int MIXED_TAPE_FIELDS = 22;   // U V W, C (6), Cn (6), Ua (3), Up (3), Phi

int grad_alloc_mixed(f8_ctx *c, int K, int nck, int nsteps) {
    GradMem &G = c->gm;
    Dev &d = c->d;
    const size_t cs = d.cs, ni = d.ni, ncyl = c->cyl.size(), nfc = (size_t)d.nm * d.g.nz;
    if (!G.AF.grad) {
        AdjStateF &A = G.AF;
        for (float **p : {&A.lU, &A.lV, &A.lW, &A.lP, &A.lPhi}) API_CUDA(c, G.get(0, p, cs));
        for (float **p : {&A.lC, &A.lC2}) API_CUDA(c, G.get(0, p, 6 * cs));
        for (int q = 0; q < 3; ++q) {
            API_CUDA(c, G.get(0, &A.lA0[q], ni));
            API_CUDA(c, G.get(0, &A.lT0[q], ni));
            API_CUDA(c, G.get(0, &A.lUa[q], cs));
            API_CUDA(c, G.get(0, &A.lUp[q], cs));
            API_CUDA(c, G.get(0, &A.lQ[q], cs));
        }
        API_CUDA(c, G.get(0, &A.pack, 3 * ni));   // one interior array per Helmholtz solve
        API_CUDA(c, G.get(0, &A.qlo, cs));
        API_CUDA(c, G.get(0, &A.zero, ni));
        API_CUDA(c, G.get(0, &A.rdef, ni));
        API_CUDA(c, G.get(0, &A.work, ADJ_WORK_FIELDS * cs));
        API_CUDA(c, cudaMemsetAsync(A.zero, 0, ni * sizeof(float), c->s));
        API_CUDA(c, G.get(0, &A.grad, 3 + 2 * ncyl));
        API_CUDA(c, G.get(0, &G.dw_slot, 3 * std::max<size_t>(ncyl, 1)));
        G.lc_base = A.lC;
    }
    if (K > G.K) {
        G.drop_graphs();   // they hold tape addresses
        G.free_group(1);
        G.K = 0;
        API_CUDA(c, G.get(1, &G.ftape, (size_t)K * MIXED_TAPE_FIELDS * cs));
        API_CUDA(c, G.get(1, &G.fcodes, K * ni));
        API_CUDA(c, G.get(1, &G.fcodes_g, K * 2 * (size_t)d.g.nx * d.g.nz));
        API_CUDA(c, G.get(1, &G.fFc, 3 * K * std::max<size_t>(nfc, 1)));
        G.K = K;
    }
    if (nck > G.nck) {
        G.free_group(2);
        G.nck = 0;
        G.fck_slot = 15 * cs + 6 * ni;
        API_CUDA(c, G.get(2, &G.fck, nck * G.fck_slot));
        G.nck = nck;
    }
    if (nsteps > G.nsteps) {
        G.free_group(3);
        G.nsteps = 0;
        API_CUDA(c, G.get(3, &G.dw, (size_t)nsteps * std::max<size_t>(ncyl, 1) * 3));
        G.nsteps = nsteps;
    }
    return F8_OK;
}

// mixed state <-> checkpoint slot: the double-float velocity and pressure,
// C and f(C) (halo), the AB2 histories
cudaError_t ck_copy_mixed(f8_ctx *c, int slot, bool save) {
    Dev &d = c->d;
    GradMem &G = c->gm;
    const size_t cs = d.cs, ni = d.ni;
    float *base = G.fck + (size_t)slot * G.fck_slot;
    float *f[16] = {d.Uf, d.Ul, d.Vf, d.Vl, d.Wf, d.Wl, d.Pf, d.Pl, d.Cf, d.fpetf,
                    d.A0f[0], d.A0f[1], d.A0f[2], d.T0f[0], d.T0f[1], d.T0f[2]};
    const size_t n[16] = {cs, cs, cs, cs, cs, cs, cs, cs, 6 * cs, cs, ni, ni, ni, ni, ni, ni};
    size_t off = 0;
    for (int q = 0; q < 16; ++q) {
        const size_t b = n[q] * sizeof(float);
        cudaError_t e = save ? cudaMemcpyAsync(base + off, f[q], b, cudaMemcpyDeviceToDevice, c->s)
                             : cudaMemcpyAsync(f[q], base + off, b, cudaMemcpyDeviceToDevice, c->s);
        if (e != cudaSuccess) return e;
        off += n[q];
    }
    return cudaSuccess;
}

MixTape tape_slot_mixed(f8_ctx *c, int rec) {
    GradMem &G = c->gm;
    const size_t cs = c->d.cs, ni = c->d.ni, nfc = std::max<size_t>((size_t)c->d.nm * c->d.g.nz, 1);
    float *b = G.ftape + (size_t)rec * MIXED_TAPE_FIELDS * cs;
    MixTape t{};
    t.U = b; t.V = b + cs; t.W = b + 2 * cs;
    t.C = b + 3 * cs; t.Cn = b + 9 * cs;
    for (int q = 0; q < 3; ++q) {
        t.Ua[q] = b + (15 + q) * cs;
        t.Up[q] = b + (18 + q) * cs;
        t.Fc[q] = G.fFc + (3 * (size_t)rec + q) * nfc;
    }
    t.Phi = b + 21 * cs;
    t.codes = G.fcodes + rec * ni;
    t.codes_g = G.fcodes_g + rec * 2 * (size_t)c->d.g.nx * c->d.g.nz;
    return t;
}

// Launch graph ge on the context's stream, capturing it first from record()
// (which enqueues the work and undoes any host-side buffer swap it makes:
// the capture runs nothing).  nl: kernels per replay.
template <typename F>
cudaError_t replay_graph(f8_ctx *c, cudaGraphExec_t &ge, long long &nl, F &&record) {
    if (!ge) {
        const long long l0 = g_kernel_launches.load();
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        e = record();
        const cudaError_t e2 = cudaStreamEndCapture(c->s, &gr);
        nl = g_kernel_launches.load() - l0;
        g_kernel_launches -= nl;
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, gr, 0);
        if (gr) cudaGraphDestroy(gr);
        if (e != cudaSuccess) {
            ge = nullptr;
            return e;
        }
    }
    g_kernel_launches += nl;
    return cudaGraphLaunch(ge, c->s);
}

// one forward step of f8_grad on a mixed context (absolute step index s of
// the call); rec >= 0 writes the tape of the step into segment slot rec.
// Replayed from a CUDA graph (the step's own without a tape, one per tape
// slot and C parity with one) except for the AB2 start step.
cudaError_t grad_forward_step_mixed(f8_ctx *c, int step0, int s, int rec) {
    Dev &d = c->d;
    GradMem &G = c->gm;
    const int ncyl = (int)c->cyl.size();
    StepOpts o{};
    o.polymer = c->phys.beta != 1.0;
    o.ab2_first = (step0 + s + 1 == 1) && c->phys.ab2_start;
    o.ibm = ncyl > 0;
    o.poisson = F8_POISSON_FFT;
    if (!o.polymer) F8_CUDA_RET(cudaMemsetAsync(d.Cf, 0, (size_t)d.cs * d.ncomp * sizeof(float), c->s));
    MixTape t{};
    if (rec >= 0) {
        t = tape_slot_mixed(c, rec);
        o.tape = &t;
    }
    int sor = -1;
    double *dg = ncyl ? c->drag_dev + (size_t)s * ncyl * 3 : nullptr;
    if (o.ab2_first) return step_mixed(d, o, dg, &sor, c->s);
    const int p = d.Cf == c->cf_base ? 0 : 1;
    if (rec >= 0 && G.gfwd.size() < 2 * (size_t)G.K) G.gfwd.resize(2 * (size_t)G.K, nullptr);
    cudaGraphExec_t &ge = rec < 0 ? c->gexec[p] : G.gfwd[2 * rec + p];
    long long &nl = rec < 0 ? c->graph_launches : G.gfwd_launches;
    F8_CUDA_RET(replay_graph(c, ge, nl, [&] {
        float *cf0 = d.Cf, *cn0 = d.Cnf;
        const cudaError_t e = step_mixed(d, o, ncyl ? c->drag_slot : nullptr, &sor, c->s);
        d.Cf = cf0;
        d.Cnf = cn0;
        return e;
    }));
    if (o.polymer) std::swap(d.Cf, d.Cnf);
    if (dg) F8_CUDA_RET(cudaMemcpyAsync(dg, c->drag_slot, (size_t)ncyl * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    return cudaSuccess;
}

// Segments (the last R >= 1) whose tape the first forward pass keeps, so
// that the reverse sweep recomputes only the nseg - R before them: as many as
// fit, together with the checkpoints those others need, in the memory the
// gradient's tape and checkpoints already hold plus 60 % of the device's free
// memory.  F8_GRAD_KEEP_TAPE=0 in the environment keeps the last segment only.
int kept_segments_mixed(f8_ctx *c, int K, int nseg) {
    const char *env = std::getenv("F8_GRAD_KEEP_TAPE");
    if (env && env[0] == '0') return 1;
    const GradMem &G = c->gm;
    const Dev &d = c->d;
    const double cs = (double)d.cs, ni = (double)d.ni;
    const double nfc = std::max(1.0, (double)d.nm * d.g.nz);
    const double slot = MIXED_TAPE_FIELDS * cs * 4 + ni + 2.0 * d.g.nx * d.g.nz + 3 * nfc * 8;
    const double ck = (15 * cs + 6 * ni) * 4;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return 1;
    return kept_segments(G.K * slot + G.nck * ck + 0.6 * (double)fr, slot, ck, K, nseg);
}

// f8_grad on an FP32-mixed 3D context with the FFT solvers: the same
// checkpointed schedule as the FP64 gradient, with the mixed forward step
// (its tape written by the step itself) and the FP32 adjoint step.  The
// first forward pass keeps the tape of the last R segments (slots
// (seg - (nseg - R)) K ..); the segments before them are recomputed from
// their checkpoints into slots 0 .. K-1, whose first owner has been swept
// by then.
int grad_mixed(f8_ctx *c, int nsteps, int checkpoint_every, const double *drag_w, const f8_fields *seed, double *J,
               double *dJ_dparams, f8_fields *dJ_dstate, double *drag) {
    Dev &d = c->d;
    const int ncyl = (int)c->cyl.size();
    const size_t cs = d.cs, ni = d.ni;
    const int K = checkpoint_every == 0 ? nsteps : std::min(checkpoint_every, nsteps);
    const int nseg = (nsteps + K - 1) / K;
    const int R = kept_segments_mixed(c, K, nseg);
    const int nrec = nseg - R;                       // segments recomputed from a checkpoint
    if (int st = grad_alloc_mixed(c, R * K, nrec > 0 ? nrec + 1 : 0, nsteps)) return st;
    c->grad_kept_segments = R;
    if (int st = ensure_drag(c, nsteps)) return st;
    GradMem &G = c->gm;
    AdjStateF &A = G.AF;
    const size_t nw = (size_t)nsteps * ncyl * 3;
    std::vector<double> w(nw, 0.0);
    if (drag_w) std::copy(drag_w, drag_w + nw, w.begin());
    else
        for (int n = 0; n < nsteps; ++n)
            for (int l = 0; l < ncyl; ++l) w[((size_t)n * ncyl + l) * 3] = 1.0 / nsteps;
    if (nw) API_CUDA(c, cudaMemcpyAsync(G.dw, w.data(), nw * sizeof(double), cudaMemcpyHostToDevice, c->s));
    // the mixed step's counters are cumulative since the load; report this
    // call's share
    StepCounters cnt0{};
    API_CUDA(c, cudaMemcpyAsync(&cnt0, d.cnt, sizeof(cnt0), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    const int step0 = c->step;
    // forward: checkpoints at the starts of the segments to recompute, the
    // tape of the kept ones
    for (int seg = 0; seg < nseg; ++seg) {
        const int s0 = seg * K, s1 = std::min(nsteps, s0 + K);
        const bool kept = seg >= nrec;
        if (!kept) API_CUDA(c, ck_copy_mixed(c, seg, true));
        for (int s = s0; s < s1; ++s)
            API_CUDA(c, grad_forward_step_mixed(c, step0, s, kept ? (seg - nrec) * K + s - s0 : -1));
    }
    if (nrec > 0) API_CUDA(c, ck_copy_mixed(c, nrec, true));   // final state
    // adjoint of the final state
    for (float *p : {A.lU, A.lV, A.lW, A.lP}) API_CUDA(c, cudaMemsetAsync(p, 0, cs * sizeof(float), c->s));
    API_CUDA(c, cudaMemsetAsync(A.lC, 0, 6 * cs * sizeof(float), c->s));
    for (int q = 0; q < 3; ++q) {
        API_CUDA(c, cudaMemsetAsync(A.lA0[q], 0, ni * sizeof(float), c->s));
        API_CUDA(c, cudaMemsetAsync(A.lT0[q], 0, ni * sizeof(float), c->s));
    }
    API_CUDA(c, cudaMemsetAsync(A.grad, 0, (3 + 2 * ncyl) * sizeof(double), c->s));
    if (seed) {
        // host FP64 -> device FP64 staging (the load buffers) -> FP32 interior
        double *tmp = c->scratch_aos;   // 6 * cs doubles
        const double *hs[4] = {seed->u, seed->v, seed->w, seed->p};
        float *hd[4] = {A.lU, A.lV, A.lW, A.lP};
        for (int q = 0; q < 4; ++q) {
            if (!hs[q]) continue;
            API_CUDA(c, cudaMemcpyAsync(tmp, hs[q], cs * sizeof(double), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, d2f(tmp, A.lC2, (int)cs, c->s));
            API_CUDA(c, take_interior_f(A.lC2, hd[q], d.g, (int)cs, c->s));
        }
        if (seed->c) {
            API_CUDA(c, cudaMemcpyAsync(tmp, seed->c, 6 * cs * sizeof(double), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, aos_to_soa_f(tmp, A.lC2, 6, (int)cs, c->s));
            API_CUDA(c, take_interior_f(A.lC2, A.lC, d.g, (int)(6 * cs), c->s));
        }
        const double *is[6] = {seed->ax0, seed->ay0, seed->az0, seed->tx0, seed->ty0, seed->tz0};
        float *id[6] = {A.lA0[0], A.lA0[1], A.lA0[2], A.lT0[0], A.lT0[1], A.lT0[2]};
        for (int q = 0; q < 6; ++q) {
            if (!is[q]) continue;
            API_CUDA(c, cudaMemcpyAsync(tmp, is[q], ni * sizeof(double), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, d2f(tmp, id[q], (int)ni, c->s));
        }
        API_CUDA(c, cudaStreamSynchronize(c->s));
    }
    // reverse sweep over the segments
    const bool polymer = c->phys.beta != 1.0;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int s0 = seg * K, s1 = std::min(nsteps, s0 + K);
        const int base = seg >= nrec ? (seg - nrec) * K : 0;
        if (seg < nrec) {
            API_CUDA(c, ck_copy_mixed(c, seg, false));
            for (int s = s0; s < s1; ++s) API_CUDA(c, grad_forward_step_mixed(c, step0, s, s - s0));
        }
        for (int s = s1 - 1; s >= s0; --s) {
            const int rec = base + s - s0;
            const MixTape t = tape_slot_mixed(c, rec);
            const bool ab2_first = (step0 + s + 1 == 1) && c->phys.ab2_start;
            if (ab2_first) {
                API_CUDA(c, step_mixed_adjoint(d, A, t, G.dw + (size_t)s * ncyl * 3, true, polymer, c->s));
                continue;
            }
            // replayed from the graph of tape slot rec and adjoint C parity,
            // reading this step's drag weights from a fixed slot
            if (ncyl)
                API_CUDA(c, cudaMemcpyAsync(G.dw_slot, G.dw + (size_t)s * ncyl * 3, (size_t)ncyl * 3 * sizeof(double),
                                            cudaMemcpyDeviceToDevice, c->s));
            if (G.grev.size() < 2 * (size_t)G.K) G.grev.resize(2 * (size_t)G.K, nullptr);
            const int p = A.lC == G.lc_base ? 0 : 1;
            API_CUDA(c, replay_graph(c, G.grev[2 * rec + p], G.grev_launches, [&] {
                float *l0 = A.lC, *l1 = A.lC2;
                const cudaError_t e = step_mixed_adjoint(d, A, t, G.dw_slot, false, polymer, c->s);
                A.lC = l0;
                A.lC2 = l1;
                return e;
            }));
            if (polymer) std::swap(A.lC, A.lC2);
        }
    }
    if (nrec > 0) API_CUDA(c, ck_copy_mixed(c, nrec, false));
    c->step = step0 + nsteps;
    // results
    std::vector<double> hd((size_t)std::max<size_t>(nw, 1));
    if (nw) API_CUDA(c, cudaMemcpyAsync(hd.data(), c->drag_dev, nw * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    std::vector<double> gr(3 + 2 * ncyl);
    API_CUDA(c, cudaMemcpyAsync(gr.data(), A.grad, gr.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    StepCounters cnt{};
    API_CUDA(c, cudaMemcpyAsync(&cnt, d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, c->s));
    if (dJ_dstate) {
        auto get = [&](double *dst, const float *src, size_t n) -> cudaError_t {
            if (!dst) return cudaSuccess;
            cudaError_t e = f2d(src, c->scratch_aos, (int)n, c->s);
            if (e != cudaSuccess) return e;
            e = cudaMemcpyAsync(dst, c->scratch_aos, n * sizeof(double), cudaMemcpyDeviceToHost, c->s);
            if (e != cudaSuccess) return e;
            return cudaStreamSynchronize(c->s);   // the staging buffer is reused
        };
        API_CUDA(c, get(dJ_dstate->u, A.lU, cs));
        API_CUDA(c, get(dJ_dstate->v, A.lV, cs));
        API_CUDA(c, get(dJ_dstate->w, A.lW, cs));
        API_CUDA(c, get(dJ_dstate->p, A.lP, cs));
        if (dJ_dstate->c) {
            API_CUDA(c, soa_to_aos_f(A.lC, c->scratch_aos, 6, (int)cs, c->s));
            API_CUDA(c, cudaMemcpyAsync(dJ_dstate->c, c->scratch_aos, 6 * cs * sizeof(double), cudaMemcpyDeviceToHost,
                                        c->s));
            API_CUDA(c, cudaStreamSynchronize(c->s));
        }
        double *od[6] = {dJ_dstate->ax0, dJ_dstate->ay0, dJ_dstate->az0, dJ_dstate->tx0, dJ_dstate->ty0, dJ_dstate->tz0};
        const float *os[6] = {A.lA0[0], A.lA0[1], A.lA0[2], A.lT0[0], A.lT0[1], A.lT0[2]};
        for (int q = 0; q < 6; ++q) API_CUDA(c, get(od[q], os[q], ni));
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    if (dJ_dstate) {
        if (dJ_dstate->phi) std::fill(dJ_dstate->phi, dJ_dstate->phi + cs, 0.0);
        for (double *p : {dJ_dstate->fx, dJ_dstate->fy, dJ_dstate->fz})
            if (p) std::fill(p, p + ni, 0.0);
    }
    if (J) {
        double sum = 0.0;
        for (size_t q = 0; q < nw; ++q) sum += w[q] * hd[q];
        *J = sum;
    }
    if (drag && nw) std::copy(hd.begin(), hd.begin() + nw, drag);
    if (dJ_dparams) std::copy(gr.begin(), gr.end(), dJ_dparams);
    const StepCounters dc{cnt.newton_iters - cnt0.newton_iters, cnt.newton_unconverged - cnt0.newton_unconverged,
                          cnt.nan_cells - cnt0.nan_cells, cnt.copy_timeouts - cnt0.copy_timeouts};
    c->cnt_prev = cnt;
    c->last_newton_iters = (long long)dc.newton_iters;
    c->last_newton_unconv = (long long)dc.newton_unconverged;
    if (dc.copy_timeouts) {
        c->last_error = "a bulk-copy wait of the projection kernel ran out; the step is incomplete";
        return F8_ERR_CUDA;
    }
    if (dc.nan_cells) return F8_ERR_NAN;
    if (dc.newton_unconverged) return F8_WARN_NEWTON;
    return F8_OK;
}

TapeStep tape_step(f8_ctx *c, int rec) {
    GradMem &G = c->gm;
    const size_t cs = c->d.cs, ni = c->d.ni, nfc = (size_t)c->d.nm * c->d.g.nz;
    TapeStep t{};
    t.U = G.tU + rec * cs; t.V = G.tV + rec * cs; t.W = G.tW + rec * cs;
    t.C = G.tC + (size_t)rec * 6 * cs; t.Cn = G.tCm + (size_t)rec * 6 * cs;
    t.codes = G.tcodes + rec * ni;
    t.codes_g = G.tcodes_g + rec * 2 * (size_t)c->d.g.nx * c->d.g.nz;
    for (int q = 0; q < 3; ++q) {
        t.Ua[q] = G.tUa + (3 * rec + q) * cs;
        t.Up[q] = G.tUp + (3 * rec + q) * cs;
        t.Fc[q] = G.tFc + (3 * rec + q) * nfc;
    }
    t.Phi = G.tPhi + rec * cs;
    return t;
}

}  // namespace

extern "C" {

static int grad_impl(f8_ctx *c, int nsteps, int checkpoint_every, const double *drag_w, const f8_fields *seed,
                     double *J, double *dJ_dparams, f8_fields *dJ_dstate, double *drag) {
    if (!c || nsteps < 1 || checkpoint_every < 0) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    if (c->phys.ibm_repeats != 1) return F8_ERR_UNSUPPORTED;
    if (c->precision == F8_MIXED) {
        if (c->grid.dim != 3) return F8_ERR_UNSUPPORTED;
        if (c->poisson != F8_POISSON_FFT) return F8_ERR_UNSUPPORTED;
        return grad_mixed(c, nsteps, checkpoint_every, drag_w, seed, J, dJ_dparams, dJ_dstate, drag);
    }
    Dev &d = c->d;
    const int ncyl = (int)c->cyl.size();
    const size_t cs = d.cs, ni = d.ni;
    const int K = checkpoint_every == 0 ? nsteps : std::min(checkpoint_every, nsteps);
    const int nseg = (nsteps + K - 1) / K;
    if (int st = grad_alloc(c, K, nseg, nsteps)) return st;
    if (int st = ensure_drag(c, nsteps)) return st;
    GradMem &G = c->gm;
    AdjState &A = G.A;
    const size_t nw = (size_t)nsteps * ncyl * 3;
    std::vector<double> w(nw, 0.0);
    if (drag_w) std::copy(drag_w, drag_w + nw, w.begin());
    else
        for (int n = 0; n < nsteps; ++n)
            for (int l = 0; l < ncyl; ++l) w[((size_t)n * ncyl + l) * 3] = 1.0 / nsteps;
    if (nw) API_CUDA(c, cudaMemcpyAsync(G.dw, w.data(), nw * sizeof(double), cudaMemcpyHostToDevice, c->s));
    API_CUDA(c, cudaMemsetAsync(d.cnt, 0, sizeof(StepCounters), c->s));
    c->cnt_prev = StepCounters{};   // f8_step reports differences from this
    API_CUDA(c, cudaMemsetAsync(c->nan_dev, 0, sizeof(unsigned long long), c->s));
    G.sor_capped = 0;
    const int step0 = c->step;
    // forward: checkpoints at the segment starts, the tape of the last segment
    for (int seg = 0; seg < nseg; ++seg) {
        const int s0 = seg * K, s1 = std::min(nsteps, s0 + K);
        const bool last = seg == nseg - 1;
        if (!last) API_CUDA(c, ck_copy(c, seg, true));
        for (int s = s0; s < s1; ++s) API_CUDA(c, grad_forward_step(c, step0, s, last ? s - s0 : -1));
    }
    API_CUDA(c, count_nonfinite(d.U, d.cs, c->nan_dev, c->s));
    if (nseg > 1) API_CUDA(c, ck_copy(c, nseg - 1, true));   // final state
    // adjoint of the final state
    for (double *p : {A.lU, A.lV, A.lW, A.lP}) API_CUDA(c, cudaMemsetAsync(p, 0, cs * sizeof(double), c->s));
    API_CUDA(c, cudaMemsetAsync(A.lC, 0, 6 * cs * sizeof(double), c->s));
    for (int q = 0; q < 3; ++q) {
        API_CUDA(c, cudaMemsetAsync(A.lA0[q], 0, ni * sizeof(double), c->s));
        API_CUDA(c, cudaMemsetAsync(A.lT0[q], 0, ni * sizeof(double), c->s));
    }
    API_CUDA(c, cudaMemsetAsync(A.grad, 0, (3 + 2 * ncyl) * sizeof(double), c->s));
    if (seed) {
        double *tmp = c->scratch_aos;   // 6 * cs doubles
        const double *hs[4] = {seed->u, seed->v, seed->w, seed->p};
        double *hd[4] = {A.lU, A.lV, A.lW, A.lP};
        for (int q = 0; q < 4; ++q) {
            if (!hs[q]) continue;
            API_CUDA(c, cudaMemcpyAsync(tmp, hs[q], cs * sizeof(double), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, take_interior(tmp, hd[q], d.g, (int)cs, c->s));
        }
        if (seed->c) {
            API_CUDA(c, cudaMemcpyAsync(tmp, seed->c, d.ncomp * cs * sizeof(double), cudaMemcpyHostToDevice, c->s));
            API_CUDA(c, aos_to_soa(tmp, A.lC2, d.ncomp, (int)cs, c->s));
            API_CUDA(c, take_interior(A.lC2, A.lC, d.g, (int)(d.ncomp * cs), c->s));
        }
        const double *is[6] = {seed->ax0, seed->ay0, seed->az0, seed->tx0, seed->ty0, seed->tz0};
        double *id[6] = {A.lA0[0], A.lA0[1], A.lA0[2], A.lT0[0], A.lT0[1], A.lT0[2]};
        for (int q = 0; q < 6; ++q)
            if (is[q]) API_CUDA(c, cudaMemcpyAsync(id[q], is[q], ni * sizeof(double), cudaMemcpyHostToDevice, c->s));
        API_CUDA(c, cudaStreamSynchronize(c->s));
    }
    // the SOR variant's adjoint pressure solves, warm started from zero
    A.sor = c->poisson == F8_POISSON_SOR;
    A.sor_omega = c->phys.sor_omega; A.sor_eps = c->phys.sor_eps; A.sor_itrmax = c->phys.sor_itrmax;
    A.sor_capped = 0;
    if (A.sor) {
        if (!A.lsor) API_CUDA(c, G.get(0, &A.lsor, cs));
        API_CUDA(c, cudaMemsetAsync(A.lsor, 0, cs * sizeof(double), c->s));
    }
    // reverse sweep over the segments
    const bool polymer = c->phys.beta != 1.0;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int s0 = seg * K, s1 = std::min(nsteps, s0 + K);
        if (seg != nseg - 1) {
            API_CUDA(c, ck_copy(c, seg, false));
            for (int s = s0; s < s1; ++s) API_CUDA(c, grad_forward_step(c, step0, s, s - s0));
        }
        for (int s = s1 - 1; s >= s0; --s) {
            const TapeStep t = tape_step(c, s - s0);
            const bool ab2_first = (step0 + s + 1 == 1) && c->phys.ab2_start;
            if (d.g.dim == 3) API_CUDA(c, step_fp64_adjoint(d, A, t, G.dw + (size_t)s * ncyl * 3, ab2_first, polymer, c->s));
            else API_CUDA(c, step_fp64_adjoint2(d, A, t, G.dw + (size_t)s * ncyl * 3, ab2_first, polymer, c->s));
        }
    }
    if (nseg > 1) API_CUDA(c, ck_copy(c, nseg - 1, false));
    c->step = step0 + nsteps;
    // results
    std::vector<double> hd((size_t)std::max<size_t>(nw, 1));
    if (nw) API_CUDA(c, cudaMemcpyAsync(hd.data(), c->drag_dev, nw * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    std::vector<double> gr(3 + 2 * ncyl);
    API_CUDA(c, cudaMemcpyAsync(gr.data(), A.grad, gr.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    StepCounters cnt{};
    unsigned long long nan = 0;
    API_CUDA(c, cudaMemcpyAsync(&cnt, d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaMemcpyAsync(&nan, c->nan_dev, sizeof(nan), cudaMemcpyDeviceToHost, c->s));
    if (dJ_dstate) {
        auto get = [&](double *dst, const double *src, size_t n) -> cudaError_t {
            if (!dst) return cudaSuccess;
            return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->s);
        };
        API_CUDA(c, get(dJ_dstate->u, A.lU, cs));
        API_CUDA(c, get(dJ_dstate->v, A.lV, cs));
        API_CUDA(c, get(dJ_dstate->w, A.lW, cs));
        API_CUDA(c, get(dJ_dstate->p, A.lP, cs));
        if (dJ_dstate->c) {
            API_CUDA(c, soa_to_aos(A.lC, c->scratch_aos, d.ncomp, (int)cs, c->s));
            API_CUDA(c, get(dJ_dstate->c, c->scratch_aos, d.ncomp * cs));
        }
        double *od[6] = {dJ_dstate->ax0, dJ_dstate->ay0, dJ_dstate->az0, dJ_dstate->tx0, dJ_dstate->ty0, dJ_dstate->tz0};
        const double *os[6] = {A.lA0[0], A.lA0[1], A.lA0[2], A.lT0[0], A.lT0[1], A.lT0[2]};
        for (int q = 0; q < 6; ++q) API_CUDA(c, get(od[q], os[q], ni));
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    if (dJ_dstate) {
        if (dJ_dstate->phi) std::fill(dJ_dstate->phi, dJ_dstate->phi + cs, 0.0);
        for (double *p : {dJ_dstate->fx, dJ_dstate->fy, dJ_dstate->fz})
            if (p) std::fill(p, p + ni, 0.0);
    }
    if (J) {
        double sum = 0.0;
        for (size_t q = 0; q < nw; ++q) sum += w[q] * hd[q];
        *J = sum;
    }
    if (drag && nw) std::copy(hd.begin(), hd.begin() + nw, drag);
    if (dJ_dparams) std::copy(gr.begin(), gr.end(), dJ_dparams);
    c->cnt_prev = cnt;
    c->last_newton_iters = (long long)cnt.newton_iters;
    c->last_newton_unconv = (long long)cnt.newton_unconverged;
    if (nan) return F8_ERR_NAN;
    if (cnt.newton_unconverged) return F8_WARN_NEWTON;
    if (G.sor_capped || A.sor_capped) return F8_WARN_SOR;
    return F8_OK;
}

int f8_grad(f8_ctx *c, int nsteps, int checkpoint_every, const double *drag_w, const f8_fields *seed, double *J,
            double *dJ_dparams, f8_fields *dJ_dstate, double *drag) {
    if (!c || !c->zwalls) return grad_impl(c, nsteps, checkpoint_every, drag_w, seed, J, dJ_dparams, dJ_dstate, drag);
    f8_fields si{}, so{};
    if (seed) zwall_in(c, seed, &si, c->zbuf);
    if (dJ_dstate) zwall_stage(c, dJ_dstate, &so, c->zbuf2);
    const int st = grad_impl(c, nsteps, checkpoint_every, drag_w, seed ? &si : nullptr, J, dJ_dparams,
                             dJ_dstate ? &so : nullptr, drag);
    if (dJ_dstate && (st == F8_OK || st >= 16)) zwall_out(c, &so, dJ_dstate);
    return st;
}

int f8_diagnostics(f8_ctx *c, f8_diag *dg) {
    if (!c || !dg) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    std::memset(dg, 0, sizeof(*dg));
    DiagValues v{};
    API_CUDA(c, device_diagnostics(c->d, c->precision == F8_MIXED, c->diag_part, c->d.scal, &v, c->s));
    dg->step = c->step;
    dg->ke = v.ke;
    dg->cfl = v.cfl;
    dg->trc_min = v.trc_min; dg->trc_max = v.trc_max; dg->trc_mean = v.trc_mean; dg->trc_std = v.trc_std;
    dg->div_max = v.div_max;
    dg->nan_found = v.nan_found;
    dg->newton_iters = c->last_newton_iters;
    dg->newton_unconverged = c->last_newton_unconv;
    dg->poisson_iters = c->last_poisson_iters;
    dg->kernel_launches = c->step_launches;
    return F8_OK;
}

int f8_slice(f8_ctx *c, int axis, int variant, double *out) {
    if (c && c->zwalls) return F8_ERR_UNSUPPORTED;   // the exchanged axes are not mapped back here
    if (!c || !out || axis < 0 || axis > 2 || variant < 0 || variant > 1) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    if (c->grid.dim != 3) return F8_ERR_UNSUPPORTED;
    const int n = slice_points(c->d.g, axis);
    API_CUDA(c, device_slice(c->d, c->precision == F8_MIXED, axis, variant, c->slice_dev, c->s));
    API_CUDA(c, cudaMemcpyAsync(out, c->slice_dev, (size_t)n * 18 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

namespace {
// upload the optional mean fields; mean[] gets device pointers or nulls
int upload_means(f8_ctx *c, const double *mu, const double *mv, const double *mw, const double *mean[3]) {
    const size_t ni = c->d.ni;
    const double *src[3] = {mu, mv, mw};
    for (int q = 0; q < 3; ++q) mean[q] = nullptr;
    if (!mu && !mv && !mw) return F8_OK;
    if (!c->mean_dev) API_CUDA(c, c->alloc(&c->mean_dev, 3 * ni));
    for (int q = 0; q < 3; ++q) {
        if (!src[q]) continue;
        API_CUDA(c, cudaMemcpyAsync(c->mean_dev + q * ni, src[q], ni * sizeof(double), cudaMemcpyHostToDevice, c->s));
        mean[q] = c->mean_dev + q * ni;
    }
    return F8_OK;
}
}  // namespace

int f8_turbulence(f8_ctx *c, const double *mu, const double *mv, const double *mw, f8_turb *out) {
    if (c && c->zwalls) return F8_ERR_UNSUPPORTED;   // the exchanged axes are not mapped back here
    if (!c || !out) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    if (c->grid.dim != 3) return F8_ERR_UNSUPPORTED;
    const double *mean[3];
    if (int st = upload_means(c, mu, mv, mw, mean)) return st;
    const bool mixed = c->precision == F8_MIXED;
    TurbValues t{};
    API_CUDA(c, device_turbulence(c->d, mixed, mean, c->diag_part, c->d.scal, &t, c->s));
    DiagValues v{};
    API_CUDA(c, device_diagnostics(c->d, mixed, c->diag_part, c->d.scal, &v, c->s));
    std::memset(out, 0, sizeof(*out));
    out->k_energy = t.k_energy; out->k_staggered = t.k_staggered;
    out->lambda = t.lambda; out->re_lambda = t.re_lambda; out->epsilon = t.epsilon;
    out->l_kolmogorov = t.l_kolmogorov; out->t_kolmogorov = t.t_kolmogorov; out->u_kolmogorov = t.u_kolmogorov;
    out->ep_energy = t.ep_energy; out->trc_mean = v.trc_mean; out->trc_std = v.trc_std;
    return F8_OK;
}

int f8_spectrum(f8_ctx *c, const double *mu, const double *mv, const double *mw, double *energy) {
    if (c && c->zwalls) return F8_ERR_UNSUPPORTED;   // the exchanged axes are not mapped back here
    if (!c || !energy) return F8_ERR_ARG;
    if (!c->loaded) return F8_ERR_STATE;
    if (c->grid.dim != 3) return F8_ERR_UNSUPPORTED;
    const Geo &g = c->d.g;
    const double *mean[3];
    if (int st = upload_means(c, mu, mv, mw, mean)) return st;
    SpecWork &w = c->spec;
    if (!w.pack) {
        API_CUDA(c, spectrum_kernel_attrs());
        API_CUDA(c, c->alloc(&w.pack, (size_t)c->d.ni));
        API_CUDA(c, c->alloc(&w.H, 2 * (size_t)(g.nx / 2 + 1) * g.ny * g.nz));
        API_CUDA(c, c->alloc(&w.hist, turb_partials(g.nx)));
        API_CUDA(c, c->alloc(&c->energy_dev, (size_t)g.nx + 1));
        std::vector<double> tr, ti;
        const int nn[3] = {g.nx, g.ny, g.nz};
        for (int a = 0; a < 3; ++a) {
            make_tw(nn[a], tr, ti);
            if (int st = upload(c, &w.twr[a], tr)) return st;
            if (int st = upload(c, &w.twi[a], ti)) return st;
        }
    }
    API_CUDA(c, device_spectrum(c->d, c->precision == F8_MIXED, mean, w, c->energy_dev, c->s));
    API_CUDA(c, cudaMemcpyAsync(energy, c->energy_dev, ((size_t)g.nx + 1) * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    API_CUDA(c, cudaStreamSynchronize(c->s));
    return F8_OK;
}

int f8_stats_begin(f8_ctx *c, int mode, const double *mu, const double *mv, const double *mw, int max_steps) {
    if (c && c->zwalls) return F8_ERR_UNSUPPORTED;   // the exchanged axes are not mapped back here
    if (!c || mode < 0 || mode > 2 || max_steps < 0) return F8_ERR_ARG;
    if (c->grid.dim != 3) return F8_ERR_UNSUPPORTED;
    if (mode == 2 && (!mu || !mv || !mw)) return F8_ERR_ARG;
    const size_t ni = c->d.ni;
    c->stats_mode = 0;
    c->stats_n = 0;
    if (mode == 0) return F8_OK;
    if (!c->stats_sum) API_CUDA(c, c->alloc(&c->stats_sum, 3 * ni));
    API_CUDA(c, cudaMemsetAsync(c->stats_sum, 0, 3 * ni * sizeof(double), c->s));
    if (mode == 1 && max_steps > c->stats_max) {
        if (c->stats_probe) cudaFree(c->stats_probe);
        c->stats_probe = nullptr;
        c->stats_max = 0;
        API_CUDA(c, cudaMalloc(&c->stats_probe, (size_t)3 * max_steps * c->d.g.nz * sizeof(double)));
        c->stats_max = max_steps;
    }
    if (mode == 2) {
        const double *mean[3];
        if (int st = upload_means(c, mu, mv, mw, mean)) return st;
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    c->stats_mode = mode;
    return F8_OK;
}

int f8_stats_read(f8_ctx *c, double *su, double *sv, double *sw, double *probes, int *nsteps) {
    if (!c) return F8_ERR_ARG;
    const size_t ni = c->d.ni;
    double *dst[3] = {su, sv, sw};
    for (int q = 0; q < 3; ++q)
        if (dst[q] && c->stats_sum)
            API_CUDA(c, cudaMemcpyAsync(dst[q], c->stats_sum + q * ni, ni * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    const int n = std::min(c->stats_n, c->stats_max);
    if (probes && c->stats_probe) {
        const size_t per = (size_t)c->stats_max * c->d.g.nz;
        for (int q = 0; q < 3; ++q)
            API_CUDA(c, cudaMemcpyAsync(probes + (size_t)q * n * c->d.g.nz, c->stats_probe + q * per,
                                        (size_t)n * c->d.g.nz * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    if (nsteps) *nsteps = c->stats_n;
    return F8_OK;
}

int f8_selection_codes(f8_ctx *c, unsigned char *codes) {
    if (c && c->zwalls) return F8_ERR_UNSUPPORTED;   // the exchanged axes are not mapped back here
    if (!c || !codes) return F8_ERR_ARG;
    if (!c->loaded || c->step == c->step0 || c->phys.beta == 1.0) return F8_ERR_STATE;
    const f8::Geo &g = c->d.g;
    const int rows = f8::prows(g), r0 = f8::prow0(g);
    std::vector<unsigned char> in((size_t)g.nx * g.ny * g.nz), gh;
    API_CUDA(c, cudaMemcpyAsync(in.data(), c->d.codes, in.size(), cudaMemcpyDeviceToHost, c->s));
    if (g.walls) {
        gh.resize((size_t)g.nx * 2 * g.nz);
        API_CUDA(c, cudaMemcpyAsync(gh.data(), c->d.codes_g, gh.size(), cudaMemcpyDeviceToHost, c->s));
    }
    API_CUDA(c, cudaStreamSynchronize(c->s));
    for (int k = 1; k <= g.nz; ++k)
        for (int r = 0; r < rows; ++r) {
            const int j = r0 + r;
            for (int i = 1; i <= g.nx; ++i)
                codes[(size_t)(i - 1) + (size_t)g.nx * ((size_t)r + (size_t)rows * (k - 1))] =
                    (j >= 1 && j <= g.ny) ? in[f8::qix(g, i, j, k)] : gh[f8::gcix(g, i, j, k)];
        }
    return F8_OK;
}

int f8_markers(f8_ctx *c, int *n, double *xy) {
    if (!c) return F8_ERR_ARG;
    if (n) *n = (int)c->mk.size();
    if (xy)
        for (size_t m = 0; m < c->mk.size(); ++m) { xy[2 * m] = c->mk[m].x; xy[2 * m + 1] = c->mk[m].y; }
    return F8_OK;
}

int f8_set_timing(f8_ctx *c, int enable) {
    if (!c) return F8_ERR_ARG;
    c->timing = enable != 0;
    return F8_OK;
}

int f8_kernel_timing(f8_ctx *c, double *kernel_ms, long long *steps_timed) {
    if (!c || !kernel_ms) return F8_ERR_ARG;
    if (c->precision != F8_MIXED) return F8_ERR_UNSUPPORTED;
    for (int q = 0; q < NKERNEL; ++q) kernel_ms[q] = c->kernel_ms[q];
    if (steps_timed) *steps_timed = c->kernel_steps;
    return F8_OK;
}

int f8_timing(f8_ctx *c, double *total_ms, double *stage_ms, long long *steps_timed) {
    if (!c) return F8_ERR_ARG;
    if (total_ms) *total_ms = c->total_ms;
    if (stage_ms)
        for (int q = 0; q < NSTAGE; ++q) stage_ms[q] = c->stage_ms[q];
    if (steps_timed) *steps_timed = c->timed_steps;
    return F8_OK;
}

int f8_timing_reset(f8_ctx *c) {
    if (!c) return F8_ERR_ARG;
    c->total_ms = 0.0;
    for (int q = 0; q < NSTAGE; ++q) c->stage_ms[q] = 0.0;
    for (int q = 0; q < NKERNEL; ++q) c->kernel_ms[q] = 0.0;
    c->timed_steps = 0;
    c->kernel_steps = 0;
    c->step_launches = 0;
    return F8_OK;
}

const char *f8_strerror(int st) {
    switch (st) {
    case F8_OK: return "ok";
    case F8_ERR_ARG: return "invalid argument";
    case F8_ERR_STATE: return "call out of order (load before step)";
    case F8_ERR_NOMEM: return "device allocation failed";
    case F8_ERR_CUDA: return "CUDA runtime error";
    case F8_ERR_NAN: return "NaN in the velocity field";
    case F8_ERR_UNSUPPORTED: return "unsupported option";
    case F8_ERR_NO_DEVICE: return "no CUDA device";
    case F8_ERR_TOO_LARGE: return "grid exceeds the fixed workspace of the allocation-free solve";
    case F8_WARN_NEWTON: return "Newton iteration limit reached in some cells";
    case F8_WARN_SOR: return "SOR iteration limit reached";
    default: return "unknown status";
    }
}

void f8_destroy(f8_ctx *c) {
    if (!c) return;
    c->release();
    delete c;
}

}  // extern "C"
