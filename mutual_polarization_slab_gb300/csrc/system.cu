// System object (precomputed geometry + FFT plans), the batched matvec, and the
// GMRES / mixed-precision iterative-refinement solvers
// (EW/ewald.py:1146-1236, EW/capacitance.py:60-321).
#include <cufft.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "grid.cuh"
#include "realspace.cuh"
#include "tiles.cuh"
#include "quad.cuh"
#include "sizes.cuh"
#include <algorithm>
#include "dffft.cuh"
#include "adjoint.cuh"
#include "gradop.cuh"

using namespace mps;

// Ordinal of the current device: every process-wide cache below is keyed by it, because a cuFFT plan,
// a device buffer and a timing all belong to the device that made them.
static int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return dev;
}

// cuFFT plans are cached per process, keyed by (device, type, grid, batch), so
// building a new system for a new configuration of the same grid creates no plan.
// Each system owns its work area; the (work area, stream, exec) sequence is
// issued under one mutex.
struct PlanKey {
    int dev, type, nx, ny, nz, batch;
    bool operator<(const PlanKey &o) const {
        if (dev != o.dev) return dev < o.dev;
        if (type != o.type) return type < o.type;
        if (nx != o.nx) return nx < o.nx;
        if (ny != o.ny) return ny < o.ny;
        if (nz != o.nz) return nz < o.nz;
        return batch < o.batch;
    }
};
struct CachedPlan {
    cufftHandle h;
    size_t work;
};
static std::map<PlanKey, CachedPlan> g_plans;
static std::mutex g_plan_mu;

// Green's coefficients depend only on (grid, box, xi, eta): cached per process
// and device (like the FFT plans) and shared by every system built on the same
// grid.  Each buffer is filled on the stream of the system that needed it first;
// an event recorded there after the fill orders every other system's stream
// behind it (cudaStreamWaitEvent) before that system first reads the buffer.
// mps_kspace_cache_clear drops the cache (systems keep their references).
struct GreenKey {
    int N[3];
    int dev;
    double box[3], xi, eta[3];
    bool operator<(const GreenKey &o) const { return memcmp(this, &o, sizeof(GreenKey)) < 0; }
};
struct GreenCoef {
    double *h64 = nullptr;
    float *h32 = nullptr;
    float *hs32 = nullptr;   // H / |k|^2 of the gradient-form float32 operator (built on first use)
    float2 *tm6 = nullptr;   // double-float scale tensor H q q^T, 6 x Gc (built on first use)
    cudaEvent_t ev_h = nullptr, ev_hs32 = nullptr, ev_tm6 = nullptr;   // recorded after each fill
    ~GreenCoef() {
        if (h64) cudaFree(h64);
        if (h32) cudaFree(h32);
        if (hs32) cudaFree(hs32);
        if (tm6) cudaFree(tm6);
        if (ev_h) cudaEventDestroy(ev_h);
        if (ev_hs32) cudaEventDestroy(ev_hs32);
        if (ev_tm6) cudaEventDestroy(ev_tm6);
    }
};

// Records "buffer filled" on the filling stream.
static int green_mark_filled(cudaEvent_t *ev, cudaStream_t st) {
    if (!*ev) MPS_CUDA_TRY(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    MPS_CUDA_TRY(cudaEventRecord(*ev, st));
    return MPS_OK;
}
static std::map<GreenKey, std::shared_ptr<GreenCoef>> g_green;
static std::mutex g_green_mu;
constexpr size_t kGreenCacheMax = 4;

// Per-stage timing of the matvec (diagnostics): slab, spread, forward FFT,
// scale, inverse FFT, contract, real space.
constexpr int kStages = 7;
struct StageEvents {
    cudaEvent_t ev[kStages + 1];
    int precision;
};

// A coarser discretisation for the float32 gradient-form operator (the mixed solve's inner operator): its own
// grid, support P and spectral splitting eta, the same xi and the same pair sum.  The inner solves only have to
// reach 1e-4 .. 1e-3 of their right-hand sides, and every refinement residual uses the reference operator, so
// the inner grid is chosen for speed as long as its distance from the reference operator stays inside the
// refinement's drift bound (the grid of the tolerance rule at 2.5e-4 with the system's support P: 3e-5..6e-5).
struct InnerGrid {
    GridParams gp;
    int64_t Gc = 0;
    int32_t *start = nullptr;
    double *w64 = nullptr;
    float *w32 = nullptr, *g32 = nullptr;
    TileBins tb;
    float *grid = nullptr;   // max_rhs x G
    void *spec = nullptr;    // max_rhs x Gc complex
    std::shared_ptr<GreenCoef> green;
    bool hs32_ready = false;
};

// The Arnoldi steps of one GMRES configuration (precision, batch width, restart,
// Gram-Schmidt passes) of a system as an executable CUDA graph, with the
// persistent GMRES workspace whose addresses its kernels hold.
struct ArnoldiGraph {
    int precision = 0, nrhs = 0, restart = 0;
    bool reorth = false;
    char *ws = nullptr;
    size_t ws_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    long long body_launches = 0;   // this library's kernels per step (one execution of the loop body)
    bool failed = false;           // capture not possible here: the steps stay host-driven
};

struct mps_system {
    cudaStream_t stream = nullptr;   // creation stream: stream-ordered allocations and frees
    int64_t n = 0;
    int max_rhs = 1;
    int64_t n_diag = 1;
    double box[3];
    double xi, rc, slab_factor;
    GridParams gp;
    int64_t Gc = 0;
    double *x = nullptr;
    double *diag = nullptr;     // n_diag x n : dielectric + self
    int64_t ncell[3];
    int64_t n_pairs = 0;
    int64_t *row_ptr = nullptr;
    PairData<double> p64{};      // float64 pair data (dipole operator: built on demand from pdf)
    PairData<float> p32{};
    PairData<dfv> pdf{};         // double-float pair data of the dipole operator
    dfv *mdf = nullptr;          // double-float copy of the moments (real-space scratch), max_rhs x n x 3
    // dipole + quadrupole operator (kind 1): 9 couplings per pair and the
    // gradient/quadrupole diagonal
    int kind = 0;
    int ndof = 3;
    double *qcoef = nullptr;        // n_pairs x 9 (A..I) float64
    float *qcoef32 = nullptr;
    double *diagq = nullptr;        // n_diag x n: 15/(8 pi (eps-1)) + grad_quad_2(0)/2
    double *qkcoef = nullptr;       // half spectrum x 4: HES, HEQ/i, HGS/i, HGQ (with 1/G)
    float *qkcoef32 = nullptr;
    // polydisperse operator (kind 2): one scalar grid per vector, kernel values
    // K(d)/d of every particle's stencil, base offset node0 h - x per particle
    double *cs_base = nullptr;      // n x 3
    double *cs_g64 = nullptr;       // n x P^3
    float *cs_g32 = nullptr;
    double *cs_h64 = nullptr;       // half spectrum: exp(-(1-eta) q^2 / 4 xi^2) / q^2 / G
    float *cs_h32 = nullptr;
    int32_t *start = nullptr;
    int32_t *order = nullptr;        // particle ids sorted by (cell, id): spatial visiting order
    dfv *wdf = nullptr;              // double-float copy of w64 (built by the first double-float matvec)
    float *m32 = nullptr;            // float copy of the moments for the float32 pair sum (scratch)
    // side stream: the float32 pair sum runs beside the spread / FFT / contraction of the same matvec
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_res = nullptr;    // GMRES: residual estimates read back (a matvec may be queued behind it)
    cudaEvent_t ev_diag = nullptr;   // the last upload of the permittivity-set indices
    int diag_up_n = 0;               // entries of diag_idx that match diag_idx_host (0: none uploaded yet)
    double *rs_buf = nullptr;        // max_rhs x n x 3: the pair-sum part of a float32 matvec
    // complex permittivities: vectors are (Re m, Im m) per particle (ndof 6); the real operator runs on the
    // 2 nc real vectors [Re m_0..Re m_{nc-1}, Im m_0..Im m_{nc-1}] and the imaginary diagonal couples them
    bool cplx = false;
    int max_rhs_c = 0;               // complex vectors per matvec (max_rhs = 2 max_rhs_c real ones)
    double *diag_im = nullptr;       // n_diag x n imaginary part of the diagonal
    double *cx_in = nullptr, *cx_out = nullptr;   // 2 max_rhs_c x n x 3 scratch
    double *w64 = nullptr;
    float *w32 = nullptr;
    double *h64 = nullptr;       // owned by green (shared, cached per grid)
    float *h32 = nullptr;
    std::shared_ptr<GreenCoef> green;
    double *grid64 = nullptr;
    void *spec64 = nullptr;
    float *grid32 = nullptr;
    void *spec32 = nullptr;
    void *cgrid = nullptr;      // complex (drop-in) pipeline, 3 x G double2
    double *rgrid2 = nullptr;   // 2 x 3 x G
    double *slab = nullptr;     // max_rhs
    int32_t *diag_idx = nullptr;  // max_rhs (device)
    int32_t *diag_idx_host = nullptr;  // pinned mirror (start of the pinned block below)
    // pinned host scratch of the solvers, in the same block: the frozen flags (max_rhs) and the convergence
    // scalars read back every GMRES step (6 max_rhs doubles); pinned so the reads are plain DMA
    int32_t *host_frozen = nullptr;
    double *host_scr = nullptr;
    void *fft_work = nullptr;
    size_t fft_work_bytes = 0;
    TileBins tb64, tb32;        // tile binning for the tiled spread/contract (per precision tile depth)
    TileBins tbg;               // tiles of the gradient-form spread (depth 12 where the grid allows it)
    double *partial64 = nullptr;
    int tb_use[2] = {-1, -1};         // tuner consumer that built tb64 / tb32
    float *partial32 = nullptr;
    float *partialg = nullptr;        // partial sums of the tiled gradient-form contraction (A/B form) ...
    int64_t partialg_n = 0;           // ... and its capacity in floats
    bool tiled = true;
    bool profile = false;
    std::vector<StageEvents> pending;
    std::vector<StageEvents> spare;
    double stage_ms[3][kStages] = {{0}};   // float64, float32, double-float matvecs
    int64_t stage_count[3] = {0, 0, 0};
    DfPlan3 dfp;                 // double-float FFT plans of the grid
    int df_state = 0;            // 0 not built yet, 1 usable, -1 unsupported grid
    int resid_prec = MPS_FP64;   // operator of the refinement residuals
    float *g32 = nullptr;        // gradient factors dw_d/dr of the gradient-form operator, n x 3 x P
    int inner_prec = MPS_FP32;   // operator of the mixed solve's inner GMRES
    // this system's stream has waited for the shared lazily built Green's buffers (hs32, tm6)
    bool hs32_ready = false, tm6_ready = false;
    InnerGrid *inner = nullptr;      // coarser inner discretisation of the gradient-form operator, or null
    // Arnoldi-step graphs (captured on their own stream once every lazily built buffer of the matvec exists:
    // after the first matvec of that precision and batch width outside a capture)
    std::vector<ArnoldiGraph> graphs;
    cudaStream_t cap = nullptr;
    cudaStream_t prep = nullptr;     // first-use set-up of the double-float residual beside the first inner solve
    cudaEvent_t ev_graph = nullptr;  // recorded after each graph launch (destroying the graphs waits on it)
    std::vector<std::pair<int, int>> mv_seen;   // (precision, batch width) of the matvecs run so far
    int32_t *host_step = nullptr;    // pinned: the step counter read back after a graph launch
    int32_t *host_herr = nullptr;    // pinned: the pair fill's table-range flag (dipole systems)
    cudaEvent_t ev_build = nullptr;  // recorded after that flag's copy at the end of the build
    bool build_check = false;        // the flag has not been read yet (build_status)
    bool build_failed = false;       // it was set: every later call returns MPS_TABLE_RANGE
};

// Pinned host blocks of destroyed systems, kept for the next system (cudaMallocHost and cudaFreeHost cost a
// few hundred microseconds each; a configuration loop would pay them for every system).  Pinned memory is not
// tied to a device.
static std::mutex g_pinned_mu;
static std::multimap<size_t, void *> g_pinned_free;

static void *pinned_take(size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        auto it = g_pinned_free.lower_bound(bytes);
        if (it != g_pinned_free.end() && it->first <= 2 * bytes + 4096) {
            void *p = it->second;
            g_pinned_free.erase(it);
            return p;
        }
    }
    void *p = nullptr;
    // the block's size is kept in front of it so it can go back to the free list
    if (cudaMallocHost(&p, bytes + 64) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    *reinterpret_cast<size_t *>(p) = bytes;
    return static_cast<char *>(p) + 64;
}

static void pinned_give(void *q) {
    if (!q) return;
    void *p = static_cast<char *>(q) - 64;
    const size_t bytes = *reinterpret_cast<size_t *>(p);
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    if (g_pinned_free.size() >= 64) {   // bound what is kept
        cudaFreeHost(p);
        return;
    }
    g_pinned_free.emplace(bytes, q);
}

static bool matvec_seen(const mps_system *s, int precision, int nrhs) {
    for (const auto &p : s->mv_seen)
        if (p.first == precision && p.second == nrhs) return true;
    return false;
}

static void free_system(mps_system *s) {
    if (!s) return;
    // a matvec that failed between fork and join may leave pair-sum work on the side stream
    if (s->side) cudaStreamSynchronize(s->side);
    if (s->cap) cudaStreamSynchronize(s->cap);   // set-up work of a failed create may still run there
    if (s->prep) cudaStreamSynchronize(s->prep);
    for (auto &e : s->pending)
        for (int k = 0; k <= kStages; ++k) cudaEventDestroy(e.ev[k]);
    for (auto &e : s->spare)
        for (int k = 0; k <= kStages; ++k) cudaEventDestroy(e.ev[k]);
    void *ptrs[] = {s->x, s->diag, s->row_ptr, s->p64.nbr, s->p64.A, s->p64.BA, s->p64.rx, s->p64.ry, s->p64.rz,
                    s->p32.A, s->p32.BA, s->p32.rx, s->p32.ry, s->p32.rz, s->start, s->w64, s->w32,
                    s->grid64, s->spec64, s->grid32, s->spec32, s->cgrid, s->rgrid2, s->slab, s->diag_idx,
                    s->fft_work, s->p64.dist, s->qcoef, s->qcoef32, s->diagq, s->qkcoef, s->qkcoef32,
                    s->cs_base, s->cs_g64, s->cs_g32, s->cs_h64, s->cs_h32, s->g32, s->pdf.A, s->pdf.BA,
                    s->pdf.rx, s->pdf.ry, s->pdf.rz, s->pdf.dist, s->mdf, s->order, s->wdf, s->m32, s->diag_im,
                    s->cx_in, s->cx_out};
    for (void *p : ptrs)
        if (p) cudaFreeAsync(p, s->stream);
    if (s->ev_diag) cudaEventSynchronize(s->ev_diag);   // the last index upload reads the pinned block
    if (s->diag_idx_host) pinned_give(s->diag_idx_host);
    if (s->rs_buf) cudaFreeAsync(s->rs_buf, s->stream);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->ev_res) cudaEventDestroy(s->ev_res);
    if (s->ev_diag) cudaEventDestroy(s->ev_diag);
    if (s->ev_build) cudaEventDestroy(s->ev_build);
    if (s->ev_graph) {
        cudaEventSynchronize(s->ev_graph);
        cudaEventDestroy(s->ev_graph);
    }
    for (auto &g : s->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.ws) cudaFreeAsync(g.ws, s->stream);
    }
    if (s->cap) cudaStreamDestroy(s->cap);
    if (s->prep) cudaStreamDestroy(s->prep);
    tile_bins_free(s->tb64, s->stream);
    tile_bins_free(s->tb32, s->stream);
    tile_bins_free(s->tbg, s->stream);
    if (s->partial64) cudaFreeAsync(s->partial64, s->stream);
    if (s->partial32) cudaFreeAsync(s->partial32, s->stream);
    if (s->partialg) cudaFreeAsync(s->partialg, s->stream);
    if (InnerGrid *ig = s->inner) {
        void *ip[] = {ig->start, ig->w64, ig->w32, ig->g32, ig->grid, ig->spec};
        for (void *q : ip)
            if (q) cudaFreeAsync(q, s->stream);
        tile_bins_free(ig->tb, s->stream);
        delete ig;
    }
    delete s;
}

// Device memory of a system comes from the device's default stream-ordered pool
// with its release threshold raised, so building a system for the next
// configuration reuses the previous one's memory instead of mapping new pages.
static void configure_pool_once() {
    static std::mutex mu;
    static std::vector<bool> done;   // per device ordinal
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(mu);
    if ((size_t)dev < done.size() && done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if ((size_t)dev >= done.size()) done.resize(dev + 1, false);
    done[dev] = true;
}

template <typename P>
static int dalloc(P **p, size_t bytes, cudaStream_t st) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync((void **)p, bytes, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return e == cudaErrorMemoryAllocation ? MPS_NO_MEMORY : MPS_CUDA_ERR;
    }
    return MPS_OK;
}

// Persistent buffers shared between systems (cached Green's coefficients).
template <typename P>
static int dalloc_persistent(P **p, size_t bytes) {
    cudaError_t e = cudaMalloc((void **)p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return e == cudaErrorMemoryAllocation ? MPS_NO_MEMORY : MPS_CUDA_ERR;
    }
    return MPS_OK;
}

#define MPS_TRY(expr)           \
    do {                        \
        int _r = (expr);        \
        if (_r != MPS_OK) return _r; \
    } while (0)

#define CUFFT_TRY(expr)                              \
    do {                                             \
        if ((expr) != CUFFT_SUCCESS) return MPS_CUFFT_ERR; \
    } while (0)

static int get_plan(cufftType type, const GridParams &gp, int batch, CachedPlan *out) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    PlanKey key{current_device(), (int)type, gp.N[0], gp.N[1], gp.N[2], batch};
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        *out = it->second;
        return MPS_OK;
    }
    cufftHandle h;
    CUFFT_TRY(cufftCreate(&h));
    if (cufftSetAutoAllocation(h, 0) != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return MPS_CUFFT_ERR;
    }
    int n[3] = {gp.N[2], gp.N[1], gp.N[0]};
    size_t ws = 0;
    if (cufftMakePlanMany(h, 3, n, nullptr, 1, 0, nullptr, 1, 0, type, batch, &ws) != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return MPS_CUFFT_ERR;
    }
    CachedPlan cp{h, ws};
    g_plans[key] = cp;
    *out = cp;
    return MPS_OK;
}

static int ensure_work(mps_system *s, size_t need, cudaStream_t st) {
    if (need <= s->fft_work_bytes) return MPS_OK;
    if (s->fft_work) cudaFreeAsync(s->fft_work, st);
    s->fft_work = nullptr;
    s->fft_work_bytes = 0;
    MPS_TRY(dalloc(&s->fft_work, need, st));
    s->fft_work_bytes = need;
    return MPS_OK;
}

// Runs one cached plan on this system's work area and stream.
static int exec_plan_gp(mps_system *s, const GridParams &gp, cufftType type, int batch, void *in, void *out, int dir,
                        cudaStream_t st) {
    CachedPlan cp;
    MPS_TRY(get_plan(type, gp, batch, &cp));
    MPS_TRY(ensure_work(s, cp.work, st));
    std::lock_guard<std::mutex> lk(g_plan_mu);
    CUFFT_TRY(cufftSetWorkArea(cp.h, s->fft_work));
    CUFFT_TRY(cufftSetStream(cp.h, st));
    switch (type) {
        case CUFFT_D2Z: CUFFT_TRY(cufftExecD2Z(cp.h, (cufftDoubleReal *)in, (cufftDoubleComplex *)out)); break;
        case CUFFT_Z2D: CUFFT_TRY(cufftExecZ2D(cp.h, (cufftDoubleComplex *)in, (cufftDoubleReal *)out)); break;
        case CUFFT_R2C: CUFFT_TRY(cufftExecR2C(cp.h, (cufftReal *)in, (cufftComplex *)out)); break;
        case CUFFT_C2R: CUFFT_TRY(cufftExecC2R(cp.h, (cufftComplex *)in, (cufftReal *)out)); break;
        case CUFFT_Z2Z:
            CUFFT_TRY(cufftExecZ2Z(cp.h, (cufftDoubleComplex *)in, (cufftDoubleComplex *)out, dir));
            break;
        default: return MPS_BAD_ARG;
    }
    return MPS_OK;
}

static int exec_plan(mps_system *s, cufftType type, int batch, void *in, void *out, int dir, cudaStream_t st) {
    return exec_plan_gp(s, s->gp, type, batch, in, out, dir, st);
}

static int ensure_grids(mps_system *s, int precision, cudaStream_t st) {
    // component grids per vector: one scalar grid for the polydisperse operator
    // (complex mode: the real operator runs on max_rhs real 3-vectors)
    size_t nr = (size_t)s->max_rhs * (s->kind == MPS_POLYDISPERSE ? 1 : (s->cplx ? 3 : s->ndof));
    if (precision == MPS_FP64) {
        if (!s->grid64) MPS_TRY(dalloc(&s->grid64, nr * s->gp.G * sizeof(double), st));
        if (!s->spec64) MPS_TRY(dalloc(&s->spec64, nr * s->Gc * 2 * sizeof(double), st));
    } else {
        if (!s->grid32) MPS_TRY(dalloc(&s->grid32, nr * s->gp.G * sizeof(float), st));
        if (!s->spec32) MPS_TRY(dalloc(&s->spec32, nr * s->Gc * 2 * sizeof(float), st));
    }
    return MPS_OK;
}

static int upload_diag_idx(mps_system *s, const int32_t *diag_index, int nrhs, cudaStream_t st) {
    const int nup = s->cplx ? 2 * nrhs : nrhs;
    std::vector<int32_t> want(nup);
    for (int r = 0; r < nrhs; ++r) {
        int32_t v = diag_index ? diag_index[r] : 0;
        if (v < 0 || v >= s->n_diag) return MPS_BAD_ARG;
        want[r] = v;
        if (s->cplx) want[nrhs + r] = v;   // the imaginary halves use the same sets
    }
    // unchanged since the last upload (the usual case for repeated matvecs): no copy and no host wait, only
    // stream order behind the copy that put them there
    if (s->diag_up_n == nup && std::equal(want.begin(), want.end(), s->diag_idx_host)) {
        if (s->ev_diag) MPS_CUDA_TRY(cudaStreamWaitEvent(st, s->ev_diag, 0));
        return MPS_OK;
    }
    // stage through pinned memory so the async copy does not read caller memory late; the previous copy must
    // have finished reading the staging buffer before it is overwritten
    if (!s->ev_diag) MPS_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_diag, cudaEventDisableTiming));
    else MPS_CUDA_TRY(cudaEventSynchronize(s->ev_diag));
    std::copy(want.begin(), want.end(), s->diag_idx_host);
    MPS_CUDA_TRY(cudaMemcpyAsync(s->diag_idx, s->diag_idx_host, sizeof(int32_t) * nup, cudaMemcpyHostToDevice, st));
    MPS_CUDA_TRY(cudaEventRecord(s->ev_diag, st));
    s->diag_up_n = nup;
    return MPS_OK;
}

static int stage_begin(mps_system *s, int precision, StageEvents **ev, cudaStream_t st) {
    *ev = nullptr;
    if (!s->profile) return MPS_OK;
    StageEvents e;
    if (!s->spare.empty()) {
        e = s->spare.back();
        s->spare.pop_back();
    } else {
        for (int k = 0; k <= kStages; ++k) MPS_CUDA_TRY(cudaEventCreate(&e.ev[k]));
    }
    e.precision = precision;
    s->pending.push_back(e);
    *ev = &s->pending.back();
    MPS_CUDA_TRY(cudaEventRecord((*ev)->ev[0], st));
    return MPS_OK;
}

#define STAGE_MARK(k)                                                   \
    do {                                                                \
        if (ev) MPS_CUDA_TRY(cudaEventRecord(ev->ev[(k)], st));         \
    } while (0)

// Autotuner for the tiled kernels: the tile depth (z) is timed on the first
// system of each (grid, support, consumer, batch width) with the kernels that
// consumer runs, and the fastest is kept for the rest of the process.  The
// consumers: the float32 reference operator (tiled spread + contract), the
// float32 gradient operator (its spread; depth 12 without timing where the grid
// allows it, see tuned_depth), the float64 operator (spread) and the double-float
// operator (spread).  The reference-form float32 kernels use tb32, the gradient
// form tbg, the float64-width kernels tb64.
enum TileUse { kTileRef32 = 0, kTileGrad32 = 1, kTileF64 = 2, kTileDF = 3 };
struct TuneKey {
    int dev;
    int N[3];
    int P;
    int use;
    int nrhs;
    bool operator<(const TuneKey &o) const { return memcmp(this, &o, sizeof(TuneKey)) < 0; }
};
struct TuneResult {
    int tz;
    float ms[2];   // timings of depth 4 and 8, -1 if not run
};
static std::map<TuneKey, TuneResult> g_tune;
static std::mutex g_tune_mu;
static const int kDepths[2] = {4, 8};

static int time_tiles(mps_system *s, int use, int tz, int nrhs, const double *m, double *out, cudaStream_t st,
                      float *ms) {
    TileBins tb;
    MPS_TRY(tile_bins_build(s->start, s->n, s->gp, tz, tb, st));
    float *partial = nullptr;
    if (use == kTileRef32) {
        MPS_TRY(tile_bins_pentry(s->start, s->gp, tb, st));
        MPS_TRY(dalloc(&partial, (size_t)tb.nentries * 9 * sizeof(float), st));
    }
    cudaEvent_t e0, e1;
    MPS_CUDA_TRY(cudaEventCreate(&e0));
    MPS_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int rc = MPS_OK;
    for (int rep = 0; rep < 4 && rc == MPS_OK; ++rep) {
        cudaEventRecord(e0, st);
        switch (use) {
            case kTileRef32:
                rc = spread_tiled<float>(m, s->n, nrhs, s->start, s->w32, s->gp, tb, s->grid32, st);
                if (rc == MPS_OK)
                    rc = contract_tiled<float>(s->grid32, s->n, nrhs, s->start, s->w32, s->gp, tb, partial, out, st);
                break;
            case kTileGrad32:
                rc = spread_grad_tiled(m, s->n, nrhs, s->start, s->w32, s->g32, s->gp, tb, s->grid32, st);
                break;
            case kTileF64:
                rc = spread_tiled<double>(m, s->n, nrhs, s->start, s->w64, s->gp, tb, s->grid64, st);
                break;
            default:
                rc = spread_tiled_df(m, s->n, nrhs, s->start, s->wdf, s->gp, tb, (dfv *)s->grid64, st);
                break;
        }
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && t < best) best = t;   // first repetition warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (partial) cudaFreeAsync(partial, st);
    tile_bins_free(tb, st);
    *ms = best;
    return rc;
}

static bool tile_depth_known(const mps_system *s, int use);

static int tuned_depth(mps_system *s, int use, cudaStream_t st, int *tz) {
    // MPS_TILE_DEPTH=4 or 8 fixes the depth instead of timing (A/B comparisons and tests); not cached
    if (const char *fd = getenv("MPS_TILE_DEPTH")) {
        const int d = atoi(fd);
        if ((d == 4 || d == 8 || ((d == 12 || d == 16) && use == kTileGrad32)) && tiles_supported(s->gp, d)) {
            *tz = d;
            return MPS_OK;
        }
    }
    // The gradient-form spread takes depth 12 where the grid allows it: timed alone depth 8 is a few per cent
    // faster, but the whole gradient matvec is faster with fewer, wider CTAs that leave room for the pair sum
    // running beside it on the side stream (depth 16: 4-6 % faster than 8 at N = 1e5, 192^3 and 144^3; depth 12,
    // at 4 blocks per SM against 3, another 0.6 % of the whole solve at 144^3).
    if (use == kTileGrad32 && tiles_supported(s->gp, 12)) {
        *tz = 12;
        return MPS_OK;
    }
    TuneKey key;
    memset(&key, 0, sizeof(key));
    key.dev = current_device();
    for (int k = 0; k < 3; ++k) key.N[k] = s->gp.N[k];
    key.P = s->gp.P;
    key.use = use;
    key.nrhs = s->max_rhs < 3 ? s->max_rhs : 3;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            *tz = it->second.tz;
            return MPS_OK;
        }
    }
    TuneResult res{0, {-1.f, -1.f}};
    int ok = 0;
    for (int i = 0; i < 2; ++i) ok += tiles_supported(s->gp, kDepths[i]) ? 1 : 0;
    if (ok == 0) {
        *tz = 0;
        return MPS_OK;
    }
    const int nrhs = key.nrhs;
    const int64_t tot = (int64_t)nrhs * 3 * s->n;
    double *m = nullptr, *out = nullptr;
    MPS_TRY(dalloc(&m, sizeof(double) * tot, st));
    MPS_TRY(dalloc(&out, sizeof(double) * tot, st));
    MPS_CUDA_TRY(cudaMemsetAsync(m, 0, sizeof(double) * tot, st));
    float best = 1e30f;
    for (int i = 0; i < 2; ++i) {
        if (!tiles_supported(s->gp, kDepths[i])) continue;
        float ms = 0.f;
        int rc = time_tiles(s, use, kDepths[i], nrhs, m, out, st, &ms);
        if (rc != MPS_OK) {
            cudaFreeAsync(m, st);
            cudaFreeAsync(out, st);
            return rc;
        }
        res.ms[i] = ms;
        if (ms < best) {
            best = ms;
            res.tz = kDepths[i];
        }
    }
    cudaFreeAsync(m, st);
    cudaFreeAsync(out, st);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = res;
    }
    *tz = res.tz;
    return MPS_OK;
}

// The tile depth of a consumer is settled without timing: fixed by MPS_TILE_DEPTH, the gradient form's fixed
// depth, or already timed in this process for this (device, grid, support, consumer, batch width).
static bool tile_depth_known(const mps_system *s, int use) {
    if (const char *fd = getenv("MPS_TILE_DEPTH")) {
        const int d = atoi(fd);
        if (d == 4 || d == 8 || ((d == 12 || d == 16) && use == kTileGrad32)) return true;
    }
    if (use == kTileGrad32) return true;
    TuneKey key;
    memset(&key, 0, sizeof(key));
    key.dev = current_device();
    for (int k = 0; k < 3; ++k) key.N[k] = s->gp.N[k];
    key.P = s->gp.P;
    key.use = use;
    key.nrhs = s->max_rhs < 3 ? s->max_rhs : 3;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune.find(key) != g_tune.end();
}

// Lazily bins the particles for the tiled kernels of one precision (tile depth
// from the autotuner, timed for the consumer that asks first).
static int ensure_tiles(mps_system *s, int use, cudaStream_t st, bool *used) {
    *used = false;
    // the tiled kernels use the separable Gaussian weights of the dipole operator
    if (!s->tiled || s->kind != MPS_DIPOLE || !s->w32 || !s->w64) return MPS_OK;
    const bool dbl = use == kTileF64 || use == kTileDF;
    const bool grad = use == kTileGrad32;
    TileBins &tb = dbl ? s->tb64 : (grad ? s->tbg : s->tb32);
    if (!tb.mem) {
        MPS_TRY(ensure_grids(s, dbl ? MPS_FP64 : MPS_FP32, st));
        int tz = 0;
        MPS_TRY(tuned_depth(s, use, st, &tz));
        if (tz == 0 || !tiles_supported(s->gp, tz)) {
            s->tiled = false;
            return MPS_OK;
        }
        MPS_TRY(tile_bins_build(s->start, s->n, s->gp, tz, tb, st));
        if (!grad) s->tb_use[dbl ? 0 : 1] = use;
    }
    if (!dbl && !s->partial32 && use == kTileRef32)
        MPS_TRY(dalloc(&s->partial32, (size_t)tb.nentries * 9 * sizeof(float), st));
    *used = true;
    return MPS_OK;
}

static bool df_usable(mps_system *s);

// Float32 pair sum (accumulates into out) on the system's float copy of the moments.
static int real_space_f32(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    if (!s->m32) MPS_TRY(dalloc(&s->m32, sizeof(float) * m32_floats(s->n, s->max_rhs), st));
    return real_space_csr_f32(m, s->m32, out, s->n, nrhs, s->row_ptr, s->p32, s->diag, s->diag_idx, s->slab, true,
                              s->order, st);
}

// Float64 pair data of the dipole operator, converted from the double-float list
// the first time a float64 path needs it.
static int ensure_p64(mps_system *s, cudaStream_t st) {
    if (s->kind != MPS_DIPOLE || s->p64.A) return MPS_OK;
    const size_t b = sizeof(double) * (size_t)s->n_pairs;
    MPS_TRY(dalloc(&s->p64.A, b, st));
    MPS_TRY(dalloc(&s->p64.BA, b, st));
    MPS_TRY(dalloc(&s->p64.rx, b, st));
    MPS_TRY(dalloc(&s->p64.ry, b, st));
    MPS_TRY(dalloc(&s->p64.rz, b, st));
    MPS_TRY(dalloc(&s->p64.dist, b, st));
    return pairs_df_to_f64(s->pdf, s->n_pairs, s->p64, st);
}

// The float32 operator runs cuFFT R2C/C2R + a scale pass; MPS_FFT32=own in the
// environment selects the hand-written transforms of dffft.cu (scale fused into
// the z pass) instead, where the grid allows.
static bool own_fft32() {
    const char *e = getenv("MPS_FFT32");
    return e && strcmp(e, "own") == 0;
}

template <typename T>
static int matvec_impl(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    const bool dbl = sizeof(T) == 8;
    const bool own_fft = !dbl && own_fft32() && df_usable(s);
    bool use_tiles = false;
    MPS_TRY(ensure_tiles(s, dbl ? kTileF64 : kTileRef32, st, &use_tiles));
    const TileBins &tb = dbl ? s->tb64 : s->tb32;
    T *partial = dbl ? (T *)s->partial64 : (T *)s->partial32;
    MPS_TRY(ensure_grids(s, dbl ? MPS_FP64 : MPS_FP32, st));
    T *grid = dbl ? (T *)s->grid64 : (T *)s->grid32;
    void *spec = dbl ? s->spec64 : s->spec32;
    const T *w = dbl ? (const T *)s->w64 : (const T *)s->w32;
    const T *hh = dbl ? (const T *)s->h64 : (const T *)s->h32;
    const double vol = s->box[0] * s->box[1] * s->box[2];
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, dbl ? MPS_FP64 : MPS_FP32, &ev, st));
    if (s->slab_factor != 0.0) MPS_TRY(slab_terms(m, s->n, nrhs, s->slab_factor / vol, s->slab, st));
    STAGE_MARK(1);
    if (use_tiles)
        MPS_TRY(spread_tiled<T>(m, s->n, nrhs, s->start, w, s->gp, tb, grid, st));
    else
        MPS_TRY(spread<T>(m, s->n, nrhs, s->start, w, s->gp, grid, st));
    STAGE_MARK(2);
    if (own_fft) {
        MPS_TRY(f32_forward_xy((const float *)grid, (float2 *)spec, 3 * nrhs, s->gp, s->dfp, st));
        STAGE_MARK(3);
        MPS_TRY(f32_z_scale_dipole((float2 *)spec, nrhs, s->gp, s->dfp, (const float *)hh, st));
        STAGE_MARK(4);
        MPS_TRY(f32_inverse_yx((float2 *)spec, (float *)grid, 3 * nrhs, s->gp, s->dfp, st));
        STAGE_MARK(5);
    } else {
        MPS_TRY(exec_plan(s, dbl ? CUFFT_D2Z : CUFFT_R2C, 3 * nrhs, grid, spec, 0, st));
        STAGE_MARK(3);
        MPS_TRY(scale_half<T>(spec, nrhs, s->gp, hh, st));
        STAGE_MARK(4);
        MPS_TRY(exec_plan(s, dbl ? CUFFT_Z2D : CUFFT_C2R, 3 * nrhs, spec, grid, 0, st));
        STAGE_MARK(5);
    }
    // float64: the warp-per-particle gather keeps more lanes busy, which is what
    // matters at GB300's float64 issue rate; float32: the shared-memory tile.
    if (use_tiles && !dbl) {
        MPS_TRY(tile_bins_pentry(s->start, s->gp, s->tb32, st));
        MPS_TRY(contract_tiled<T>(grid, s->n, nrhs, s->start, w, s->gp, tb, partial, out, st));
    }
    else
        MPS_TRY(contract<T>(grid, s->n, nrhs, s->start, w, s->gp, out, st));
    STAGE_MARK(6);
    if (dbl) {
        MPS_TRY(ensure_p64(s, st));
        MPS_TRY(real_space_csr<double>(m, out, s->n, nrhs, s->row_ptr, s->p64, s->diag, s->diag_idx, s->slab, true, st));
    } else {
        MPS_TRY(real_space_f32(s, m, out, nrhs, st));
    }
    STAGE_MARK(7);
    return MPS_OK;
}

// Float64-accurate matvec without float64 issue in the wave-space stages: the
// tiled spread and contraction accumulate in double-float arithmetic (float64
// weights and grids), the FFTs and Green's scale are the double-float transforms
// of dffft.cu; the pair sum is the float64 kernel.
// First-use setup of the double-float operator: weights, tile bins (autotuned depth), grids, scale tensor.
static int df_prepare(mps_system *s, cudaStream_t st, bool *use_tiles_out) {
    const int64_t nw = (int64_t)s->n * 3 * s->gp.P;
    if (!s->wdf) {
        MPS_TRY(dalloc(&s->wdf, sizeof(dfv) * (size_t)nw, st));
        MPS_TRY(weights_df(s->w64, nw, s->wdf, st));
    }
    bool use_tiles = false;
    MPS_TRY(ensure_tiles(s, kTileDF, st, &use_tiles));
    MPS_TRY(ensure_grids(s, MPS_FP64, st));
    if (!s->tm6_ready) {
        std::lock_guard<std::mutex> lk(g_green_mu);
        if (!s->green->tm6) {
            float2 *tm = nullptr;
            MPS_TRY(dalloc_persistent(&tm, sizeof(float2) * 6 * s->Gc));
            MPS_TRY(df_scale_table(s->gp, s->green->h64, tm, st));
            MPS_TRY(green_mark_filled(&s->green->ev_tm6, st));
            s->green->tm6 = tm;
        } else {
            MPS_CUDA_TRY(cudaStreamWaitEvent(st, s->green->ev_tm6, 0));   // filled by another system
        }
        s->tm6_ready = true;
    }
    *use_tiles_out = use_tiles;
    return MPS_OK;
}

// Wave-space field grids of nrhs moment vectors with the float64-accurate operator: double-float spread,
// FFTs and dipole scale; the 3 nrhs component grids are left in s->grid64 as (hi, lo) float pairs.  Stage
// marks 2..5 of the calling matvec (ev may be null).
static int df_field_grids(mps_system *s, const double *m, int nrhs, StageEvents *ev, cudaStream_t st,
                          bool *use_tiles_out) {
    bool use_tiles = false;
    MPS_TRY(df_prepare(s, st, &use_tiles));
    dfv *grid = (dfv *)s->grid64;           // (hi, lo) float pairs: the size of a double
    float4 *spec = (float4 *)s->spec64;     // float4 per complex value: the size of a double2
    const int64_t gvals = (int64_t)3 * nrhs * s->gp.G;
    if (use_tiles) {
        MPS_TRY(spread_tiled_df(m, s->n, nrhs, s->start, s->wdf, s->gp, s->tb64, grid, st));
    } else {
        MPS_TRY(spread<double>(m, s->n, nrhs, s->start, s->w64, s->gp, s->grid64, st));
        MPS_TRY(f64_to_dfv_inplace(s->grid64, gvals, st));
    }
    STAGE_MARK(2);
    MPS_TRY(df_forward_xy((const float2 *)grid, spec, 3 * nrhs, s->gp, s->dfp, st));
    STAGE_MARK(3);
    MPS_TRY(df_z_scale_dipole(spec, nrhs, s->gp, s->dfp, s->h64, s->green->tm6, st));
    STAGE_MARK(4);
    MPS_TRY(df_inverse_yx(spec, (float2 *)grid, 3 * nrhs, s->gp, s->dfp, st));
    STAGE_MARK(5);
    *use_tiles_out = use_tiles;
    return MPS_OK;
}

static bool pair_sum_beside(const StageEvents *ev);
static int pair_sum_fork(mps_system *s, const double *m, int nrhs, cudaStream_t st, bool df);
static int pair_sum_join(mps_system *s, double *out, int nrhs, cudaStream_t st);

static int matvec_df(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    const double vol = s->box[0] * s->box[1] * s->box[2];
    bool prepared_tiles = false;
    MPS_TRY(df_prepare(s, st, &prepared_tiles));   // first-use setup outside the stage timing
    (void)prepared_tiles;
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, MPS_DF, &ev, st));
    if (s->slab_factor != 0.0) MPS_TRY(slab_terms(m, s->n, nrhs, s->slab_factor / vol, s->slab, st));
    // the double-float pair sum runs beside the wave-space stages on the side stream, like the float32 one
    // (18.80 against 18.82 ms for the mixed step at the bench workload; the same sums, bit for bit)
    const bool beside = pair_sum_beside(ev);
    if (beside) MPS_TRY(pair_sum_fork(s, m, nrhs, st, true));
    STAGE_MARK(1);
    bool use_tiles = false;
    MPS_TRY(df_field_grids(s, m, nrhs, ev, st, &use_tiles));
    dfv *grid = (dfv *)s->grid64;
    const int64_t gvals = (int64_t)3 * nrhs * s->gp.G;
    const char *ce = getenv("MPS_DF_CONTRACT");   // "tiled": the tiled contraction (A/B timing)
    const bool tiled_contract = use_tiles && ce && strcmp(ce, "tiled") == 0;
    if (s->gp.P <= kMaxP && !tiled_contract) {
        MPS_TRY(contract_df_warp(grid, s->n, nrhs, s->order, s->start, s->wdf, s->gp, out, st));
    } else if (use_tiles) {
        if (!s->partial64) MPS_TRY(dalloc(&s->partial64, (size_t)s->tb64.nentries * 9 * sizeof(double), st));
        MPS_TRY(tile_bins_pentry(s->start, s->gp, s->tb64, st));
        MPS_TRY(contract_tiled_df(grid, s->n, nrhs, s->start, s->w64, s->gp, s->tb64, s->partial64, out, st));
    } else {
        MPS_TRY(dfv_to_f64_inplace(s->grid64, gvals, st));
        MPS_TRY(contract<double>(s->grid64, s->n, nrhs, s->start, s->w64, s->gp, out, st));
    }
    STAGE_MARK(6);
    if (beside) {
        MPS_TRY(pair_sum_join(s, out, nrhs, st));
    } else {
        if (!s->mdf) MPS_TRY(dalloc(&s->mdf, sizeof(dfv) * 3 * (size_t)s->n * s->max_rhs, st));
        MPS_TRY(real_space_csr_df(m, s->mdf, out, s->n, nrhs, s->row_ptr, s->pdf, s->diag, s->diag_idx, s->slab,
                                  true, s->order, st));
    }
    STAGE_MARK(7);
    return MPS_OK;
}

static bool df_usable(mps_system *s) {
    if (s->kind != MPS_DIPOLE) return false;
    if (s->df_state == 0) {
        if (df_plan(s->gp, &s->dfp) != MPS_OK) return false;
        s->df_state = s->dfp.ok ? 1 : -1;
    }
    return s->df_state == 1;
}

// Dipole + quadrupole operator (8 moments per sphere, CQ/MatrixVectorMultiply.m:31-77):
// the same spread / FFT / scale / FFT / contract / real-space stages over 8
// component grids per vector.
template <typename T>
static int matvec_quad(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    const bool dbl = sizeof(T) == 8;
    MPS_TRY(ensure_grids(s, dbl ? MPS_FP64 : MPS_FP32, st));
    T *grid = dbl ? (T *)s->grid64 : (T *)s->grid32;
    void *spec = dbl ? s->spec64 : s->spec32;
    const T *w = dbl ? (const T *)s->w64 : (const T *)s->w32;
    const T *kc = dbl ? (const T *)s->qkcoef : (const T *)s->qkcoef32;
    const T *pc = dbl ? (const T *)s->qcoef : (const T *)s->qcoef32;
    const PairData<T> &pd = *(const PairData<T> *)(dbl ? (const void *)&s->p64 : (const void *)&s->p32);
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, dbl ? MPS_FP64 : MPS_FP32, &ev, st));
    STAGE_MARK(1);
    MPS_TRY(spread_gen<T>(m, s->n, nrhs, 8, s->start, w, s->gp, grid, st));
    STAGE_MARK(2);
    MPS_TRY(exec_plan(s, dbl ? CUFFT_D2Z : CUFFT_R2C, 8 * nrhs, grid, spec, 0, st));
    STAGE_MARK(3);
    MPS_TRY(scale_quad<T>(spec, nrhs, s->gp, kc, st));
    STAGE_MARK(4);
    MPS_TRY(exec_plan(s, dbl ? CUFFT_Z2D : CUFFT_C2R, 8 * nrhs, spec, grid, 0, st));
    STAGE_MARK(5);
    MPS_TRY(contract_gen<T>(grid, s->n, nrhs, 8, s->start, w, s->gp, out, st));
    STAGE_MARK(6);
    MPS_TRY(real_space_quad<T>(m, out, s->n, nrhs, s->row_ptr, pd.nbr, pd.rx, pd.ry, pd.rz, pc, s->diag, s->diagq,
                               s->diag_idx, st));
    STAGE_MARK(7);
    return MPS_OK;
}

// The float32 pair sum is independent of the wave-space stages of the same
// matvec: pair_sum_fork runs it on the system's side stream into rs_buf (from
// the point the moments are ready on st), pair_sum_join makes st wait for it and
// adds it into out after the contraction.  MPS_PAIR_STREAM=same keeps it on st
// after the contraction (A/B timing); so do profiled matvecs (their stage times
// are taken on st).
__global__ void k_axpy1(const double *__restrict__ x, double *__restrict__ y, int64_t total);

static bool pair_sum_beside(const StageEvents *ev) {
    const char *ps = getenv("MPS_PAIR_STREAM");
    return ev == nullptr && !(ps && strcmp(ps, "same") == 0);
}

static int pair_sum_fork(mps_system *s, const double *m, int nrhs, cudaStream_t st, bool df) {
    if (!s->side) {
        MPS_CUDA_TRY(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
        MPS_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
        MPS_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    }
    // the real operator's vectors: 3 components per particle (complex systems run it on 2 nc real vectors)
    const size_t vals = (size_t)3 * s->n * s->max_rhs;
    if (!s->rs_buf) MPS_TRY(dalloc(&s->rs_buf, sizeof(double) * vals, st));
    if (!df && !s->m32) MPS_TRY(dalloc(&s->m32, sizeof(float) * m32_floats(s->n, s->max_rhs), st));
    if (df && !s->mdf) MPS_TRY(dalloc(&s->mdf, sizeof(dfv) * 3 * (size_t)s->n * s->max_rhs, st));
    MPS_CUDA_TRY(cudaEventRecord(s->ev_fork, st));
    MPS_CUDA_TRY(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
    if (df)
        MPS_TRY(real_space_csr_df(m, s->mdf, s->rs_buf, s->n, nrhs, s->row_ptr, s->pdf, s->diag, s->diag_idx,
                                  s->slab, false, s->order, s->side));
    else
        MPS_TRY(real_space_csr_f32(m, s->m32, s->rs_buf, s->n, nrhs, s->row_ptr, s->p32, s->diag, s->diag_idx,
                                   s->slab, false, s->order, s->side));
    MPS_CUDA_TRY(cudaEventRecord(s->ev_join, s->side));
    return MPS_OK;
}

static int pair_sum_join(mps_system *s, double *out, int nrhs, cudaStream_t st) {
    MPS_CUDA_TRY(cudaStreamWaitEvent(st, s->ev_join, 0));
    const int64_t tot = (int64_t)nrhs * s->n * 3;
    k_axpy1<<<grid_for(tot, 256), 256, 0, st>>>(s->rs_buf, out, tot);
    count_launch();
    MPS_CUDA_TRY(cudaGetLastError());
    return MPS_OK;
}

// Polydisperse operator (CS/ComputeField.m:23-57): scalar spread of the dipoles
// as charges, one FFT pair per vector, vector contraction, real space with the
// per-pair couplings of the two radii.
template <typename T>
static int matvec_cs(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    const bool dbl = sizeof(T) == 8;
    MPS_TRY(ensure_grids(s, dbl ? MPS_FP64 : MPS_FP32, st));
    T *grid = dbl ? (T *)s->grid64 : (T *)s->grid32;
    void *spec = dbl ? s->spec64 : s->spec32;
    const T *g = dbl ? (const T *)s->cs_g64 : (const T *)s->cs_g32;
    const T *hc = dbl ? (const T *)s->cs_h64 : (const T *)s->cs_h32;
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, dbl ? MPS_FP64 : MPS_FP32, &ev, st));
    const bool beside = !dbl && pair_sum_beside(ev);
    if (beside) MPS_TRY(pair_sum_fork(s, m, nrhs, st, false));
    STAGE_MARK(1);
    MPS_TRY(spread_cs<T>(m, s->n, nrhs, s->start, s->cs_base, g, s->gp, grid, st));
    STAGE_MARK(2);
    MPS_TRY(exec_plan(s, dbl ? CUFFT_D2Z : CUFFT_R2C, nrhs, grid, spec, 0, st));
    STAGE_MARK(3);
    MPS_TRY(scale_cs<T>(spec, nrhs, s->gp, hc, st));
    STAGE_MARK(4);
    MPS_TRY(exec_plan(s, dbl ? CUFFT_Z2D : CUFFT_C2R, nrhs, spec, grid, 0, st));
    STAGE_MARK(5);
    MPS_TRY(contract_cs<T>(grid, s->n, nrhs, s->start, s->cs_base, g, s->gp, out, st));
    STAGE_MARK(6);
    if (dbl)
        MPS_TRY(real_space_csr<double>(m, out, s->n, nrhs, s->row_ptr, s->p64, s->diag, s->diag_idx, s->slab, true, st));
    else if (beside)
        MPS_TRY(pair_sum_join(s, out, nrhs, st));
    else
        MPS_TRY(real_space_f32(s, m, out, nrhs, st));
    STAGE_MARK(7);
    return MPS_OK;
}

// Gradient form of the float32 operator (gradop.cu): one scalar grid per vector.

static int matvec_grad_inner(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st);

// The gradient-form contraction: staged home blocks (default), one warp per particle gathering from L2
// (MPS_GRAD_CONTRACT=warp), or the tiled partial sums on tiles of depth 4 or 8 (MPS_GRAD_CONTRACT=tiled); the
// other forms are kept for A/B timing.  The home and warp forms give bit-identical results.
enum { kGradHome = 0, kGradWarp = 1, kGradTiled = 2 };
static int grad_contract_mode(const GridParams &gp, const TileBins &tb) {
    const char *e = getenv("MPS_GRAD_CONTRACT");
    if (e && strcmp(e, "tiled") == 0 && (tb.tz == 4 || tb.tz == 8)) return kGradTiled;
    if (e && strcmp(e, "warp") == 0) return kGradWarp;
    return contract_grad_home_supported(gp) ? kGradHome : kGradWarp;
}

static int grad_contract(mps_system *s, const float *grid, int nrhs, const int32_t *start, const float *w,
                         const float *g, const GridParams &gp, TileBins &tb, double *out, cudaStream_t st) {
    const int mode = grad_contract_mode(gp, tb);
    if (mode == kGradTiled) {
        if (s->partialg_n < tb.nentries * 9) {
            if (s->partialg) MPS_CUDA_TRY(cudaFreeAsync(s->partialg, st));
            s->partialg = nullptr;
            s->partialg_n = 0;
            MPS_TRY(dalloc(&s->partialg, (size_t)tb.nentries * 9 * sizeof(float), st));
            s->partialg_n = tb.nentries * 9;
        }
        MPS_TRY(tile_bins_pentry(start, gp, tb, st));
        return contract_grad_tiled(grid, s->n, nrhs, start, w, g, gp, tb, s->partialg, out, st);
    }
    if (mode == kGradHome) {
        MPS_TRY(tile_bins_home(start, s->n, gp, tb, st));
        return contract_grad_home(grid, s->n, nrhs, start, w, g, gp, tb, out, st);
    }
    return contract_grad_warp(grid, s->n, nrhs, s->order, start, w, g, gp, out, st);
}

static int matvec_grad(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    // the gradient form exists for the dipole operator only: the others run their own float32 operator
    if (s->kind == MPS_DIPOLE_QUADRUPOLE) return matvec_quad<float>(s, m, out, nrhs, st);
    if (s->kind == MPS_POLYDISPERSE) return matvec_cs<float>(s, m, out, nrhs, st);
    if (s->inner) return matvec_grad_inner(s, m, out, nrhs, st);
    if (!s->g32 && s->w64) {
        MPS_TRY(dalloc(&s->g32, sizeof(float) * 3 * s->n * s->gp.P, st));
        MPS_TRY(grad_factors(s->x, s->n, s->gp, s->w64, s->g32, st));
    }
    bool use_tiles = false;
    MPS_TRY(ensure_tiles(s, kTileGrad32, st, &use_tiles));
    if (!use_tiles) return matvec_impl<float>(s, m, out, nrhs, st);
    MPS_TRY(ensure_grids(s, MPS_FP32, st));
    if (!s->hs32_ready) {
        std::lock_guard<std::mutex> lk(g_green_mu);
        if (!s->green->hs32) {
            float *hs = nullptr;
            MPS_TRY(dalloc_persistent(&hs, sizeof(float) * s->Gc));
            MPS_TRY(grad_scale_coef(s->gp, s->green->h64, hs, st));
            MPS_TRY(green_mark_filled(&s->green->ev_hs32, st));
            s->green->hs32 = hs;
        } else {
            MPS_CUDA_TRY(cudaStreamWaitEvent(st, s->green->ev_hs32, 0));   // filled by another system
        }
        s->hs32_ready = true;
    }
    const double vol = s->box[0] * s->box[1] * s->box[2];
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, MPS_FP32, &ev, st));
    // the pair sum runs beside the wave-space stages (pair_sum_fork / pair_sum_join)
    const bool beside = pair_sum_beside(ev);
    if (s->slab_factor != 0.0) MPS_TRY(slab_terms(m, s->n, nrhs, s->slab_factor / vol, s->slab, st));
    if (beside) MPS_TRY(pair_sum_fork(s, m, nrhs, st, false));
    STAGE_MARK(1);
    MPS_TRY(spread_grad_tiled(m, s->n, nrhs, s->start, s->w32, s->g32, s->gp, s->tbg, s->grid32, st));
    STAGE_MARK(2);
    MPS_TRY(exec_plan(s, CUFFT_R2C, nrhs, s->grid32, s->spec32, 0, st));
    STAGE_MARK(3);
    MPS_TRY(scale_cs<float>(s->spec32, nrhs, s->gp, s->green->hs32, st));
    STAGE_MARK(4);
    MPS_TRY(exec_plan(s, CUFFT_C2R, nrhs, s->spec32, s->grid32, 0, st));
    STAGE_MARK(5);
    MPS_TRY(grad_contract(s, s->grid32, nrhs, s->start, s->w32, s->g32, s->gp, s->tbg, out, st));
    STAGE_MARK(6);
    if (beside)
        MPS_TRY(pair_sum_join(s, out, nrhs, st));
    else
        MPS_TRY(real_space_f32(s, m, out, nrhs, st));
    STAGE_MARK(7);
    return MPS_OK;
}

// The gradient-form operator on the inner grid: the same stages as matvec_grad with the inner grid's geometry,
// tiles, grids, Green's coefficient and FFT plans (its tiles, weights and factors are built with the system).
// The inner grid's gradient-form scale coefficient H / |k|^2, from the process cache or computed on stream st.
static int inner_hs32(mps_system *s, cudaStream_t st) {
    InnerGrid &ig = *s->inner;
    if (ig.hs32_ready) return MPS_OK;
    std::lock_guard<std::mutex> lk(g_green_mu);
    if (!ig.green->hs32) {
        float *hs = nullptr;
        MPS_TRY(dalloc_persistent(&hs, sizeof(float) * ig.Gc));
        MPS_TRY(grad_scale_coef(ig.gp, ig.green->h64, hs, st));
        MPS_TRY(green_mark_filled(&ig.green->ev_hs32, st));
        ig.green->hs32 = hs;
    } else {
        MPS_CUDA_TRY(cudaStreamWaitEvent(st, ig.green->ev_hs32, 0));   // filled by another system
    }
    ig.hs32_ready = true;
    return MPS_OK;
}

static int matvec_grad_inner(mps_system *s, const double *m, double *out, int nrhs, cudaStream_t st) {
    InnerGrid &ig = *s->inner;
    if (!ig.grid) MPS_TRY(dalloc(&ig.grid, (size_t)s->max_rhs * ig.gp.G * sizeof(float), st));
    if (!ig.spec) MPS_TRY(dalloc(&ig.spec, (size_t)s->max_rhs * ig.Gc * 2 * sizeof(float), st));
    MPS_TRY(inner_hs32(s, st));
    const double vol = s->box[0] * s->box[1] * s->box[2];
    StageEvents *ev = nullptr;
    MPS_TRY(stage_begin(s, MPS_FP32, &ev, st));
    const bool beside = pair_sum_beside(ev);
    if (s->slab_factor != 0.0) MPS_TRY(slab_terms(m, s->n, nrhs, s->slab_factor / vol, s->slab, st));
    if (beside) MPS_TRY(pair_sum_fork(s, m, nrhs, st, false));
    STAGE_MARK(1);
    MPS_TRY(spread_grad_tiled(m, s->n, nrhs, ig.start, ig.w32, ig.g32, ig.gp, ig.tb, ig.grid, st));
    STAGE_MARK(2);
    MPS_TRY(exec_plan_gp(s, ig.gp, CUFFT_R2C, nrhs, ig.grid, ig.spec, 0, st));
    STAGE_MARK(3);
    MPS_TRY(scale_cs<float>(ig.spec, nrhs, ig.gp, ig.green->hs32, st));
    STAGE_MARK(4);
    MPS_TRY(exec_plan_gp(s, ig.gp, CUFFT_C2R, nrhs, ig.spec, ig.grid, 0, st));
    STAGE_MARK(5);
    MPS_TRY(grad_contract(s, ig.grid, nrhs, ig.start, ig.w32, ig.g32, ig.gp, ig.tb, out, st));
    STAGE_MARK(6);
    if (beside)
        MPS_TRY(pair_sum_join(s, out, nrhs, st));
    else
        MPS_TRY(real_space_f32(s, m, out, nrhs, st));
    STAGE_MARK(7);
    return MPS_OK;
}

static int matvec_real(mps_system *s, const double *m, double *out, int nrhs, int precision, cudaStream_t st) {
    if (precision == MPS_FP32_GRAD) return matvec_grad(s, m, out, nrhs, st);
    if (precision == MPS_DF) {
        if (df_usable(s)) return matvec_df(s, m, out, nrhs, st);
        precision = MPS_FP64;
    }
    if (s->kind == MPS_POLYDISPERSE)
        return precision == MPS_FP64 ? matvec_cs<double>(s, m, out, nrhs, st) : matvec_cs<float>(s, m, out, nrhs, st);
    if (s->kind == MPS_DIPOLE_QUADRUPOLE)
        return precision == MPS_FP64 ? matvec_quad<double>(s, m, out, nrhs, st)
                                     : matvec_quad<float>(s, m, out, nrhs, st);
    return precision == MPS_FP64 ? matvec_impl<double>(s, m, out, nrhs, st) : matvec_impl<float>(s, m, out, nrhs, st);
}

// (Re m, Im m) per particle -> the 2 nc real vectors, and back with the imaginary
// diagonal's coupling: out_re = Mu + Re(D) u - Im(D) v, out_im = Mv + Re(D) v + Im(D) u
// (Mu, Mv from the real operator, which already adds Re(D)).
__global__ void k_cplx_split(const double *__restrict__ m6, int nc, int64_t n, double *__restrict__ cx) {
    const int64_t tot = (int64_t)nc * n * 3;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = t / (n * 3), a = (t / 3) % n;
        const int c = (int)(t % 3);
        const double *src = m6 + (q * n + a) * 6;
        cx[t] = src[c];
        cx[tot + t] = src[3 + c];
    }
}

__global__ void k_cplx_join(const double *__restrict__ cx, const double *__restrict__ mx, const double *__restrict__ di,
                            const int32_t *__restrict__ didx, int nc, int64_t n, double *__restrict__ out6) {
    const int64_t tot = (int64_t)nc * n * 3;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = t / (n * 3), a = (t / 3) % n;
        const int c = (int)(t % 3);
        const double dim = di[(int64_t)didx[q] * n + a];
        const double u = cx[t], v = cx[tot + t];
        double *dst = out6 + (q * n + a) * 6;
        dst[c] = mx[t] - dim * v;
        dst[3 + c] = mx[tot + t] + dim * u;
    }
}

static int matvec_cplx(mps_system *s, const double *m6, double *out6, int nc, int precision, cudaStream_t st) {
    const size_t bytes = sizeof(double) * 2 * (size_t)s->max_rhs_c * s->n * 3;
    if (!s->cx_in) MPS_TRY(dalloc(&s->cx_in, bytes, st));
    if (!s->cx_out) MPS_TRY(dalloc(&s->cx_out, bytes, st));
    const int64_t tot = (int64_t)nc * s->n * 3;
    k_cplx_split<<<grid_for(tot, 256), 256, 0, st>>>(m6, nc, s->n, s->cx_in);
    count_launch();
    MPS_CUDA_TRY(cudaGetLastError());
    MPS_TRY(matvec_real(s, s->cx_in, s->cx_out, 2 * nc, precision, st));
    k_cplx_join<<<grid_for(tot, 256), 256, 0, st>>>(s->cx_in, s->cx_out, s->diag_im, s->diag_idx, nc, s->n, out6);
    count_launch();
    MPS_CUDA_TRY(cudaGetLastError());
    return MPS_OK;
}

static int matvec_any(mps_system *s, const double *m, double *out, int nrhs, int precision, cudaStream_t st) {
    const int rc =
        s->cplx ? matvec_cplx(s, m, out, nrhs, precision, st) : matvec_real(s, m, out, nrhs, precision, st);
    if (rc == MPS_OK && !matvec_seen(s, precision, nrhs)) s->mv_seen.push_back({precision, nrhs});
    return rc;
}

// ---------------------------------------------------------------------------
// Krylov kernels (float64).  Vectors of length n3 = ndof n; nrhs independent
// systems stacked with stride n3 (vectors) / ld (bases).
// ---------------------------------------------------------------------------
constexpr int kDotThreads = 256;
constexpr int kDotItems = 8;
constexpr int kDotChunk = kDotThreads * kDotItems;
constexpr int kMaxCols = 64;

// partial[r][blk][c] = sum over the block's rows of V_r[c][i] * w_r[i]; the last
// block of each system to finish (ticket counter, threadfence pattern) sums the
// partials in block order and writes out[r][c]: one launch, fixed summation order.
// With jd non-null the column count is ncols + *jd (the Arnoldi step held on the
// device by a captured graph).
__global__ void __launch_bounds__(kDotThreads) k_multidot(const double *__restrict__ V, int64_t ldv, int64_t vstride,
                                                          int ncols, const double *__restrict__ w, int64_t wstride,
                                                          int64_t n3, double *__restrict__ partial, int nblk,
                                                          unsigned *__restrict__ tickets, double *__restrict__ out,
                                                          int64_t ostride, const int32_t *__restrict__ jd) {
    __shared__ double red[kDotThreads / 32][kMaxCols];
    __shared__ bool last;
    const int r = blockIdx.y;
    if (jd) ncols += *jd;   // graph form: the column count follows the device step counter
    const double *Vr = V + r * vstride;
    const double *wr = w + r * wstride;
    const int64_t i0 = (int64_t)blockIdx.x * kDotChunk;
    double wv[kDotItems];
#pragma unroll
    for (int k = 0; k < kDotItems; ++k) {
        int64_t i = i0 + (int64_t)k * kDotThreads + threadIdx.x;
        wv[k] = i < n3 ? wr[i] : 0.0;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // columns interleaved in fours: the loads of the next columns overlap this column's shuffle reduction
#pragma unroll 4
    for (int c = 0; c < ncols; ++c) {
        const double *Vc = Vr + (int64_t)c * ldv;
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < kDotItems; ++k) {
            int64_t i = i0 + (int64_t)k * kDotThreads + threadIdx.x;
            if (i < n3) acc += Vc[i] * wv[k];
        }
        acc = warp_sum(acc);
        if (lane == 0) red[wid][c] = acc;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kDotThreads / 32; ++q) s += red[q][c];
        partial[((int64_t)r * nblk + blockIdx.x) * kMaxCols + c] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&tickets[r], 1u) == (unsigned)(nblk - 1);
    __syncthreads();
    if (!last) return;
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += __ldcg(partial + ((int64_t)r * nblk + b) * kMaxCols + c);
        out[(int64_t)r * ostride + c] = s;
    }
    if (threadIdx.x == 0) tickets[r] = 0u;
}

// w_r[i] -= sum_c V_r[c][i] * h_r[c]
__global__ void k_sub_basis(const double *__restrict__ V, int64_t ldv, int64_t vstride, int ncols,
                            const double *__restrict__ h, int64_t hstride, double *__restrict__ w, int64_t wstride,
                            int64_t n3, const int32_t *__restrict__ jd = nullptr) {
    __shared__ double hs[kMaxCols];
    const int r = blockIdx.y;
    if (jd) ncols += *jd;
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) hs[c] = h[(int64_t)r * hstride + c];
    __syncthreads();
    const double *Vr = V + r * vstride;
    double *wr = w + r * wstride;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = wr[i];
        for (int c = 0; c < ncols; ++c) acc -= Vr[(int64_t)c * ldv + i] * hs[c];
        wr[i] = acc;
    }
}

// x_r[i] += sum_c V_r[c][i] * y_r[c] for c < k_r
__global__ void k_add_basis(const double *__restrict__ V, int64_t ldv, int64_t vstride, const double *__restrict__ y,
                            int64_t ystride, const int32_t *__restrict__ kcount, double *__restrict__ x,
                            int64_t xstride, int64_t n3) {
    __shared__ double ys[kMaxCols];
    const int r = blockIdx.y;
    const int k = kcount[r];
    for (int c = threadIdx.x; c < k; c += blockDim.x) ys[c] = y[(int64_t)r * ystride + c];
    __syncthreads();
    const double *Vr = V + r * vstride;
    double *xr = x + r * xstride;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = xr[i];
        for (int c = 0; c < k; ++c) acc += Vr[(int64_t)c * ldv + i] * ys[c];
        xr[i] = acc;
    }
}

// out = a - b (per system)
__global__ void k_sub(const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ out,
                      int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

// dst_r = src_r * scale_r (scale_r = 1/norm; zero norm -> zero vector)
__global__ void k_scale_vec(const double *__restrict__ src, int64_t sstride, double *__restrict__ dst,
                            int64_t dstride, const double *__restrict__ nrm, int64_t nstride, int64_t n3) {
    const int r = blockIdx.y;
    const double v = nrm[r * nstride];
    const double f = v != 0.0 ? 1.0 / v : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x)
        dst[r * dstride + i] = src[r * sstride + i] * f;
}

__global__ void k_sqrt_copy(const double *__restrict__ a, double *__restrict__ b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = sqrt(a[i]);
}

// y += x
__global__ void k_axpy1(const double *__restrict__ x, double *__restrict__ y, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        y[i] += x[i];
}

// out_r = sum_{c <= kcount[r] + extra - 1} coef_r[c] V_r[c]   (overwrites)
__global__ void k_combine_basis(const double *__restrict__ V, int64_t ldv, int64_t vstride,
                                const double *__restrict__ coef, int64_t cstride, const int32_t *__restrict__ kcount,
                                int extra, double *__restrict__ out, int64_t ostride, int64_t n3) {
    __shared__ double cs_[kMaxCols + 1];
    const int r = blockIdx.y;
    const int k = kcount[r] + extra;
    for (int c = threadIdx.x; c < k; c += blockDim.x) cs_[c] = coef[(int64_t)r * cstride + c];
    __syncthreads();
    const double *Vr = V + r * vstride;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int c = 0; c < k; ++c) acc += Vr[(int64_t)c * ldv + i] * cs_[c];
        out[r * ostride + i] = acc;
    }
}

struct GmresState {
    double *H;      // [r][(restart+1) * restart], column j at offset j*(restart+1)
    double *cs, *sn;  // [r][restart]
    double *g;      // [r][restart+1]
    double *h1, *h2;  // [r][kMaxCols]
    double *nrm2;   // [r]
    double *beta;   // [r]
    double *bnorm;  // [r]
    double *res;    // [r] residual estimate / true relres
    int32_t *kcount;  // [r] columns of the cycle's best iterate so far (strictly smallest residual estimate)
    int32_t *kfull;   // [r] columns built in the cycle
    double *y;      // [r][restart]
};

// Start of a cycle: beta = sqrt(nrm2), g = [beta, 0...], relres = beta / bnorm.
__global__ void k_cycle_start(GmresState st, int restart, int nrhs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrhs) return;
    const double b = sqrt(st.nrm2[r]);
    st.beta[r] = b;
    for (int i = 0; i <= restart; ++i) st.g[r * (restart + 1) + i] = 0.0;
    st.g[r * (restart + 1)] = b;
    st.res[r] = st.bnorm[r] > 0 ? b / st.bnorm[r] : 0.0;
    st.kcount[r] = 0;
    st.kfull[r] = 0;
}

// Arnoldi column j: H[:,j] = h1 + h2, H[j+1,j] = ||w||, then Givens rotations.
__global__ void k_arnoldi_givens(GmresState st, int restart, int j, int nrhs, const int32_t *__restrict__ frozen,
                                 const int32_t *__restrict__ jd = nullptr) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrhs) return;
    if (frozen[r]) return;
    if (jd) j = *jd;
    const int ld = restart + 1;
    double *Hc = st.H + (int64_t)r * ld * restart + (int64_t)j * ld;
    for (int i = 0; i <= j; ++i) Hc[i] = st.h1[r * kMaxCols + i] + st.h2[r * kMaxCols + i];
    const double wn = sqrt(st.nrm2[r]);
    st.nrm2[r] = wn;  // the following normalisation of w divides by the norm
    Hc[j + 1] = wn;
    double *cs = st.cs + r * restart, *sn = st.sn + r * restart, *g = st.g + r * ld;
    for (int i = 0; i < j; ++i) {
        const double t = cs[i] * Hc[i] + sn[i] * Hc[i + 1];
        Hc[i + 1] = -sn[i] * Hc[i] + cs[i] * Hc[i + 1];
        Hc[i] = t;
    }
    const double a = Hc[j], b = Hc[j + 1];
    const double den = hypot(a, b);
    if (den == 0.0) {
        cs[j] = 1.0;
        sn[j] = 0.0;
    } else {
        cs[j] = a / den;
        sn[j] = b / den;
    }
    Hc[j] = cs[j] * a + sn[j] * b;
    Hc[j + 1] = 0.0;
    const double gj = g[j];
    g[j] = cs[j] * gj;
    g[j + 1] = -sn[j] * gj;
    // the cycle keeps its best iterate: the least-squares solution over the first k columns, k where the
    // residual estimate last decreased strictly (EW/capacitance.py:174-191); the estimate never rises in exact
    // arithmetic, so k = j + 1 unless it stagnates
    const double est = st.bnorm[r] > 0 ? fabs(g[j + 1]) / st.bnorm[r] : 0.0;
    st.kfull[r] = j + 1;
    if (est < st.res[r]) {
        st.res[r] = est;
        st.kcount[r] = j + 1;
    }
}

// Coefficients u (length k+1) of the least-squares residual b - A x_k = V_{k+1} u:
// u = G_0^T ... G_{k-1}^T (0, ..., 0, g_k), i.e. the Arnoldi relation, no matvec.
__global__ void k_ls_residual_coeffs(GmresState st, int restart, int nrhs, double *__restrict__ u, int ustride) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrhs) return;
    const int ld = restart + 1;
    const int k = st.kcount[r];
    double *ur = u + (int64_t)r * ustride;
    for (int i = 0; i <= k; ++i) ur[i] = 0.0;
    ur[k] = st.g[r * ld + k];
    const double *cs = st.cs + r * restart, *sn = st.sn + r * restart;
    for (int i = k - 1; i >= 0; --i) {
        const double a = ur[i], b = ur[i + 1];
        ur[i] = cs[i] * a - sn[i] * b;
        ur[i + 1] = sn[i] * a + cs[i] * b;
    }
}

// Back substitution H[:k,:k] y = g[:k].
__global__ void k_backsolve(GmresState st, int restart, int nrhs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrhs) return;
    const int ld = restart + 1;
    int k = st.kcount[r];
    if (k == 0) {   // no step improved on the cycle's start: the full cycle's least-squares solution, as the reference
        k = st.kfull[r];
        st.kcount[r] = k;
    }
    const double *H = st.H + (int64_t)r * ld * restart;
    const double *g = st.g + r * ld;
    double *y = st.y + r * restart;
    for (int i = k - 1; i >= 0; --i) {
        double v = g[i];
        for (int c = i + 1; c < k; ++c) v -= H[(int64_t)c * ld + i] * y[c];
        const double d = H[(int64_t)i * ld + i];
        y[i] = d != 0.0 ? v / d : 0.0;
    }
}

static char *carve_ws(char *&p, size_t bytes) {
    uintptr_t u = ((uintptr_t)p + 255) & ~(uintptr_t)255;
    p = (char *)(u + bytes);
    return (char *)u;
}

// Dots of the first ncols basis vectors with w, for every system.  The scratch
// holds nrhs * nblk * kMaxCols partials followed by nrhs zeroed tickets
// (multidot_bytes / multidot_init).
static int multidot(const double *V, int64_t ldv, int64_t vstride, int ncols, const double *w, int64_t wstride,
                    int64_t n3, int nrhs, double *partial, double *out, int64_t ostride, cudaStream_t s,
                    const int32_t *jd = nullptr) {
    const int nblk = (int)((n3 + kDotChunk - 1) / kDotChunk);
    unsigned *tickets = (unsigned *)(partial + (size_t)nrhs * nblk * kMaxCols);
    dim3 g(nblk, nrhs);
    k_multidot<<<g, kDotThreads, 0, s>>>(V, ldv, vstride, ncols, w, wstride, n3, partial, nblk, tickets, out, ostride,
                                         jd);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

static size_t multidot_bytes(int64_t n3, int nrhs) {
    const int nblk = (int)((n3 + kDotChunk - 1) / kDotChunk);
    return sizeof(double) * (size_t)nrhs * nblk * kMaxCols + sizeof(unsigned) * (size_t)(nrhs + 2);
}

static int multidot_init(double *partial, int64_t n3, int nrhs, cudaStream_t s) {
    const int nblk = (int)((n3 + kDotChunk - 1) / kDotChunk);
    MPS_CUDA_TRY(cudaMemsetAsync(partial + (size_t)nrhs * nblk * kMaxCols, 0, sizeof(unsigned) * (size_t)nrhs, s));
    return MPS_OK;
}

// ---------------------------------------------------------------------------
// Arnoldi steps as one CUDA graph launch.  A while-conditional node repeats the
// step body -- matvec of vin, Gram-Schmidt against V[0..j], Givens update, the
// next basis vector (also copied to vin), loop control -- with the step index j
// held on the device (jd).  The loop control freezes the systems whose residual
// estimate reached the tolerance and ends the loop when all are frozen or j
// reaches restart: j grows by one per execution, so the loop ends after at most
// restart - j0 steps.  The host reads the estimates once per graph launch.
// ---------------------------------------------------------------------------

// V[j+1]_r = w_r / nrm_r (j = *jd; zero norm -> zero vector), copied to vin as well.
__global__ void k_next_basis(const double *__restrict__ w, double *__restrict__ V, int64_t ldv,
                             const int32_t *__restrict__ jd, const double *__restrict__ nrm, double *__restrict__ vin,
                             int64_t n3) {
    const int r = blockIdx.y;
    const double v = nrm[r];
    const double f = v != 0.0 ? 1.0 / v : 0.0;
    double *dst = V + (int64_t)(*jd + 1) * ldv + (int64_t)r * n3;
    double *d2 = vin + (int64_t)r * n3;
    const double *src = w + (int64_t)r * n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = src[i] * f;
        dst[i] = x;
        d2[i] = x;
    }
}

// End of a step: freeze the systems that reached the tolerance, advance j, and
// repeat the body while some system is active and j < restart.
__global__ void k_loop_ctrl(const double *__restrict__ res, int32_t *__restrict__ frozen,
                            const double *__restrict__ tol, int nrhs, int32_t *__restrict__ jd, int restart,
                            cudaGraphConditionalHandle h) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const double t = *tol;
    bool active = false;
    for (int r = 0; r < nrhs; ++r) {
        if (!frozen[r] && res[r] <= t) frozen[r] = 1;
        active = active || !frozen[r];
    }
    const int j = *jd + 1;
    *jd = j;
    cudaGraphSetConditional(h, (active && j < restart) ? 1u : 0u);
}

__global__ void k_graph_enter(int32_t *__restrict__ jd, int j0, double *__restrict__ tol_d, double tol) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *jd = j0;
        *tol_d = tol;
    }
}

// Workspace of gmres_core (the graph form adds vin, jd and the device tolerance).
struct GmresWs {
    double *V, *w, *vin, *partial, *u, *tol_d;
    int32_t *frozen, *jd;
    GmresState S;
};

static size_t gmres_ws_bytes(int64_t n3, int nrhs, int restart) {
    const int ld = restart + 1;
    const int64_t ldv = (int64_t)nrhs * n3;
    size_t bytes = 0;
    bytes += 256 + sizeof(double) * (size_t)ld * ldv;                 // V
    bytes += 2 * (256 + sizeof(double) * (size_t)ldv);                // w vin
    bytes += 256 + sizeof(double) * (size_t)nrhs * ld * restart;      // H
    bytes += 2 * (256 + sizeof(double) * (size_t)nrhs * restart);     // cs sn
    bytes += 256 + sizeof(double) * (size_t)nrhs * ld;                // g
    bytes += 2 * (256 + sizeof(double) * (size_t)nrhs * kMaxCols);    // h1 h2
    bytes += 4 * (256 + sizeof(double) * (size_t)nrhs);               // nrm2 beta bnorm res
    bytes += 3 * (256 + sizeof(int32_t) * (size_t)nrhs);              // kcount kfull frozen
    bytes += 256 + sizeof(double) * (size_t)nrhs * restart;           // y
    bytes += 256 + multidot_bytes(n3, nrhs);                          // partial + tickets
    bytes += 256 + sizeof(double) * (size_t)nrhs * (kMaxCols + 1);    // u
    bytes += 2 * (256 + sizeof(double));                              // jd tol_d
    return bytes;
}

static GmresWs gmres_ws_carve(char *base, int64_t n3, int nrhs, int restart) {
    const int ld = restart + 1;
    const int64_t ldv = (int64_t)nrhs * n3;
    char *p = base;
    GmresWs g;
    g.V = (double *)carve_ws(p, sizeof(double) * (size_t)ld * ldv);
    g.w = (double *)carve_ws(p, sizeof(double) * (size_t)ldv);
    g.vin = (double *)carve_ws(p, sizeof(double) * (size_t)ldv);
    g.S.H = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * ld * restart);
    g.S.cs = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * restart);
    g.S.sn = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * restart);
    g.S.g = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * ld);
    g.S.h1 = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * kMaxCols);
    g.S.h2 = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * kMaxCols);
    g.S.nrm2 = (double *)carve_ws(p, sizeof(double) * nrhs);
    g.S.beta = (double *)carve_ws(p, sizeof(double) * nrhs);
    g.S.bnorm = (double *)carve_ws(p, sizeof(double) * nrhs);
    g.S.res = (double *)carve_ws(p, sizeof(double) * nrhs);
    g.S.kcount = (int32_t *)carve_ws(p, sizeof(int32_t) * nrhs);
    g.S.kfull = (int32_t *)carve_ws(p, sizeof(int32_t) * nrhs);
    g.frozen = (int32_t *)carve_ws(p, sizeof(int32_t) * nrhs);
    g.S.y = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * restart);
    g.partial = (double *)carve_ws(p, multidot_bytes(n3, nrhs));
    g.u = (double *)carve_ws(p, sizeof(double) * (size_t)nrhs * (kMaxCols + 1));
    g.jd = (int32_t *)carve_ws(p, sizeof(double));
    g.tol_d = (double *)carve_ws(p, sizeof(double));
    return g;
}

// Graph form on unless MPS_GMRES_GRAPH=0 (host-driven steps, kept for A/B timing); never while stage
// profiling records events inside the matvecs.
static bool graphs_enabled(const mps_system *s) {
    if (s->profile) return false;
    const char *v = getenv("MPS_GMRES_GRAPH");
    return !(v && v[0] == '0');
}

static int matvec_any(mps_system *s, const double *m, double *out, int nrhs, int precision, cudaStream_t st);

// Captures the step body for g's configuration on the system's capture stream
// and instantiates it.  A capture the runtime refuses (or any error inside it)
// marks g failed and returns MPS_OK: the caller keeps the host-driven steps.
static int arnoldi_graph_build(mps_system *s, ArnoldiGraph &g, const GmresWs &W, int64_t n3) {
    const int nrhs = g.nrhs, restart = g.restart;
    const int64_t ldv = (int64_t)nrhs * n3;
    if (!s->cap) MPS_CUDA_TRY(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    MPS_CUDA_TRY(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};   // the rest zero
    cudaGraphNode_t node;
    cudaError_t ce = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    if (ce == cudaSuccess) {
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        ce = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    }
    if (ce != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(graph);
        g.failed = true;
        return MPS_OK;
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs = s->cap;
    const dim3 vgrid(grid_for(n3, 256, 152 * 8), nrhs);
    capture_count_begin();
    ce = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    int e = ce == cudaSuccess ? MPS_OK : MPS_CUDA_ERR;
    if (e == MPS_OK) {
        auto launched = [&]() { return cudaGetLastError() == cudaSuccess ? MPS_OK : MPS_CUDA_ERR; };
        e = matvec_any(s, W.vin, W.w, nrhs, g.precision, cs);
        if (e == MPS_OK) e = multidot(W.V, ldv, n3, 1, W.w, n3, n3, nrhs, W.partial, W.S.h1, kMaxCols, cs, W.jd);
        if (e == MPS_OK) {
            k_sub_basis<<<vgrid, 256, 0, cs>>>(W.V, ldv, n3, 1, W.S.h1, kMaxCols, W.w, n3, n3, W.jd);
            count_launch();
            e = launched();
        }
        if (e == MPS_OK && g.reorth) {
            e = multidot(W.V, ldv, n3, 1, W.w, n3, n3, nrhs, W.partial, W.S.h2, kMaxCols, cs, W.jd);
            if (e == MPS_OK) {
                k_sub_basis<<<vgrid, 256, 0, cs>>>(W.V, ldv, n3, 1, W.S.h2, kMaxCols, W.w, n3, n3, W.jd);
                count_launch();
                e = launched();
            }
        }
        if (e == MPS_OK) e = multidot(W.w, n3, n3, 1, W.w, n3, n3, nrhs, W.partial, W.S.nrm2, 1, cs);
        if (e == MPS_OK) {
            k_arnoldi_givens<<<(nrhs + 31) / 32, 32, 0, cs>>>(W.S, restart, 0, nrhs, W.frozen, W.jd);
            count_launch();
            e = launched();
        }
        if (e == MPS_OK) {
            k_next_basis<<<vgrid, 256, 0, cs>>>(W.w, W.V, ldv, W.jd, W.S.nrm2, W.vin, n3);
            count_launch();
            e = launched();
        }
        if (e == MPS_OK) {
            k_loop_ctrl<<<1, 32, 0, cs>>>(W.S.res, W.frozen, W.tol_d, nrhs, W.jd, restart, h);
            count_launch();
            e = launched();
        }
        cudaGraph_t out = nullptr;
        ce = cudaStreamEndCapture(cs, &out);
        if (ce != cudaSuccess) e = MPS_CUDA_ERR;
    }
    const long long per_step = capture_count_end();
    cudaGraphExec_t exec = nullptr;
    if (e == MPS_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) e = MPS_CUDA_ERR;
    cudaGraphDestroy(graph);
    if (e != MPS_OK) {
        cudaGetLastError();   // a refused capture leaves no sticky error; clear the recorded one
        g.failed = true;
        return MPS_OK;
    }
    g.exec = exec;
    g.body_launches = per_step;
    return MPS_OK;
}

// Core restarted GMRES (Arnoldi with classical Gram-Schmidt applied twice, Givens
// rotations, all float64) for nrhs systems with batched matvecs of the given
// precision.  x holds the initial guess on entry and the solution on exit.
// Basis layout V[j][r][i]: basis vector j of every system is one contiguous
// nrhs x n3 block, which is exactly the batched matvec's input.
struct GmresFlags {
    bool zero_guess = false;   // x is zero on entry: the first residual is b itself (no matvec)
    bool final_check = true;   // end with a true residual b - A x (one more matvec)
    bool ls_restart = false;   // restart cycles start from the least-squares residual (Arnoldi relation)
    double *r_out = nullptr;   // optional: final residual vectors (nrhs x n3)
    bool reorth = true;        // classical Gram-Schmidt twice (false: once; enough for the inner solves of the
                               // mixed refinement, whose relative targets are 1e-4..0.5 in float64 arithmetic)
};

static int gmres_core(mps_system *s, const double *b, double *x, int nrhs, double tol, int restart, int maxit,
                      int precision, int *conv, double *relres_out, int *cycles_out, int *mv_count,
                      cudaStream_t st, GmresFlags fl = GmresFlags()) {
    const int64_t n3 = (int64_t)s->ndof * s->n;
    const int64_t ldv = (int64_t)nrhs * n3;
    // The graph form keeps one persistent workspace per configuration (its kernels hold the addresses);
    // otherwise the workspace lives for this call.
    ArnoldiGraph *ag = nullptr;
    if (graphs_enabled(s)) {
        for (auto &g : s->graphs)
            if (g.precision == precision && g.nrhs == nrhs && g.restart == restart && g.reorth == fl.reorth) ag = &g;
        if (!ag) {
            ArnoldiGraph g;
            g.precision = precision;
            g.nrhs = nrhs;
            g.restart = restart;
            g.reorth = fl.reorth;
            g.ws_bytes = gmres_ws_bytes(n3, nrhs, restart);
            MPS_CUDA_TRY(cudaMallocAsync((void **)&g.ws, g.ws_bytes, st));
            s->graphs.push_back(g);
            ag = &s->graphs.back();
        }
        if (ag->failed) ag = nullptr;
    }
    char *base = nullptr;
    if (ag) {
        base = ag->ws;
    } else {
        MPS_CUDA_TRY(cudaMallocAsync((void **)&base, gmres_ws_bytes(n3, nrhs, restart), st));
    }
    const GmresWs W = gmres_ws_carve(ag ? ag->ws : base, n3, nrhs, restart);
    double *V = W.V;
    double *w = W.w;
    GmresState S = W.S;
    int32_t *frozen = W.frozen;
    double *partial = W.partial;
    double *u = W.u;
    {
        int e = multidot_init(partial, n3, nrhs, st);
        if (e == MPS_OK && !fl.reorth &&
            cudaMemsetAsync(S.h2, 0, sizeof(double) * (size_t)nrhs * kMaxCols, st) != cudaSuccess)
            e = MPS_CUDA_ERR;
        if (e) {
            if (!ag) cudaFreeAsync(base, st);
            return e;
        }
    }

    double *hres = s->host_scr;         // pinned (nrhs)
    int32_t *hfrozen = s->host_frozen;  // pinned (nrhs)
    for (int r = 0; r < nrhs; ++r) hfrozen[r] = 0;
    int rc = MPS_OK;
    const dim3 vgrid(grid_for(n3, 256, 152 * 8), nrhs);
    int cyc = 0;
    auto release = [&]() {
        if (!ag) cudaFreeAsync(base, st);
    };
    auto fail = [&](int code) {
        release();
        return code;
    };
#define GM_TRY(expr)                       \
    do {                                   \
        int _r = (expr);                   \
        if (_r != MPS_OK) return fail(_r); \
    } while (0)
#define GM_LAUNCH()                     \
    do {                                \
        count_launch();                 \
        GM_CUDA(cudaGetLastError());    \
    } while (0)
#define GM_CUDA(expr)                                      \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) {                           \
            set_last_error(_e, #expr, __FILE__, __LINE__); \
            return fail(MPS_CUDA_ERR);                     \
        }                                                  \
    } while (0)

    // ||b|| per system
    GM_TRY(multidot(b, n3, n3, 1, b, n3, n3, nrhs, partial, S.nrm2, 1, st));
    k_sqrt_copy<<<(nrhs + 31) / 32, 32, 0, st>>>(S.nrm2, S.bnorm, nrhs);
    GM_LAUNCH();
    for (int r = 0; r < nrhs; ++r) conv[r] = 0;
    bool resid_ready = false;     // V[0] already holds b - A x (unnormalised)
    bool at_start_exit = false;   // left the loop at a cycle start: V[0] is the residual
    bool w_is_resid = false;      // w holds the least-squares residual of the last cycle
    for (cyc = 0; cyc < maxit; ++cyc) {
        // r0 = b - A x  -> V[0] (unnormalised)
        if (!resid_ready) {
            if (cyc == 0 && fl.zero_guess) {
                GM_CUDA(cudaMemcpyAsync(V, b, sizeof(double) * ldv, cudaMemcpyDeviceToDevice, st));
            } else {
                GM_TRY(matvec_any(s, x, w, nrhs, precision, st));
                ++*mv_count;
                k_sub<<<grid_for(ldv, 256), 256, 0, st>>>(b, w, V, ldv);
                GM_LAUNCH();
            }
        }
        resid_ready = false;
        w_is_resid = false;
        GM_TRY(multidot(V, ldv, n3, 1, V, n3, n3, nrhs, partial, S.nrm2, 1, st));
        k_cycle_start<<<(nrhs + 31) / 32, 32, 0, st>>>(S, restart, nrhs);
        GM_LAUNCH();
        GM_CUDA(cudaMemcpyAsync(hres, S.res, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        // The step graph is captured and instantiated here, on the host, while the GPU still works through the
        // residual's matvec and norms queued above, rather than at the first step after the wait (GPU idle).
        // (19.22 against 19.27 ms for the mixed step at the bench workload)
        if (ag && !ag->failed && !ag->exec && matvec_seen(s, precision, nrhs)) GM_TRY(arnoldi_graph_build(s, *ag, W, n3));
        GM_CUDA(cudaStreamSynchronize(st));
        bool all = true;
        for (int r = 0; r < nrhs; ++r) {
            relres_out[r] = hres[r];
            conv[r] = hres[r] <= tol;
            hfrozen[r] = conv[r];
            all = all && conv[r];
        }
        if (all) {
            at_start_exit = true;
            break;
        }
        GM_CUDA(cudaMemcpyAsync(frozen, hfrozen, sizeof(int32_t) * nrhs, cudaMemcpyHostToDevice, st));
        k_scale_vec<<<vgrid, 256, 0, st>>>(V, n3, V, n3, S.beta, 1, n3);
        GM_LAUNCH();
        // With a float32 operator (a matvec of about a millisecond), step j + 1's matvec is queued before the
        // host waits for step j's residual estimates whenever their trend says step j cannot finish every
        // system: the estimate after step j, extrapolated from the last two, is above 2 tol for some active
        // system.  The wait then overlaps that matvec instead of leaving the GPU idle; a wrong guess costs one
        // discarded matvec (w is rewritten before it is read again).
        const bool may_speculate = !ag && (precision == MPS_FP32 || precision == MPS_FP32_GRAD);
        std::vector<double> hlast(hres, hres + nrhs), hprev(nrhs, -1.0);
        auto likely_continues = [&]() {
            for (int r = 0; r < nrhs; ++r) {
                if (hfrozen[r]) continue;
                const double ratio = hprev[r] > 0.0 ? std::min(1.0, hlast[r] / hprev[r]) : 0.5;
                if (hlast[r] * ratio > 2.0 * tol) return true;
            }
            return false;
        };
        bool queued = false;   // step j's matvec already queued into w
        for (int j = 0; j < restart; ++j) {
            // graph form: the remaining steps of the cycle in one launch, once a matvec of this precision and
            // batch width has run outside a capture (every lazily built buffer and FFT plan exists)
            if (ag && !ag->failed && !queued && (ag->exec || matvec_seen(s, precision, nrhs))) {
                if (!ag->exec) GM_TRY(arnoldi_graph_build(s, *ag, W, n3));
                if (ag->exec) {
                    GM_CUDA(cudaMemcpyAsync(W.vin, V + (int64_t)j * ldv, sizeof(double) * ldv,
                                            cudaMemcpyDeviceToDevice, st));
                    k_graph_enter<<<1, 32, 0, st>>>(W.jd, j, W.tol_d, tol);
                    GM_LAUNCH();
                    GM_CUDA(cudaGraphLaunch(ag->exec, st));
                    if (!s->ev_graph) GM_CUDA(cudaEventCreateWithFlags(&s->ev_graph, cudaEventDisableTiming));
                    GM_CUDA(cudaEventRecord(s->ev_graph, st));
                    GM_CUDA(cudaMemcpyAsync(hres, S.res, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
                    GM_CUDA(cudaMemcpyAsync(hfrozen, frozen, sizeof(int32_t) * nrhs, cudaMemcpyDeviceToHost, st));
                    GM_CUDA(cudaMemcpyAsync(s->host_step, W.jd, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
                    GM_CUDA(cudaStreamSynchronize(st));
                    const int steps = *s->host_step - j;
                    *mv_count += steps;
                    add_launches(ag->body_launches * steps);
                    break;
                }
            }
            if (!queued) {
                GM_TRY(matvec_any(s, V + (int64_t)j * ldv, w, nrhs, precision, st));
                ++*mv_count;
            }
            queued = false;
            // classical Gram-Schmidt, twice (once for the inner solves of the mixed refinement)
            GM_TRY(multidot(V, ldv, n3, j + 1, w, n3, n3, nrhs, partial, S.h1, kMaxCols, st));
            k_sub_basis<<<vgrid, 256, 0, st>>>(V, ldv, n3, j + 1, S.h1, kMaxCols, w, n3, n3);
            GM_LAUNCH();
            if (fl.reorth) {
                GM_TRY(multidot(V, ldv, n3, j + 1, w, n3, n3, nrhs, partial, S.h2, kMaxCols, st));
                k_sub_basis<<<vgrid, 256, 0, st>>>(V, ldv, n3, j + 1, S.h2, kMaxCols, w, n3, n3);
                GM_LAUNCH();
            }
            GM_TRY(multidot(w, n3, n3, 1, w, n3, n3, nrhs, partial, S.nrm2, 1, st));
            k_arnoldi_givens<<<(nrhs + 31) / 32, 32, 0, st>>>(S, restart, j, nrhs, frozen);
            GM_LAUNCH();
            k_scale_vec<<<vgrid, 256, 0, st>>>(w, n3, V + (int64_t)(j + 1) * ldv, n3, S.nrm2, 1, n3);
            GM_LAUNCH();
            GM_CUDA(cudaMemcpyAsync(hres, S.res, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
            if (may_speculate && j + 1 < restart && likely_continues()) {
                if (!s->ev_res) GM_CUDA(cudaEventCreateWithFlags(&s->ev_res, cudaEventDisableTiming));
                GM_CUDA(cudaEventRecord(s->ev_res, st));
                GM_TRY(matvec_any(s, V + (int64_t)(j + 1) * ldv, w, nrhs, precision, st));
                ++*mv_count;
                queued = true;
                GM_CUDA(cudaEventSynchronize(s->ev_res));
            } else {
                GM_CUDA(cudaStreamSynchronize(st));
            }
            for (int r = 0; r < nrhs; ++r) {
                hprev[r] = hlast[r];
                hlast[r] = hres[r];
            }
            bool done = true, changed = false;
            for (int r = 0; r < nrhs; ++r) {
                if (!hfrozen[r] && hres[r] <= tol) {
                    hfrozen[r] = 1;
                    changed = true;
                }
                done = done && hfrozen[r];
            }
            if (done) break;
            if (changed)
                GM_CUDA(cudaMemcpyAsync(frozen, hfrozen, sizeof(int32_t) * nrhs, cudaMemcpyHostToDevice, st));
        }
        k_backsolve<<<(nrhs + 31) / 32, 32, 0, st>>>(S, restart, nrhs);
        GM_LAUNCH();
        k_add_basis<<<vgrid, 256, 0, st>>>(V, ldv, n3, S.y, restart, S.kcount, x, n3, n3);
        GM_LAUNCH();
        for (int r = 0; r < nrhs; ++r) relres_out[r] = hres[r];
        if (fl.ls_restart || (fl.r_out && cyc == maxit - 1)) {
            k_ls_residual_coeffs<<<(nrhs + 31) / 32, 32, 0, st>>>(S, restart, nrhs, u, kMaxCols + 1);
            GM_LAUNCH();
            k_combine_basis<<<vgrid, 256, 0, st>>>(V, ldv, n3, u, kMaxCols + 1, S.kcount, 1, w, n3, n3);
            GM_LAUNCH();
            w_is_resid = true;
            if (fl.ls_restart && cyc + 1 < maxit) {
                GM_CUDA(cudaMemcpyAsync(V, w, sizeof(double) * ldv, cudaMemcpyDeviceToDevice, st));
                resid_ready = true;
            }
        }
    }
    if (fl.r_out) {
        if (at_start_exit) {
            GM_CUDA(cudaMemcpyAsync(fl.r_out, V, sizeof(double) * ldv, cudaMemcpyDeviceToDevice, st));
        } else if (w_is_resid) {
            GM_CUDA(cudaMemcpyAsync(fl.r_out, w, sizeof(double) * ldv, cudaMemcpyDeviceToDevice, st));
        } else {
            GM_TRY(matvec_any(s, x, w, nrhs, precision, st));
            ++*mv_count;
            k_sub<<<grid_for(ldv, 256), 256, 0, st>>>(b, w, fl.r_out, ldv);
            GM_LAUNCH();
        }
    }
    if (!fl.final_check) {
        for (int r = 0; r < nrhs; ++r) {
            conv[r] = relres_out[r] <= tol;
            if (!conv[r]) rc = MPS_NOT_CONVERGED;
        }
        *cycles_out = cyc;
        release();
        return rc;
    }
    // final true residual
    GM_TRY(matvec_any(s, x, w, nrhs, precision, st));
    ++*mv_count;
    k_sub<<<grid_for(ldv, 256), 256, 0, st>>>(b, w, w, ldv);
    GM_LAUNCH();
    GM_TRY(multidot(w, n3, n3, 1, w, n3, n3, nrhs, partial, S.nrm2, 1, st));
    {
        double *nr = s->host_scr + nrhs, *nb = s->host_scr + 2 * nrhs;
        GM_CUDA(cudaMemcpyAsync(nr, S.nrm2, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        GM_CUDA(cudaMemcpyAsync(nb, S.bnorm, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        GM_CUDA(cudaStreamSynchronize(st));
        for (int r = 0; r < nrhs; ++r) {
            relres_out[r] = nb[r] > 0 ? sqrt(nr[r]) / nb[r] : 0.0;
            conv[r] = relres_out[r] <= tol;
            if (!conv[r]) rc = MPS_NOT_CONVERGED;
        }
    }
    *cycles_out = cyc;
    release();
#undef GM_TRY
#undef GM_CUDA
#undef GM_LAUNCH
    return rc;
}

// Relative residuals ||b - A x|| / ||b|| with the float64 operator; r receives b - A x.
static int true_residual(mps_system *s, const double *b, const double *x, double *r, double *ax, int nrhs,
                         double *partial, double *nrm, std::vector<double> &relres, cudaStream_t st) {
    const int64_t n3 = (int64_t)s->ndof * s->n;
    MPS_TRY(matvec_any(s, x, ax, nrhs, s->resid_prec, st));
    k_sub<<<grid_for((int64_t)nrhs * n3, 256), 256, 0, st>>>(b, ax, r, (int64_t)nrhs * n3);
    MPS_LAUNCH_CHECK();
    MPS_TRY(multidot(r, n3, n3, 1, r, n3, n3, nrhs, partial, nrm, 1, st));
    MPS_TRY(multidot(b, n3, n3, 1, b, n3, n3, nrhs, partial, nrm + nrhs, 1, st));
    double *hn = s->host_scr + 3 * nrhs;   // pinned (2 nrhs)
    MPS_CUDA_TRY(cudaMemcpyAsync(hn, nrm, sizeof(double) * 2 * nrhs, cudaMemcpyDeviceToHost, st));
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    for (int q = 0; q < nrhs; ++q) relres[q] = hn[nrhs + q] > 0 ? sqrt(hn[q]) / sqrt(hn[nrhs + q]) : 0.0;
    return MPS_OK;
}

// Norms ||r_q|| / ||b_q|| for every system (host result).
static int rel_norms(const double *r, const double *b, int64_t n3, int nrhs, double *partial, double *nrm,
                     std::vector<double> &rel, double *hn, cudaStream_t st) {
    MPS_TRY(multidot(r, n3, n3, 1, r, n3, n3, nrhs, partial, nrm, 1, st));
    MPS_TRY(multidot(b, n3, n3, 1, b, n3, n3, nrhs, partial, nrm + nrhs, 1, st));
    MPS_CUDA_TRY(cudaMemcpyAsync(hn, nrm, sizeof(double) * 2 * nrhs, cudaMemcpyDeviceToHost, st));
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    for (int q = 0; q < nrhs; ++q) rel[q] = hn[nrhs + q] > 0 ? sqrt(hn[q]) / sqrt(hn[nrhs + q]) : 0.0;
    return MPS_OK;
}

// Mixed precision: float32-operator GMRES (float64 Arnoldi) for the solve and
// every correction, float64 for the refinement residual.
//   step 0: x1 = GMRES32(b, from x0)
//   r = b - A64 x1                       (the one float64 matvec)
//   repeat: d = GMRES32(r, from 0); x += d; r <- b - A32-consistent residual
// With residual_policy 0 the residual after a correction is the inner GMRES's
// least-squares residual (Arnoldi relation: r - A32 d = V_{k+1} u), exact up to
// float32 rounding on the small correction d; with policy 1 every step
// recomputes b - A64 x.  verify != 0 adds a final float64 true residual.
static int refine_mixed(mps_system *s, const double *b, double *x, int nrhs, const mps_solve_opts *o, int *conv,
                        double *relres_out, int *cycles_out, int *mv64, int *mv32, cudaStream_t st) {
    const int64_t n3 = (int64_t)s->ndof * s->n;
    const int64_t tot = (int64_t)nrhs * n3;
    const int nblk = (int)((n3 + kDotChunk - 1) / kDotChunk);
    const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
    const int inner_maxit = o->inner_maxit > 0 ? o->inner_maxit : 4;
    const bool incremental = o->residual_policy == 0;
    double *buf = nullptr;
    const size_t bytes = sizeof(double) * (4 * (size_t)tot + 2 * nrhs) + multidot_bytes(n3, nrhs);
    MPS_CUDA_TRY(cudaMallocAsync((void **)&buf, bytes, st));
    double *r = buf, *dx = buf + tot, *ax = buf + 2 * tot, *rn = buf + 3 * tot, *nrm = buf + 4 * tot,
           *partial = nrm + 2 * nrhs;
    (void)nblk;
    {
        int e0 = multidot_init(partial, n3, nrhs, st);
        if (e0) {
            cudaFreeAsync(buf, st);
            return e0;
        }
    }
    std::vector<double> rel(nrhs);
    std::vector<int> ic(nrhs);
    std::vector<double> ir(nrhs);
    int rc = MPS_NOT_CONVERGED;
    int step = 0;
    int e = MPS_OK;
    // The double-float residual's first-use set-up (weights, tiles, grids, scale tensor) runs on the system's
    // prep stream beside the first inner solve, when nothing in it has to be timed (its tile depth is known).
    cudaEvent_t ev_prep = nullptr;
    if (s->resid_prec == MPS_DF && df_usable(s) && !s->wdf && tile_depth_known(s, kTileDF)) {
        cudaEvent_t ev_in = nullptr;
        bool ok = (s->prep || cudaStreamCreateWithFlags(&s->prep, cudaStreamNonBlocking) == cudaSuccess) &&
                  cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventRecord(ev_in, st) == cudaSuccess && cudaStreamWaitEvent(s->prep, ev_in, 0) == cudaSuccess;
        if (ev_in) cudaEventDestroy(ev_in);
        bool used = false;
        if (ok) ok = df_prepare(s, s->prep, &used) == MPS_OK;
        ok = ok && cudaEventCreateWithFlags(&ev_prep, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventRecord(ev_prep, s->prep) == cudaSuccess;
        if (!ok) {
            cudaFreeAsync(buf, st);
            if (ev_prep) cudaEventDestroy(ev_prep);
            return MPS_CUDA_ERR;
        }
    }
    {
        GmresFlags f0;
        f0.final_check = false;
        f0.ls_restart = true;
        f0.reorth = false;
        int icyc = 0;
        e = gmres_core(s, b, x, nrhs, inner_tol, o->restart, inner_maxit, s->inner_prec, ic.data(), ir.data(), &icyc, mv32,
                       st, f0);
    }
    if (ev_prep) {
        if (cudaStreamWaitEvent(st, ev_prep, 0) != cudaSuccess && e == MPS_OK) e = MPS_CUDA_ERR;
        cudaEventDestroy(ev_prep);
    }
    if (e == MPS_OK || e == MPS_NOT_CONVERGED) {
        e = true_residual(s, b, x, r, ax, nrhs, partial, nrm, rel, st);
        ++*mv64;
    }
    // With the gradient-form inner operator the Arnoldi-relation residual tracks
    // r - A' d, which differs from the true r - A d by (A - A') d: about
    // kGradMismatch times the residual the correction started from (the form's
    // relative distance from the reference operator is measured at 5e-6..1.1e-4
    // for supports P = 10..8).  The drift adds up over the corrections since the
    // last true residual; when it could exceed the target, one true residual decides.
    // A coarser inner grid (when the system has one) adds its discretisation's distance to the gradient form's
    // own; the inner grids chosen by the Python layer keep it at 3e-5..6e-5 (measured), inside the same bound.
    constexpr double kGradMismatch = 3e-4;
    bool estimated = false;
    std::vector<double> drift(nrhs, 0.0);
    for (step = 1; e == MPS_OK; ++step) {
        bool all = true;
        for (int q = 0; q < nrhs; ++q) {
            conv[q] = rel[q] <= o->tol;
            all = all && conv[q];
        }
        if (all && estimated && s->inner_prec == MPS_FP32_GRAD) {
            bool sure = true;
            for (int q = 0; q < nrhs; ++q) sure = sure && drift[q] + rel[q] <= o->tol;
            if (!sure) {
                e = true_residual(s, b, x, r, ax, nrhs, partial, nrm, rel, st);
                ++*mv64;
                estimated = false;
                std::fill(drift.begin(), drift.end(), 0.0);
                if (e) break;
                all = true;
                for (int q = 0; q < nrhs; ++q) {
                    conv[q] = rel[q] <= o->tol;
                    all = all && conv[q];
                }
            }
        }
        for (int q = 0; q < nrhs; ++q) {
            relres_out[q] = rel[q];
            // a converged system gets a zero right-hand side: its correction stays zero
            if (conv[q] && cudaMemsetAsync(r + q * n3, 0, sizeof(double) * n3, st) != cudaSuccess) e = MPS_CUDA_ERR;
        }
        if (e) break;
        if (all) {
            rc = MPS_OK;
            break;
        }
        if (step > o->maxit) break;
        if (cudaMemsetAsync(dx, 0, sizeof(double) * tot, st) != cudaSuccess) {
            e = MPS_CUDA_ERR;
            break;
        }
        GmresFlags fl;
        fl.zero_guess = true;
        fl.final_check = false;
        fl.ls_restart = true;
        fl.reorth = false;
        fl.r_out = incremental ? rn : nullptr;
        // the correction only has to take the worst residual below the target:
        // relative tolerance max(inner_tol, 0.3 tol / relres), at most 0.5
        double worst = 0.0;
        for (int q = 0; q < nrhs; ++q)
            if (!conv[q]) worst = std::max(worst, rel[q]);
        double step_tol = inner_tol;
        if (worst > 0.0) step_tol = std::max(inner_tol, std::min(0.5, 0.3 * o->tol / worst));
        for (int q = 0; q < nrhs; ++q) drift[q] += kGradMismatch * rel[q];
        int icyc = 0;
        int g = gmres_core(s, r, dx, nrhs, step_tol, o->restart, inner_maxit, s->inner_prec, ic.data(), ir.data(), &icyc,
                           mv32, st, fl);
        if (g != MPS_OK && g != MPS_NOT_CONVERGED) {
            e = g;
            break;
        }
        k_axpy1<<<grid_for(tot, 256), 256, 0, st>>>(dx, x, tot);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) {
            e = MPS_CUDA_ERR;
            break;
        }
        if (incremental) {
            if (cudaMemcpyAsync(r, rn, sizeof(double) * tot, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
                e = MPS_CUDA_ERR;
                break;
            }
            e = rel_norms(r, b, n3, nrhs, partial, nrm, rel, s->host_scr + 3 * nrhs, st);
            estimated = true;
        } else {
            e = true_residual(s, b, x, r, ax, nrhs, partial, nrm, rel, st);
            ++*mv64;
            std::fill(drift.begin(), drift.end(), 0.0);
        }
    }
    if (e == MPS_OK && o->verify) {
        e = true_residual(s, b, x, r, ax, nrhs, partial, nrm, rel, st);
        ++*mv64;
        if (e == MPS_OK) {
            rc = MPS_OK;
            for (int q = 0; q < nrhs; ++q) {
                relres_out[q] = rel[q];
                conv[q] = rel[q] <= o->tol;
                if (!conv[q]) rc = MPS_NOT_CONVERGED;
            }
        }
    }
    if (e != MPS_OK) rc = e;
    *cycles_out = step;
    cudaFreeAsync(buf, st);
    return rc;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// The Green's coefficients of a grid from the process cache (keyed by device, grid, box, xi, eta), computed on
// stream st and entered in the cache when absent; a cached entry filled on another stream is waited for.
static int acquire_green(const GridParams &gp, const double *box, double xi, int64_t Gc,
                         std::shared_ptr<GreenCoef> &out, cudaStream_t st) {
    GreenKey key;
    memset(&key, 0, sizeof(key));
    key.dev = current_device();
    for (int k = 0; k < 3; ++k) {
        key.N[k] = gp.N[k];
        key.box[k] = box[k];
        key.eta[k] = gp.eta[k];
    }
    key.xi = xi;
    std::lock_guard<std::mutex> lk(g_green_mu);
    auto it = g_green.find(key);
    if (it != g_green.end()) {
        out = it->second;
        MPS_CUDA_TRY(cudaStreamWaitEvent(st, out->ev_h, 0));
        return MPS_OK;
    }
    auto gc = std::make_shared<GreenCoef>();
    MPS_TRY(dalloc_persistent(&gc->h64, sizeof(double) * Gc));
    MPS_TRY(dalloc_persistent(&gc->h32, sizeof(float) * Gc));
    MPS_TRY(green_half(gp, gc->h64, gc->h32, st));
    MPS_TRY(green_mark_filled(&gc->ev_h, st));
    if (g_green.size() >= kGreenCacheMax) g_green.clear();  // systems keep their own reference
    g_green[key] = gc;
    out = gc;
    return MPS_OK;
}

// Grid geometry (start nodes, separable weights) and Green's coefficients of a dipole or quadrupole system, on
// stream gs: none of it depends on the pair list, so the caller runs it on the side stream beside the pair-list
// construction (and the inner grid's set-up on a third stream).
static int setup_grids(mps_system *s, const mps_system_desc *d, cudaStream_t gs) {
    const int64_t n = d->n;
#define GS_TRY(expr)                   \
    do {                               \
        const int _r = (expr);         \
        if (_r != MPS_OK) return _r;   \
    } while (0)
    GS_TRY(dalloc(&s->start, sizeof(int32_t) * 3 * n, gs));
    GS_TRY(dalloc(&s->w64, sizeof(double) * 3 * n * d->P, gs));
    GS_TRY(dalloc(&s->w32, sizeof(float) * 3 * n * d->P, gs));
    GS_TRY(grid_geometry(s->x, n, s->gp, s->start, s->w64, s->w32, gs));
    GS_TRY(acquire_green(s->gp, d->box, d->xi, s->Gc, s->green, gs));
    s->h64 = s->green->h64;
    s->h32 = s->green->h32;
#undef GS_TRY
    return MPS_OK;
}

// The inner grid of the gradient-form operator, when asked for (dipole operator, tiled kernels), on stream gs.
static int setup_inner_grid(mps_system *s, const mps_system_desc *d, cudaStream_t gs) {
    const int64_t n = d->n;
#define GS_TRY(expr)                   \
    do {                               \
        const int _r = (expr);         \
        if (_r != MPS_OK) return _r;   \
    } while (0)
    if (d->inner_P > 0) {
        for (int k = 0; k < 3; ++k)
            if (d->inner_Ngrid[k] < d->inner_P) GS_TRY(MPS_BAD_ARG);
        if (d->inner_P > kMaxP) GS_TRY(MPS_BAD_ARG);
        s->inner = new InnerGrid();
        InnerGrid &ig = *s->inner;
        ig.gp = make_grid_params(d->inner_Ngrid, d->box, d->xi, nullptr, d->inner_P);
        if (!tiles_supported(ig.gp, 8)) GS_TRY(MPS_BAD_ARG);
        ig.Gc = (int64_t)(ig.gp.N[0] / 2 + 1) * ig.gp.N[1] * ig.gp.N[2];
        GS_TRY(dalloc(&ig.start, sizeof(int32_t) * 3 * n, gs));
        GS_TRY(dalloc(&ig.w64, sizeof(double) * 3 * n * ig.gp.P, gs));
        GS_TRY(dalloc(&ig.w32, sizeof(float) * 3 * n * ig.gp.P, gs));
        GS_TRY(dalloc(&ig.g32, sizeof(float) * 3 * n * ig.gp.P, gs));
        GS_TRY(grid_geometry(s->x, n, ig.gp, ig.start, ig.w64, ig.w32, gs));
        GS_TRY(grad_factors(s->x, n, ig.gp, ig.w64, ig.g32, gs));
        // depth 12 as for the system's own gradient-form tiles (tuned_depth); MPS_TILE_DEPTH overrides it
        int tz_in = tiles_supported(ig.gp, 12) ? 12 : 8;
        if (const char *fd = getenv("MPS_TILE_DEPTH")) {
            const int dz = atoi(fd);
            if ((dz == 4 || dz == 8 || dz == 12 || dz == 16) && tiles_supported(ig.gp, dz)) tz_in = dz;
        }
        GS_TRY(tile_bins_build(ig.start, n, ig.gp, tz_in, ig.tb, gs));
        if (contract_grad_home_supported(ig.gp)) GS_TRY(tile_bins_home(ig.start, n, ig.gp, ig.tb, gs));
        GS_TRY(acquire_green(ig.gp, d->box, d->xi, ig.Gc, ig.green, gs));
        // the inner operator's scale coefficient too: the first inner matvec then finds it ready
        GS_TRY(inner_hs32(s, gs));
    }
#undef GS_TRY
    return MPS_OK;
}

extern "C" int mps_system_create(const mps_system_desc *d, mps_system **out, mps_stream_t stream) {
    if (!d || !out) return MPS_BAD_ARG;
    *out = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    if (d->n < 1 || !d->x || !d->lambdap || d->n_diag < 1 || !(d->xi > 0) || !(d->rc > 0) || d->P < 1 ||
        d->max_rhs < 1)
        return MPS_BAD_ARG;
    if (d->kind != MPS_DIPOLE && d->kind != MPS_DIPOLE_QUADRUPOLE && d->kind != MPS_POLYDISPERSE) return MPS_BAD_ARG;
    if (d->kind != MPS_POLYDISPERSE && (!d->perp || !d->para || !d->rvals || d->n_tab < 2)) return MPS_BAD_ARG;
    if (d->kind == MPS_POLYDISPERSE) {
        if (!d->radius || d->slab_factor != 0.0) return MPS_BAD_ARG;
        if (d->radius_class && (!d->sizes_tables || !d->rvals || d->n_tab < 2 || d->n_class < 1)) return MPS_BAD_ARG;
    }
    // the quadrupole operator has no slab term (CQ/MatrixVectorMultiply.m)
    if (d->kind == MPS_DIPOLE_QUADRUPOLE && (!d->quad_tables || d->slab_factor != 0.0)) return MPS_BAD_ARG;
    // complex permittivities: dipole operator only
    if (d->lambdap_imag && d->kind != MPS_DIPOLE) return MPS_BAD_ARG;
    for (int k = 0; k < 3; ++k) {
        if (!(d->box[k] > 0) || d->Ngrid[k] < 1) return MPS_BAD_ARG;
        if (d->Ngrid[k] < d->P) return MPS_BAD_ARG;  // the stencil wraps at most once
        if (d->rc > d->box[k] / 2.0) return MPS_RC_GT_HALF_BOX;
    }
    if (d->P > 32) return MPS_BAD_ARG;
    configure_pool_once();
    mps_system *s = new mps_system();
    s->stream = st;
    s->n = d->n;
    s->cplx = d->lambdap_imag != nullptr;
    s->max_rhs_c = s->cplx ? d->max_rhs : 0;
    s->max_rhs = s->cplx ? 2 * d->max_rhs : d->max_rhs;   // real vectors per matvec
    s->n_diag = d->n_diag;
    memcpy(s->box, d->box, sizeof(s->box));
    s->xi = d->xi;
    s->rc = d->rc;
    s->slab_factor = d->slab_factor;
    s->kind = d->kind;
    s->ndof = d->kind == MPS_DIPOLE_QUADRUPOLE ? 8 : (s->cplx ? 6 : 3);
    s->gp = make_grid_params(d->Ngrid, d->box, d->xi, d->eta, d->P);
    s->Gc = (int64_t)(s->gp.N[0] / 2 + 1) * s->gp.N[1] * s->gp.N[2];
    const int64_t n = d->n;
    int rc = MPS_OK;
#define CR_TRY(expr)               \
    do {                           \
        rc = (expr);               \
        if (rc != MPS_OK) {        \
            free_system(s);        \
            return rc;             \
        }                          \
    } while (0)
    CR_TRY(dalloc(&s->x, sizeof(double) * 3 * n, st));
    if (cudaMemcpyAsync(s->x, d->x, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        CR_TRY(MPS_CUDA_ERR);
    CR_TRY(dalloc(&s->diag, sizeof(double) * n * d->n_diag, st));
    if (s->kind == MPS_POLYDISPERSE)
        CR_TRY(cs_diag(d->lambdap, n, d->n_diag, d->radius, d->radius_class, d->n_class,
                       d->radius_class ? d->sizes_tables : nullptr, d->n_tab, d->xi, s->diag, st));
    else if (s->cplx) {
        CR_TRY(dalloc(&s->diag_im, sizeof(double) * n * d->n_diag, st));
        CR_TRY(build_diag_complex(d->lambdap, d->lambdap_imag, n * d->n_diag, d->perp, s->diag, s->diag_im, st));
    } else {
        CR_TRY(build_diag(d->lambdap, n * d->n_diag, d->perp, s->diag, st));
    }
    CR_TRY(dalloc(&s->slab, sizeof(double) * s->max_rhs, st));
    if (cudaMemsetAsync(s->slab, 0, sizeof(double) * s->max_rhs, st) != cudaSuccess) CR_TRY(MPS_CUDA_ERR);
    CR_TRY(dalloc(&s->diag_idx, sizeof(int32_t) * s->max_rhs, st));
    {
        const size_t ints = ((size_t)2 * s->max_rhs + 1) & ~(size_t)1;   // even: the doubles stay 8-byte aligned
        const size_t pinned = sizeof(int32_t) * ints + sizeof(double) * (6 * s->max_rhs + 2);
        s->diag_idx_host = static_cast<int32_t *>(pinned_take(pinned));
        if (!s->diag_idx_host) CR_TRY(MPS_NO_MEMORY);
        s->host_frozen = s->diag_idx_host + s->max_rhs;
        s->host_scr = reinterpret_cast<double *>(s->diag_idx_host + ints);
        s->host_step = reinterpret_cast<int32_t *>(s->host_scr + 6 * s->max_rhs);
        s->host_herr = reinterpret_cast<int32_t *>(s->host_scr + 6 * s->max_rhs + 1);
    }
    if (cudaMemsetAsync(s->diag_idx, 0, sizeof(int32_t) * s->max_rhs, st) != cudaSuccess) CR_TRY(MPS_CUDA_ERR);
    // grids and k-space on the side stream, beside the pair list below (joined before returning)
    const bool grids_on_side = s->kind != MPS_POLYDISPERSE;
    if (grids_on_side) {
        if (cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(s->ev_fork, st) != cudaSuccess ||
            cudaStreamWaitEvent(s->side, s->ev_fork, 0) != cudaSuccess ||
            cudaStreamWaitEvent(s->cap, s->ev_fork, 0) != cudaSuccess)
            CR_TRY(MPS_CUDA_ERR);
        // setup_grids / setup_inner_grid are enqueued below, while the GPU counts the pairs
    }
    // cell list + pair CSR
    compute_ncell(d->box, d->rc, s->ncell);
    const int64_t ncells = s->ncell[0] * s->ncell[1] * s->ncell[2];
    int64_t *cell3 = nullptr, *cnt27 = nullptr, *off27 = nullptr;
    void *bins = nullptr, *scan_tmp = nullptr;
    int *err = nullptr;
    float *xf = nullptr;
    unsigned *maxbits = nullptr;
    double maxabs = 0.0;
    CR_TRY(dalloc(&xf, sizeof(float) * 3 * n, st));
    CR_TRY(dalloc(&maxbits, sizeof(unsigned) * 4, st));
    CR_TRY(dalloc(&cell3, sizeof(int64_t) * 3 * n, st));
    CR_TRY(dalloc(&bins, cell_bins_bytes(n, ncells), st));
    CR_TRY(dalloc(&cnt27, sizeof(int64_t) * 27 * n, st));
    CR_TRY(dalloc(&off27, sizeof(int64_t) * 27 * n, st));
    CR_TRY(dalloc(&scan_tmp, scan_workspace(27 * n), st));
    CR_TRY(dalloc(&err, sizeof(int), st));
    auto tmp_free = [&]() {
        cudaFreeAsync(cell3, st);
        cudaFreeAsync(bins, st);
        cudaFreeAsync(cnt27, st);
        cudaFreeAsync(off27, st);
        cudaFreeAsync(scan_tmp, st);
        cudaFreeAsync(err, st);
        cudaFreeAsync(xf, st);
        cudaFreeAsync(maxbits, st);
    };
    CellBins cb;
    rc = cell_assign(s->x, n, d->box, s->ncell, cell3, st);
    if (!rc) rc = cell_bins_build(cell3, n, s->ncell, bins, cb, st);
    if (!rc) rc = dalloc(&s->order, sizeof(int32_t) * n, st);
    if (!rc && n > 0 && cudaMemcpyAsync(s->order, cb.sorted, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st) !=
                            cudaSuccess)
        rc = MPS_CUDA_ERR;
    if (!rc) s->gp.order = s->order;
    int64_t np = 0;
    if (!rc) rc = positions_f32(s->x, n, xf, maxbits, &maxabs, st);
    int64_t *last2 = reinterpret_cast<int64_t *>(s->host_scr);   // page-locked, free until the first solve
    if (!rc) rc = csr_pairs_count(s->x, xf, maxabs, d->box, d->rc, cb, cnt27, off27, scan_tmp, last2, st);
    // the grid geometry and k-space (side stream) and the inner grid (the capture stream, idle until the first
    // solve) are enqueued while the GPU runs the count: their host work (allocations, cache lookups, launches)
    // no longer delays the pair list, the longest chain of the build
    if (!rc && grids_on_side) rc = setup_grids(s, d, s->side);
    if (!rc && grids_on_side) rc = setup_inner_grid(s, d, s->cap);
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = MPS_CUDA_ERR;
    if (!rc) np = last2[0] + last2[1];
    if (rc) {
        tmp_free();
        free_system(s);
        return rc;
    }
    s->n_pairs = np;
    rc = dalloc(&s->row_ptr, sizeof(int64_t) * (n + 1), st);
    if (!rc) rc = dalloc(&s->p64.nbr, sizeof(int32_t) * np, st);
    const bool df_pairs = s->kind == MPS_DIPOLE;   // double-float pair list, float64 copy on demand
    PairData<double> &pfill = s->p64;
    if (df_pairs) {
        if (!rc) rc = dalloc(&s->pdf.A, sizeof(dfv) * np, st);
        if (!rc) rc = dalloc(&s->pdf.BA, sizeof(dfv) * np, st);
        if (!rc) rc = dalloc(&s->pdf.rx, sizeof(dfv) * np, st);
        if (!rc) rc = dalloc(&s->pdf.ry, sizeof(dfv) * np, st);
        if (!rc) rc = dalloc(&s->pdf.rz, sizeof(dfv) * np, st);
        if (!rc) rc = dalloc(&s->pdf.dist, sizeof(dfv) * np, st);
    } else {
        if (!rc) rc = dalloc(&pfill.A, sizeof(double) * np, st);
        if (!rc) rc = dalloc(&pfill.BA, sizeof(double) * np, st);
        if (!rc) rc = dalloc(&pfill.rx, sizeof(double) * np, st);
        if (!rc) rc = dalloc(&pfill.ry, sizeof(double) * np, st);
        if (!rc) rc = dalloc(&pfill.rz, sizeof(double) * np, st);
    }
    if (!rc) rc = dalloc(&s->p32.A, sizeof(float) * np, st);
    if (!rc) rc = dalloc(&s->p32.BA, sizeof(float) * np, st);
    if (!rc) rc = dalloc(&s->p32.rx, sizeof(float) * np, st);
    if (!rc) rc = dalloc(&s->p32.ry, sizeof(float) * np, st);
    if (!rc) rc = dalloc(&s->p32.rz, sizeof(float) * np, st);
    s->p32.nbr = s->p64.nbr;
    s->pdf.nbr = s->p64.nbr;
    // separations (float64) of the other operators, which derive their couplings from them
    if (!rc && !df_pairs) rc = dalloc(&s->p64.dist, sizeof(double) * np, st);
    // the polydisperse couplings depend on the pair's radii: filled in below
    const int64_t fill_ntab = s->kind == MPS_POLYDISPERSE ? 0 : d->n_tab;
    if (!rc && cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) rc = MPS_CUDA_ERR;
    if (!rc && df_pairs) {
        float2 *xdf = nullptr;
        void *tabbuf = nullptr;
        DfTab tab;
        rc = dalloc(&xdf, sizeof(float2) * 3 * n, st);
        if (!rc) rc = dalloc(&tabbuf, df_tab_bytes(d->n_tab), st);
        if (!rc) rc = positions_df(s->x, n, xdf, st);
        if (!rc) rc = df_tab_build(d->perp, d->para, d->rvals, d->n_tab, tabbuf, tab, st);
        if (!rc)
            rc = csr_pairs_fill_df(s->x, xf, xdf, maxabs, d->box, d->rc, cb, cnt27, off27, tab, s->row_ptr, s->pdf,
                                   s->p32, err, st);
        if (xdf) cudaFreeAsync(xdf, st);
        if (tabbuf) cudaFreeAsync(tabbuf, st);
    } else if (!rc) {
        rc = csr_pairs_fill(s->x, xf, maxabs, d->box, d->rc, cb, cnt27, off27, d->perp, d->para, d->rvals, fill_ntab,
                            s->row_ptr, s->p64, s->p32, err, st);
    }
    int herr = 0;
    if (s->kind == MPS_DIPOLE) {
        // The table-range flag is read by the first call that uses the system (build_status), not here: the
        // host goes on to the caller's first solve while the GPU still fills the pair list.
        if (!rc && cudaMemcpyAsync(s->host_herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = MPS_CUDA_ERR;
        if (!rc && (cudaEventCreateWithFlags(&s->ev_build, cudaEventDisableTiming) != cudaSuccess ||
                    cudaEventRecord(s->ev_build, st) != cudaSuccess))
            rc = MPS_CUDA_ERR;
        if (!rc) s->build_check = true;
    } else {
        if (!rc && cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = MPS_CUDA_ERR;
        if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = MPS_CUDA_ERR;
    }
    tmp_free();
    if (!rc && herr) rc = MPS_TABLE_RANGE;
    if (!rc && s->kind == MPS_POLYDISPERSE) {
        int *perr = nullptr;
        rc = dalloc(&perr, sizeof(int), st);
        if (!rc && cudaMemsetAsync(perr, 0, sizeof(int), st) != cudaSuccess) rc = MPS_CUDA_ERR;
        if (!rc)
            rc = cs_pair_coefs(s->row_ptr, s->p64.nbr, s->p64.dist, n, d->radius, d->radius_class, d->n_class,
                               d->radius_class ? d->sizes_tables : nullptr, d->rvals, d->n_tab, d->xi, s->p64, s->p32,
                               perr, st);
        if (!rc && cudaMemcpyAsync(&herr, perr, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = MPS_CUDA_ERR;
        if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = MPS_CUDA_ERR;
        if (perr) cudaFreeAsync(perr, st);
        if (!rc && herr) rc = MPS_TABLE_RANGE;
        if (s->p64.dist) cudaFreeAsync(s->p64.dist, st);
        s->p64.dist = nullptr;
    }
    if (!rc && s->kind == MPS_DIPOLE_QUADRUPOLE) {
        // nine couplings per pair from the stored separations, then the
        // separations are dropped
        rc = dalloc(&s->qcoef, sizeof(double) * 9 * np, st);
        if (!rc) rc = dalloc(&s->qcoef32, sizeof(float) * 9 * np, st);
        int *qerr = nullptr;
        if (!rc) rc = dalloc(&qerr, sizeof(int), st);
        if (!rc && cudaMemsetAsync(qerr, 0, sizeof(int), st) != cudaSuccess) rc = MPS_CUDA_ERR;
        if (!rc)
            rc = quad_pair_coefs(s->p64.dist, np, d->perp, d->para, d->quad_tables, d->rvals, d->n_tab, s->qcoef,
                                 s->qcoef32, qerr, st);
        if (!rc && cudaMemcpyAsync(&herr, qerr, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = MPS_CUDA_ERR;
        if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = MPS_CUDA_ERR;
        if (qerr) cudaFreeAsync(qerr, st);
        if (!rc && herr) rc = MPS_TABLE_RANGE;
        if (s->p64.dist) cudaFreeAsync(s->p64.dist, st);
        s->p64.dist = nullptr;
        if (!rc) rc = dalloc(&s->diagq, sizeof(double) * n * d->n_diag, st);
        if (!rc) rc = quad_diag(d->lambdap, n * d->n_diag, d->quad_tables + 4 * d->n_tab, s->diagq, st);
        if (!rc) rc = dalloc(&s->qkcoef, sizeof(double) * 4 * s->Gc, st);
        if (!rc) rc = dalloc(&s->qkcoef32, sizeof(float) * 4 * s->Gc, st);
        if (!rc) rc = quad_kcoef(s->gp, s->qkcoef, s->qkcoef32, st);
    }
    if (rc) {
        free_system(s);
        return rc;
    }
    if (s->kind == MPS_POLYDISPERSE) {
        const int64_t P3 = (int64_t)d->P * d->P * d->P;
        CR_TRY(dalloc(&s->start, sizeof(int32_t) * 3 * n, st));
        CR_TRY(dalloc(&s->cs_base, sizeof(double) * 3 * n, st));
        CR_TRY(dalloc(&s->cs_g64, sizeof(double) * n * P3, st));
        CR_TRY(dalloc(&s->cs_g32, sizeof(float) * n * P3, st));
        CR_TRY(dalloc(&s->cs_h64, sizeof(double) * s->Gc, st));
        CR_TRY(dalloc(&s->cs_h32, sizeof(float) * s->Gc, st));
        CR_TRY(cs_geometry(s->x, n, s->gp, d->radius, d->xi, s->gp.eta[0], s->start, s->cs_base, s->cs_g64,
                           s->cs_g32, st));
        CR_TRY(cs_green(s->gp, s->gp.eta[0], d->xi, s->cs_h64, s->cs_h32, st));
        *out = s;
        return MPS_OK;
    }
    // the grid and k-space set-up ran on the side and capture streams beside the pair list: join them
    if (grids_on_side) {
        cudaEvent_t ev_inner = nullptr;
        const bool ok = cudaEventRecord(s->ev_join, s->side) == cudaSuccess &&
                        cudaStreamWaitEvent(st, s->ev_join, 0) == cudaSuccess &&
                        cudaEventCreateWithFlags(&ev_inner, cudaEventDisableTiming) == cudaSuccess &&
                        cudaEventRecord(ev_inner, s->cap) == cudaSuccess &&
                        cudaStreamWaitEvent(st, ev_inner, 0) == cudaSuccess;
        if (ev_inner) cudaEventDestroy(ev_inner);
        if (!ok) CR_TRY(MPS_CUDA_ERR);
    }
#undef CR_TRY
    *out = s;
    return MPS_OK;
}

extern "C" void mps_system_destroy(mps_system *sys) {
    if (sys) cudaDeviceSynchronize();
    free_system(sys);
}

// The result of the build's table-range check (MPS_TABLE_RANGE when a pair separation fell outside the
// real-space table), read once the build's copy of the flag has completed.
static int build_status(mps_system *s) {
    if (!s->build_check) return s->build_failed ? MPS_TABLE_RANGE : MPS_OK;
    MPS_CUDA_TRY(cudaEventSynchronize(s->ev_build));
    s->build_check = false;
    if (*s->host_herr) s->build_failed = true;
    return s->build_failed ? MPS_TABLE_RANGE : MPS_OK;
}

extern "C" int mps_system_info(const mps_system *sys, int64_t *n_pairs, int64_t *ncell) {
    if (!sys) return MPS_BAD_ARG;
    if (n_pairs) *n_pairs = sys->n_pairs;
    if (ncell)
        for (int d = 0; d < 3; ++d) ncell[d] = sys->ncell[d];
    return MPS_OK;
}

static int rhs_limit(const mps_system *s) { return s->cplx ? s->max_rhs_c : s->max_rhs; }

extern "C" int mps_matvec(mps_system *sys, const double *m, double *out, int32_t nrhs, const int32_t *diag_index,
                          int32_t precision, mps_stream_t stream) {
    if (!sys || !m || !out || nrhs < 1 || nrhs > rhs_limit(sys)) return MPS_BAD_ARG;
    if (precision != MPS_FP64 && precision != MPS_FP32 && precision != MPS_DF && precision != MPS_FP32_GRAD)
        return MPS_BAD_ARG;
    MPS_TRY(build_status(sys));
    cudaStream_t st = (cudaStream_t)stream;
    MPS_TRY(upload_diag_idx(sys, diag_index, nrhs, st));
    return matvec_any(sys, m, out, nrhs, precision, st);
}

extern "C" int mps_matvec_complex(mps_system *sys, const double *m_ri, double *out_ri, int32_t diag_index,
                                  mps_stream_t stream) {
    if (!sys || !m_ri || !out_ri || sys->max_rhs < 2 || sys->kind != MPS_DIPOLE || sys->cplx) return MPS_BAD_ARG;
    MPS_TRY(build_status(sys));
    cudaStream_t st = (cudaStream_t)stream;
    int32_t di[2] = {diag_index, diag_index};
    MPS_TRY(upload_diag_idx(sys, di, 2, st));
    const int64_t G = sys->gp.G;
    if (!sys->rgrid2) MPS_TRY(dalloc(&sys->rgrid2, sizeof(double) * 6 * G, st));
    if (!sys->cgrid) MPS_TRY(dalloc(&sys->cgrid, sizeof(double) * 2 * 3 * G, st));
    const double vol = sys->box[0] * sys->box[1] * sys->box[2];
    MPS_TRY(slab_terms(m_ri, sys->n, 2, sys->slab_factor / vol, sys->slab, st));
    MPS_TRY(spread<double>(m_ri, sys->n, 2, sys->start, sys->w64, sys->gp, sys->rgrid2, st));
    MPS_TRY(pack_complex(sys->rgrid2, G, sys->cgrid, st));
    MPS_TRY(exec_plan(sys, CUFFT_Z2Z, 3, sys->cgrid, sys->cgrid, CUFFT_FORWARD, st));
    MPS_TRY(scale_full_c2c(sys->cgrid, sys->gp, st));
    MPS_TRY(exec_plan(sys, CUFFT_Z2Z, 3, sys->cgrid, sys->cgrid, CUFFT_INVERSE, st));
    MPS_TRY(unpack_complex(sys->cgrid, G, sys->rgrid2, st));
    MPS_TRY(contract<double>(sys->rgrid2, sys->n, 2, sys->start, sys->w64, sys->gp, out_ri, st));
    MPS_TRY(ensure_p64(sys, st));
    return real_space_csr<double>(m_ri, out_ri, sys->n, 2, sys->row_ptr, sys->p64, sys->diag, sys->diag_idx, sys->slab,
                                  true, st);
}

// The solver options every solve entry point accepts (host-side check, no CUDA call).
static bool solve_opts_valid(const mps_solve_opts *o) {
    if (!o || o->restart < 1 || o->restart >= kMaxCols || o->maxit < 1 || !(o->tol > 0)) return false;
    if (o->precision != MPS_FP64 && o->precision != MPS_FP32 && o->precision != MPS_DF) return false;
    if (o->residual_precision != MPS_FP64 && o->residual_precision != MPS_DF) return false;
    return o->inner_operator == 0 || o->inner_operator == 1;
}

extern "C" int mps_gmres(mps_system *sys, const double *b, const double *x0, double *x, int32_t nrhs,
                         const int32_t *diag_index, const mps_solve_opts *opts, mps_solve_info *info,
                         mps_stream_t stream) {
    if (!sys || !b || !x || nrhs < 1 || nrhs > rhs_limit(sys) || !solve_opts_valid(opts)) return MPS_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    MPS_TRY(upload_diag_idx(sys, diag_index, nrhs, st));
    const int64_t n3 = (int64_t)sys->ndof * sys->n;
    const size_t vbytes = sizeof(double) * (size_t)nrhs * n3;
    if (x0 == nullptr) {
        MPS_CUDA_TRY(cudaMemsetAsync(x, 0, vbytes, st));
    } else if (x0 != x) {
        MPS_CUDA_TRY(cudaMemcpyAsync(x, x0, vbytes, cudaMemcpyDeviceToDevice, st));
    }
    std::vector<int> conv(nrhs, 0);
    std::vector<double> relres(nrhs, 0.0);
    int cycles = 0, mv64 = 0, mv32 = 0;
    int rc;
    sys->resid_prec = opts->residual_precision;
    sys->inner_prec = opts->inner_operator == 1 ? MPS_FP32_GRAD : MPS_FP32;
    if (opts->precision == MPS_FP64 || opts->precision == MPS_DF) {
        rc = gmres_core(sys, b, x, nrhs, opts->tol, opts->restart, opts->maxit, opts->precision, conv.data(),
                        relres.data(), &cycles, &mv64, st);
    } else {
        rc = refine_mixed(sys, b, x, nrhs, opts, conv.data(), relres.data(), &cycles, &mv64, &mv32, st);
    }
    if (info) {
        for (int q = 0; q < nrhs; ++q) {
            info[q].converged = conv[q];
            info[q].relres = relres[q];
            info[q].cycles = cycles;
            info[q].matvecs_fp64 = mv64;
            info[q].matvecs_fp32 = mv32;
        }
    }
    // the build's table-range check, read after the solve (which the pair fill preceded on the stream)
    const int bs = build_status(sys);
    return bs != MPS_OK ? bs : rc;
}

// ---------------------------------------------------------------------------
// Many configurations (the parfor over configurations of CH/CapacitanceTensorSpectrum.m:45 and
// CS/CapacitanceTensorSpectrum.m:44)
// ---------------------------------------------------------------------------
constexpr int kMaxBatchStreams = 32;

// Builds, solves and releases one configuration on stream st.  Everything the system runs is on st or on its
// own side streams, so waiting for st (and, in free_system, for those) is enough before the release: unlike
// mps_system_destroy, the other workers' streams keep running.
static int solve_batch_item(mps_batch_item *it, const mps_solve_opts *o, cudaStream_t st) {
    mps_system *s = nullptr;
    int rc = mps_system_create(&it->desc, &s, (mps_stream_t)st);
    if (rc == MPS_OK)
        rc = mps_gmres(s, it->b, it->x0, it->x, it->nrhs, it->diag_index, o, it->info, (mps_stream_t)st);
    if (cudaStreamSynchronize(st) != cudaSuccess && (rc == MPS_OK || rc == MPS_NOT_CONVERGED)) rc = MPS_CUDA_ERR;
    if (s) free_system(s);
    return rc;
}

extern "C" int mps_solve_batched(mps_batch_item *items, int32_t n_items, const mps_solve_opts *opts,
                                 int32_t n_streams, mps_stream_t stream) {
    if (n_items < 0 || (n_items > 0 && !items) || !solve_opts_valid(opts) || n_streams < 1) return MPS_BAD_ARG;
    if (n_items == 0) return MPS_OK;
    int dev = 0;
    MPS_CUDA_TRY(cudaGetDevice(&dev));
    // largest configurations first, so the last ones to start are the short ones
    std::vector<int32_t> order((size_t)n_items);
    for (int32_t i = 0; i < n_items; ++i) {
        order[i] = i;
        items[i].status = MPS_CUDA_ERR;   // until a worker has run it
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return items[a].desc.n * (int64_t)items[a].nrhs > items[b].desc.n * (int64_t)items[b].nrhs;
    });
    cudaEvent_t ready = nullptr;
    MPS_CUDA_TRY(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    if (cudaEventRecord(ready, (cudaStream_t)stream) != cudaSuccess) {
        cudaEventDestroy(ready);
        return MPS_CUDA_ERR;
    }
    std::atomic<int32_t> next{0};
    auto work = [&]() {
        cudaStream_t ws = nullptr;
        try {
            if (cudaSetDevice(dev) != cudaSuccess || cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking) != cudaSuccess ||
                cudaStreamWaitEvent(ws, ready, 0) != cudaSuccess) {
                if (ws) cudaStreamDestroy(ws);
                return;   // the other workers take this one's share
            }
            for (int32_t k = next.fetch_add(1); k < n_items; k = next.fetch_add(1)) {
                mps_batch_item *it = &items[order[k]];
                it->status = solve_batch_item(it, opts, ws);
            }
        } catch (...) {   // no exception crosses the C ABI; the items not run keep MPS_CUDA_ERR
        }
        if (ws) {
            cudaStreamSynchronize(ws);
            cudaStreamDestroy(ws);
        }
    };
    const int nw = std::min({(int)n_streams, (int)n_items, kMaxBatchStreams});
    std::vector<std::thread> threads;
    try {
        for (int w = 1; w < nw; ++w) threads.emplace_back(work);
    } catch (...) {   // fewer threads than asked: the workers started (and this thread) share the items
    }
    work();
    for (auto &t : threads) t.join();
    cudaEventDestroy(ready);
    int rc = MPS_OK;
    for (int32_t i = 0; i < n_items; ++i) {
        const int si = items[i].status;
        if (si != MPS_OK && si != MPS_NOT_CONVERGED) return si;
        if (si == MPS_NOT_CONVERGED) rc = MPS_NOT_CONVERGED;
    }
    return rc;
}

extern "C" int mps_system_profile(mps_system *sys, int32_t enable) {
    if (!sys) return MPS_BAD_ARG;
    sys->profile = enable != 0;
    return MPS_OK;
}

extern "C" int mps_system_stage_times(mps_system *sys, double *ms, int64_t *count) {
    if (!sys || !ms || !count) return MPS_BAD_ARG;
    for (auto &e : sys->pending) {
        MPS_CUDA_TRY(cudaEventSynchronize(e.ev[kStages]));
        const int p = e.precision == MPS_FP64 ? 0 : (e.precision == MPS_FP32 ? 1 : 2);
        for (int k = 0; k < kStages; ++k) {
            float t = 0.f;
            MPS_CUDA_TRY(cudaEventElapsedTime(&t, e.ev[k], e.ev[k + 1]));
            sys->stage_ms[p][k] += t;
        }
        sys->stage_count[p] += 1;
        sys->spare.push_back(e);
    }
    sys->pending.clear();
    for (int p = 0; p < 3; ++p) {
        for (int k = 0; k < kStages; ++k) ms[p * kStages + k] = sys->stage_ms[p][k];
        count[p] = sys->stage_count[p];
        for (int k = 0; k < kStages; ++k) sys->stage_ms[p][k] = 0.0;
        sys->stage_count[p] = 0;
    }
    return MPS_OK;
}

__global__ void k_field_combine(const double *__restrict__ wave, const double *__restrict__ real, int64_t total,
                                double *__restrict__ E) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        E[i] = -(wave[i] + real[i]);
}

extern "C" int mps_field_map(const double *x_e, int64_t n_e, const double *x_p, const double *p, int64_t n_p,
                             const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P,
                             const double *eta, const double *perp, const double *para, const double *rvals,
                             int64_t n_tab, int32_t with_real, double *E, mps_stream_t stream) {
    if (n_e < 0 || n_p < 0 || !box || !Ngrid || !eta || !(xi > 0) || !(rc > 0) || P < 1 || n_tab < 2) return MPS_BAD_ARG;
    if ((n_e > 0 && (!x_e || !E)) || (n_p > 0 && (!x_p || !p)) || !perp || !para || !rvals) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (Ngrid[d] < P || !(box[d] > 0)) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (rc > 0.5 * box[d]) return MPS_RC_GT_HALF_BOX;
    if (n_e == 0) return MPS_OK;
    configure_pool_once();
    cudaStream_t st = (cudaStream_t)stream;
    const GridParams gp = make_grid_params(Ngrid, box, xi, eta, P);
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    int32_t *start_p = nullptr, *start_e = nullptr;
    double *w_p = nullptr, *w_e = nullptr, *grid = nullptr, *spec = nullptr, *H = nullptr, *wave = nullptr,
           *real = nullptr;
    void *work = nullptr;
    auto cleanup = [&]() {
        void *ptrs[] = {start_p, start_e, w_p, w_e, grid, spec, H, wave, real, work};
        for (void *q : ptrs)
            if (q) cudaFreeAsync(q, st);
    };
    int rc_ = MPS_OK;
    rc_ = dalloc(&start_p, sizeof(int32_t) * 3 * (size_t)(n_p > 0 ? n_p : 1), st);
    if (!rc_) rc_ = dalloc(&w_p, sizeof(double) * 3 * (size_t)P * (n_p > 0 ? n_p : 1), st);
    if (!rc_) rc_ = dalloc(&start_e, sizeof(int32_t) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&w_e, sizeof(double) * 3 * (size_t)P * n_e, st);
    if (!rc_) rc_ = dalloc(&grid, sizeof(double) * 3 * (size_t)gp.G, st);
    if (!rc_) rc_ = dalloc(&spec, sizeof(double) * 2 * 3 * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&H, sizeof(double) * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&wave, sizeof(double) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&real, sizeof(double) * 3 * (size_t)n_e, st);
    // wave space: spread the source dipoles, D2Z, H k^k^ scale, Z2D, contract at the probes
    if (!rc_) rc_ = grid_geometry(x_p, n_p, gp, start_p, w_p, nullptr, st);
    if (!rc_) rc_ = spread<double>(p, n_p, 1, start_p, w_p, gp, grid, st);
    if (!rc_) rc_ = green_half(gp, H, nullptr, st);
    CachedPlan fwd{}, inv{};
    if (!rc_) rc_ = get_plan(CUFFT_D2Z, gp, 3, &fwd);
    if (!rc_) rc_ = get_plan(CUFFT_Z2D, gp, 3, &inv);
    if (!rc_) rc_ = dalloc(&work, std::max(fwd.work, inv.work) + 16, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(fwd.h, work) != CUFFT_SUCCESS || cufftSetStream(fwd.h, st) != CUFFT_SUCCESS ||
            cufftExecD2Z(fwd.h, (cufftDoubleReal *)grid, (cufftDoubleComplex *)spec) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) rc_ = scale_half<double>(spec, 1, gp, H, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(inv.h, work) != CUFFT_SUCCESS || cufftSetStream(inv.h, st) != CUFFT_SUCCESS ||
            cufftExecZ2D(inv.h, (cufftDoubleComplex *)spec, (cufftDoubleReal *)grid) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) rc_ = grid_geometry(x_e, n_e, gp, start_e, w_e, nullptr, st);
    if (!rc_) rc_ = contract<double>(grid, n_e, 1, start_e, w_e, gp, wave, st);
    // real space: sources within rc of each probe
    const bool do_real = with_real && n_p > 0;
    if (!rc_ && do_real) rc_ = probe_real_space(x_e, n_e, x_p, p, n_p, box, rc, perp, para, rvals, n_tab, real, st);
    if (!rc_ && !do_real && cudaMemsetAsync(real, 0, sizeof(double) * 3 * (size_t)n_e, st) != cudaSuccess)
        rc_ = MPS_CUDA_ERR;
    if (!rc_) {
        k_field_combine<<<grid_for(3 * n_e, 256), 256, 0, st>>>(wave, real, 3 * n_e, E);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc_ = MPS_CUDA_ERR;
    }
    cleanup();
    return rc_;
}

extern "C" int mps_field_map_quad(const double *x_e, int64_t n_e, const double *x_p, const double *sq, int64_t n_p,
                                  const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P,
                                  const double *eta, const double *tab9, const double *rvals, int64_t n_tab,
                                  int32_t with_real, double *EG, mps_stream_t stream) {
    if (n_e < 0 || n_p < 0 || !box || !Ngrid || !eta || !(xi > 0) || !(rc > 0) || P < 1 || n_tab < 2) return MPS_BAD_ARG;
    if ((n_e > 0 && (!x_e || !EG)) || (n_p > 0 && (!x_p || !sq)) || !tab9 || !rvals) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (Ngrid[d] < P || !(box[d] > 0)) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (rc > 0.5 * box[d]) return MPS_RC_GT_HALF_BOX;
    if (n_e == 0) return MPS_OK;
    configure_pool_once();
    cudaStream_t st = (cudaStream_t)stream;
    const GridParams gp = make_grid_params(Ngrid, box, xi, eta, P);
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    int32_t *start_p = nullptr, *start_e = nullptr;
    double *w_p = nullptr, *w_e = nullptr, *grid = nullptr, *spec = nullptr, *kc = nullptr, *wave = nullptr,
           *real = nullptr;
    void *work = nullptr;
    auto cleanup = [&]() {
        void *ptrs[] = {start_p, start_e, w_p, w_e, grid, spec, kc, wave, real, work};
        for (void *q : ptrs)
            if (q) cudaFreeAsync(q, st);
    };
    int rc_ = dalloc(&start_p, sizeof(int32_t) * 3 * (size_t)(n_p > 0 ? n_p : 1), st);
    if (!rc_) rc_ = dalloc(&w_p, sizeof(double) * 3 * (size_t)P * (n_p > 0 ? n_p : 1), st);
    if (!rc_) rc_ = dalloc(&start_e, sizeof(int32_t) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&w_e, sizeof(double) * 3 * (size_t)P * n_e, st);
    if (!rc_) rc_ = dalloc(&grid, sizeof(double) * 8 * (size_t)gp.G, st);
    if (!rc_) rc_ = dalloc(&spec, sizeof(double) * 2 * 8 * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&kc, sizeof(double) * 4 * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&wave, sizeof(double) * 8 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&real, sizeof(double) * 8 * (size_t)n_e, st);
    // wave space: the 8 source grids, D2Z, the dipole/quadrupole scale, Z2D, contract at the probes
    if (!rc_) rc_ = grid_geometry(x_p, n_p, gp, start_p, w_p, nullptr, st);
    if (!rc_ && n_p > 0) rc_ = spread_gen<double>(sq, n_p, 1, 8, start_p, w_p, gp, grid, st);
    if (!rc_ && n_p == 0 && cudaMemsetAsync(grid, 0, sizeof(double) * 8 * (size_t)gp.G, st) != cudaSuccess)
        rc_ = MPS_CUDA_ERR;
    if (!rc_) rc_ = quad_kcoef(gp, kc, nullptr, st);
    CachedPlan fwd{}, inv{};
    if (!rc_) rc_ = get_plan(CUFFT_D2Z, gp, 8, &fwd);
    if (!rc_) rc_ = get_plan(CUFFT_Z2D, gp, 8, &inv);
    if (!rc_) rc_ = dalloc(&work, std::max(fwd.work, inv.work) + 16, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(fwd.h, work) != CUFFT_SUCCESS || cufftSetStream(fwd.h, st) != CUFFT_SUCCESS ||
            cufftExecD2Z(fwd.h, (cufftDoubleReal *)grid, (cufftDoubleComplex *)spec) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) rc_ = scale_quad<double>(spec, 1, gp, kc, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(inv.h, work) != CUFFT_SUCCESS || cufftSetStream(inv.h, st) != CUFFT_SUCCESS ||
            cufftExecZ2D(inv.h, (cufftDoubleComplex *)spec, (cufftDoubleReal *)grid) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) rc_ = grid_geometry(x_e, n_e, gp, start_e, w_e, nullptr, st);
    if (!rc_) rc_ = contract_gen<double>(grid, n_e, 1, 8, start_e, w_e, gp, wave, st);
    const bool do_real = with_real && n_p > 0;
    if (!rc_ && do_real)
        rc_ = probe_real_space_quad(x_e, n_e, x_p, sq, n_p, box, rc, tab9, rvals, n_tab, real, st);
    if (!rc_ && !do_real && cudaMemsetAsync(real, 0, sizeof(double) * 8 * (size_t)n_e, st) != cudaSuccess)
        rc_ = MPS_CUDA_ERR;
    if (!rc_) {
        k_field_combine<<<grid_for(8 * n_e, 256), 256, 0, st>>>(wave, real, 8 * n_e, EG);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc_ = MPS_CUDA_ERR;
    }
    cleanup();
    return rc_;
}

__global__ void k_fill_value(double *__restrict__ a, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

extern "C" int mps_field_map_sizes(const double *x_e, int64_t n_e, const double *x_p, const double *radius,
                                   const int32_t *radius_class, int32_t n_class, const double *p, int64_t n_p,
                                   const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P,
                                   double eta, const double *perp, const double *para, const double *rvals,
                                   int64_t n_tab, int32_t with_real, double *E, mps_stream_t stream) {
    if (n_e < 0 || n_p < 1 || !box || !Ngrid || !(xi > 0) || !(rc > 0) || P < 1 || !(eta > 0) || n_tab < 2 ||
        n_class < 1)
        return MPS_BAD_ARG;
    if ((n_e > 0 && (!x_e || !E)) || !x_p || !p || !radius || !radius_class || !perp || !para || !rvals)
        return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (Ngrid[d] < P || !(box[d] > 0)) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (rc > 0.5 * box[d]) return MPS_RC_GT_HALF_BOX;
    if (n_e == 0) return MPS_OK;
    configure_pool_once();
    cudaStream_t st = (cudaStream_t)stream;
    const double eta3[3] = {eta, eta, eta};
    const GridParams gp = make_grid_params(Ngrid, box, xi, eta3, P);
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    const int64_t P3 = (int64_t)P * P * P;
    // probes are spheres of the smallest radius (Compute_Field_Sizes/ComputeField.m:33, RealSpace.m:7-8):
    // the class and radius of the particle with the smallest radius (first one on ties, as min does)
    std::vector<double> hr(n_p);
    std::vector<int32_t> hc(n_p);
    MPS_CUDA_TRY(cudaMemcpyAsync(hr.data(), radius, sizeof(double) * n_p, cudaMemcpyDeviceToHost, st));
    MPS_CUDA_TRY(cudaMemcpyAsync(hc.data(), radius_class, sizeof(int32_t) * n_p, cudaMemcpyDeviceToHost, st));
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    int64_t imin = 0;
    for (int64_t i = 1; i < n_p; ++i)
        if (hr[i] < hr[imin]) imin = i;
    const double a_min = hr[imin];
    const int32_t cmin = hc[imin];
    if (cmin < 0 || cmin >= n_class) return MPS_BAD_ARG;
    int32_t *start_p = nullptr, *start_e = nullptr;
    double *base_p = nullptr, *base_e = nullptr, *g_p = nullptr, *g_e = nullptr, *rad_e = nullptr, *grid = nullptr,
           *spec = nullptr, *hcoef = nullptr, *wave = nullptr, *real = nullptr;
    void *work = nullptr;
    auto cleanup = [&]() {
        void *ptrs[] = {start_p, start_e, base_p, base_e, g_p, g_e, rad_e, grid, spec, hcoef, wave, real, work};
        for (void *q : ptrs)
            if (q) cudaFreeAsync(q, st);
    };
    int rc_ = dalloc(&start_p, sizeof(int32_t) * 3 * (size_t)n_p, st);
    if (!rc_) rc_ = dalloc(&base_p, sizeof(double) * 3 * (size_t)n_p, st);
    if (!rc_) rc_ = dalloc(&g_p, sizeof(double) * (size_t)(n_p * P3), st);
    if (!rc_) rc_ = dalloc(&start_e, sizeof(int32_t) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&base_e, sizeof(double) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&g_e, sizeof(double) * (size_t)(n_e * P3), st);
    if (!rc_) rc_ = dalloc(&rad_e, sizeof(double) * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&grid, sizeof(double) * (size_t)gp.G, st);
    if (!rc_) rc_ = dalloc(&spec, sizeof(double) * 2 * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&hcoef, sizeof(double) * (size_t)Gc, st);
    if (!rc_) rc_ = dalloc(&wave, sizeof(double) * 3 * (size_t)n_e, st);
    if (!rc_) rc_ = dalloc(&real, sizeof(double) * 3 * (size_t)n_e, st);
    // wave space: scalar grid of the sources, D2Z, exp(-(1-eta) q^2/4 xi^2)/q^2, Z2D, contract at the probes
    if (!rc_) rc_ = cs_geometry(x_p, n_p, gp, radius, xi, eta, start_p, base_p, g_p, nullptr, st);
    if (!rc_) rc_ = spread_cs<double>(p, n_p, 1, start_p, base_p, g_p, gp, grid, st);
    if (!rc_) rc_ = cs_green(gp, eta, xi, hcoef, nullptr, st);
    CachedPlan fwd{}, inv{};
    if (!rc_) rc_ = get_plan(CUFFT_D2Z, gp, 1, &fwd);
    if (!rc_) rc_ = get_plan(CUFFT_Z2D, gp, 1, &inv);
    if (!rc_) rc_ = dalloc(&work, std::max(fwd.work, inv.work) + 16, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(fwd.h, work) != CUFFT_SUCCESS || cufftSetStream(fwd.h, st) != CUFFT_SUCCESS ||
            cufftExecD2Z(fwd.h, (cufftDoubleReal *)grid, (cufftDoubleComplex *)spec) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) rc_ = scale_cs<double>(spec, 1, gp, hcoef, st);
    if (!rc_) {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        if (cufftSetWorkArea(inv.h, work) != CUFFT_SUCCESS || cufftSetStream(inv.h, st) != CUFFT_SUCCESS ||
            cufftExecZ2D(inv.h, (cufftDoubleComplex *)spec, (cufftDoubleReal *)grid) != CUFFT_SUCCESS)
            rc_ = MPS_CUFFT_ERR;
    }
    if (!rc_) {
        k_fill_value<<<grid_for(n_e, 256), 256, 0, st>>>(rad_e, n_e, a_min);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc_ = MPS_CUDA_ERR;
    }
    if (!rc_) rc_ = cs_geometry(x_e, n_e, gp, rad_e, xi, eta, start_e, base_e, g_e, nullptr, st);
    if (!rc_) rc_ = contract_cs<double>(grid, n_e, 1, start_e, base_e, g_e, gp, wave, st);
    if (!rc_ && with_real)
        rc_ = probe_real_space_cs(x_e, n_e, x_p, p, radius_class, cmin, n_class, n_p, box, rc, perp, para, rvals,
                                  n_tab, real, st);
    if (!rc_ && !with_real && cudaMemsetAsync(real, 0, sizeof(double) * 3 * (size_t)n_e, st) != cudaSuccess)
        rc_ = MPS_CUDA_ERR;
    if (!rc_) {
        k_field_combine<<<grid_for(3 * n_e, 256), 256, 0, st>>>(wave, real, 3 * n_e, E);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc_ = MPS_CUDA_ERR;
    }
    cleanup();
    return rc_;
}

extern "C" int mps_kspace_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_green_mu);
    g_green.clear();   // systems that hold coefficients keep them until they are destroyed
    return MPS_OK;
}

extern "C" int mps_system_graphs(const mps_system *sys, int32_t *built, int32_t *failed) {
    if (!sys || !built || !failed) return MPS_BAD_ARG;
    *built = *failed = 0;
    for (const auto &g : sys->graphs) {
        if (g.exec) ++*built;
        if (g.failed) ++*failed;
    }
    return MPS_OK;
}

extern "C" int mps_system_tuning(const mps_system *sys, int32_t *tile_depth, float *ms) {
    if (!sys || !tile_depth || !ms) return MPS_BAD_ARG;
    tile_depth[0] = sys->tb64.tz;
    tile_depth[1] = sys->inner ? sys->inner->tb.tz : (sys->tbg.mem ? sys->tbg.tz : sys->tb32.tz);
    for (int p = 0; p < 2; ++p) {
        TuneKey key;
        memset(&key, 0, sizeof(key));
        key.dev = current_device();
        for (int k = 0; k < 3; ++k) key.N[k] = sys->gp.N[k];
        key.P = sys->gp.P;
        key.use = p == 1 && sys->tbg.mem ? (int)kTileGrad32 : sys->tb_use[p];
        key.nrhs = sys->max_rhs < 3 ? sys->max_rhs : 3;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        ms[2 * p] = it != g_tune.end() ? it->second.ms[0] : -1.f;
        ms[2 * p + 1] = it != g_tune.end() ? it->second.ms[1] : -1.f;
    }
    return MPS_OK;
}

extern "C" int mps_adjoint_forces(mps_system *sys, const double *m, const double *perp, const double *para,
                                  const double *rvals, int64_t n_tab, int32_t diag_index, double *forces,
                                  double *dE_deps, mps_stream_t stream) {
    if (!sys || !m || !perp || !para || !rvals || n_tab < 2 || !forces) return MPS_BAD_ARG;
    if (sys->kind != MPS_DIPOLE || sys->cplx) return MPS_BAD_ARG;
    if (diag_index < 0 || diag_index >= sys->n_diag) return MPS_BAD_ARG;
    MPS_TRY(build_status(sys));
    cudaStream_t st = (cudaStream_t)stream;
    MPS_TRY(ensure_p64(sys, st));
    const int64_t n = sys->n;
    int *err = nullptr;
    MPS_TRY(dalloc(&err, sizeof(int), st));
    int rc = MPS_OK;
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) rc = MPS_CUDA_ERR;
    if (!rc) rc = rs_force(m, n, sys->row_ptr, sys->p64, perp, para, rvals, n_tab, forces, err, st);
    // wave space: phi = IFFT(scale(FFT(spread(m)))), float64-accurate, then the weight-gradient contraction.
    // Grids the double-float FFTs support take the double-float pipeline (float64 issue is slow on GB300) and
    // convert phi to float64 in place; the others use the float64 spread and cuFFT.
    if (!rc && df_usable(sys)) {
        bool tiles_used = false;
        rc = df_field_grids(sys, m, 1, nullptr, st, &tiles_used);
        if (!rc) rc = dfv_to_f64_inplace(sys->grid64, 3 * sys->gp.G, st);
    } else if (!rc) {
        rc = ensure_grids(sys, MPS_FP64, st);
        if (!rc) rc = spread<double>(m, n, 1, sys->start, sys->w64, sys->gp, sys->grid64, st);
        if (!rc) rc = exec_plan(sys, CUFFT_D2Z, 3, sys->grid64, sys->spec64, 0, st);
        if (!rc) rc = scale_half<double>(sys->spec64, 1, sys->gp, sys->h64, st);
        if (!rc) rc = exec_plan(sys, CUFFT_Z2D, 3, sys->spec64, sys->grid64, 0, st);
    }
    if (!rc) rc = wave_force(sys->grid64, sys->x, m, n, sys->start, sys->w64, sys->gp, forces, st);
    if (!rc && dE_deps) {
        double self = 0.0;
        if (cudaMemcpyAsync(&self, perp, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = MPS_CUDA_ERR;
        if (!rc) rc = eps_grad(m, sys->diag + (int64_t)diag_index * n, self, n, dE_deps, st);
    }
    int herr = 0;
    if (!rc && cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = MPS_CUDA_ERR;
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = MPS_CUDA_ERR;
    cudaFreeAsync(err, st);
    if (!rc && herr) rc = MPS_TABLE_RANGE;
    return rc;
}
