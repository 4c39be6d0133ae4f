// Status strings, last-error record and a three-phase exclusive scan.
#include <stdio.h>

#include <atomic>
#include <string.h>

#include "common.cuh"

namespace mps {

static char g_last_error[512] = "";
static std::atomic<unsigned long long> g_launches{0};

static thread_local long long t_captured = -1;   // >= 0 while this thread captures a graph

void count_launch() {
    if (t_captured >= 0) {
        ++t_captured;
        return;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void capture_count_begin() { t_captured = 0; }
long long capture_count_end() {
    const long long c = t_captured;
    t_captured = -1;
    return c < 0 ? 0 : c;
}
void add_launches(long long k) {
    if (k > 0) g_launches.fetch_add((unsigned long long)k, std::memory_order_relaxed);
}

void set_last_error(cudaError_t e, const char *what, const char *file, int line) {
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

// ---------------------------------------------------------------------------
// Exclusive scan.  Tile = 1024 threads x 4 items.  Phase 1 writes tile sums,
// phase 2 scans the tile sums in one block (looping over chunks), phase 3
// rescans each tile with its offset.  Deterministic.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

template <typename Tin>
__device__ __forceinline__ int64_t load_or_zero(const Tin *in, int64_t i, int64_t n) {
    return i < n ? (int64_t)in[i] : 0;
}

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *sm, int64_t *total) {
    // sm: 32 entries
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) sm[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int64_t s = (lane < (int)(blockDim.x >> 5)) ? sm[lane] : 0;
        int64_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        sm[lane] = si - s;  // exclusive warp offsets
        if (lane == 31) sm[32] = si;
    }
    __syncthreads();
    int64_t res = inc - v + sm[wid];
    if (total) *total = sm[32];
    __syncthreads();
    return res;
}

template <typename Tin>
__global__ void k_scan_tiles(const Tin *in, int64_t n, int64_t *tile_sums) {
    __shared__ int64_t sm[33];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) s += load_or_zero(in, base + k, n);
    int64_t tot;
    block_exclusive_scan(s, sm, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int64_t *tile_sums, int64_t ntiles) {
    __shared__ int64_t sm[33];
    int64_t carry = 0;
    for (int64_t c = 0; c < ntiles; c += blockDim.x) {
        int64_t i = c + threadIdx.x;
        int64_t v = i < ntiles ? tile_sums[i] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_scan(v, sm, &tot);
        if (i < ntiles) tile_sums[i] = ex + carry;
        carry += tot;
    }
}

template <typename Tin>
__global__ void k_scan_apply(const Tin *in, int64_t *out, int64_t n, const int64_t *tile_off) {
    __shared__ int64_t sm[33];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = load_or_zero(in, base + k, n);
        s += v[k];
    }
    int64_t ex = block_exclusive_scan(s, sm, nullptr) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
}

size_t scan_workspace(int64_t n) {
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    return (size_t)(ntiles + 1) * sizeof(int64_t);
}

template <typename Tin>
static int scan_impl(const Tin *in, int64_t *out, int64_t n, void *tmp, cudaStream_t s) {
    if (n <= 0) return MPS_OK;
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    int64_t *sums = (int64_t *)tmp;
    k_scan_tiles<Tin><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums);
    MPS_LAUNCH_CHECK();
    k_scan_sums<<<1, kScanThreads, 0, s>>>(sums, ntiles);
    MPS_LAUNCH_CHECK();
    k_scan_apply<Tin><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, sums);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, void *tmp, cudaStream_t s) {
    return scan_impl<int64_t>(in, out, n, tmp, s);
}

int exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, void *tmp, cudaStream_t s) {
    return scan_impl<int32_t>(in, out, n, tmp, s);
}

}  // namespace mps

extern "C" const char *mps_status_string(int status) {
    switch (status) {
        case MPS_OK: return "ok";
        case MPS_BAD_ARG: return "bad argument";
        case MPS_RC_GT_HALF_BOX: return "real-space cutoff exceeds half the box size";
        case MPS_TABLE_RANGE: return "pair separation outside the real-space table";
        case MPS_NOT_CONVERGED: return "GMRES did not converge";
        case MPS_CUDA_ERR: return mps::g_last_error[0] ? mps::g_last_error : "CUDA error";
        case MPS_CUFFT_ERR: return "cuFFT error";
        case MPS_NO_MEMORY: return "out of device memory";
        case MPS_SCRATCH_LIMIT:
            return "input exceeds the fixed no-allocation scratch, or the outputs are too small for the pair count";
        default: return "unknown status";
    }
}

extern "C" int mps_abi_version(void) { return 5; }

extern "C" uint64_t mps_kernel_launches(void) { return (uint64_t)mps::g_launches.load(); }
