// Neighbour-list build for callers that must not allocate device memory.
//
// Who needs this: code that calls into this library from inside a host
// application's time step, where the application owns all device memory and
// forbids allocation while it runs.  Examples are MD engines invoking a field
// or force plugin every step, and embedded C callers working under a fixed
// memory budget.  cudaMalloc/cudaFree synchronise the whole device and can
// fail half-way through a run, so such callers cannot use the entry points
// that take a caller-sized workspace or allocate one internally.
//
// This variant keeps its scratch (cell bins, per-slot counts and offsets, scan
// partials) in one fixed, file-scope device array.  It performs no
// allocation.  It calls no cudaMalloc, no cudaFree and no allocating library
// routine.  The array is MPS_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that
// loads this library, and it stays resident until the process exits.
//
// Set-up: the first call made on a device looks up that device's copy of the
// array (cudaGetSymbolAddress) with the device current and caches the address.
// Make that first call on each device before any stream capture begins.
//
// Sharing: every call uses the same array and leaves its contents in place.
// The counts that must start at zero are cleared by the build on every call.
// Two calls whose GPU work overlaps (different streams or host threads, same
// device) race on the array; serialise them.
#include <mutex>

#include "common.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[MPS_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of this device's scratch array, looked up once per device.
int scratch_for_current_device(void **out) {
    int dev = -1;
    MPS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return MPS_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        MPS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return MPS_OK;
}
}  // namespace

extern "C" int mps_neighbor_list_noalloc(const int64_t *cell, int64_t n, const int64_t *ncell, int64_t *p1,
                                         int64_t *p2, int64_t max_pairs, int64_t *n_pairs, mps_stream_t stream) {
    if (!n_pairs || !ncell || n < 0 || max_pairs < 0) return MPS_BAD_ARG;
    *n_pairs = 0;
    for (int d = 0; d < 3; ++d)
        if (ncell[d] < 1) return MPS_BAD_ARG;
    if (n == 0) return MPS_OK;
    // size checks first: nothing touches the GPU for an input that cannot fit.  Cell counts whose
    // product would overflow (or exceed the kernels' int32 cell index) are bad input, not a size
    // that merely misses the scratch.
    const size_t need = mps_neighbor_list_workspace(n, ncell);
    if (need == SIZE_MAX) return MPS_BAD_ARG;
    if (need > (size_t)MPS_NOALLOC_SCRATCH_BYTES) return MPS_SCRATCH_LIMIT;
    void *ws = nullptr;
    int rc = scratch_for_current_device(&ws);
    if (rc != MPS_OK) return rc;
    rc = mps_neighbor_list_count(cell, n, ncell, ws, need, n_pairs, stream);
    if (rc != MPS_OK) return rc;
    if (*n_pairs > max_pairs) return MPS_SCRATCH_LIMIT;  // outputs too small: *n_pairs says how many are needed
    if (*n_pairs == 0) return MPS_OK;
    return mps_neighbor_list_fill(cell, n, ncell, ws, need, p1, p2, stream);
}
