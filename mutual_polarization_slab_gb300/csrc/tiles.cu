// Tiled spread (K4) and contract (K6).
//
// The grid is cut into 16 x 16 x TZ tiles, one CTA per tile.  Every particle is
// binned (counting sort, ids ascending inside a tile) into each tile its P^3
// stencil touches.
//   spread:   thread (tx,ty) owns the TZ nodes of its column and accumulates
//             them in registers over the tile's particles, then writes them
//             once -- every grid node is written by exactly one thread, so no
//             atomics and no zero-fill, and the summation order is fixed.
//   contract: the CTA stages its grid tile in shared memory; one warp per
//             (particle, tile) entry sums the stencil nodes inside the tile
//             into a partial; a gather kernel adds each particle's partials in
//             a fixed order.
// Both produce the same sums as the reference's per-particle loops
// (EW/ewald.py:370-467) up to summation order.
#include "tiles.cuh"

#include <climits>
#include <algorithm>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include "dfloat.cuh"

namespace mps {

constexpr int kMaxTileList = 8;  // distinct tiles per axis touched by one stencil (ceil((P-1)/T)+2)
// particles staged per spread iteration (one barrier interval): 96 measured 1.42 ms for the double-float spread
// at the bench workload against 1.57 for 32 and 1.46 for 64 (fewer barriers; the warps' shares even out)
constexpr int kChunk = 96;

bool tiles_supported(const GridParams &gp, int tz) {
    if (gp.P > kMaxP || gp.P < 1) return false;
    if (gp.N[0] < kTileX || gp.N[1] < kTileY || gp.N[2] < tz) return false;
    if ((gp.P - 1 + tz - 1) / tz + 2 > kMaxTileList) return false;
    return true;
}

// Distinct tiles of one axis touched by indices (s + j) mod N, j < P, in order of first touch.
__device__ __forceinline__ int axis_tiles(int s, int P, int N, int T, int *out) {
    int cnt = 0;
    for (int j = 0; j < P; ++j) {
        int idx = s + j;
        if (idx >= N) idx -= N;
        const int t = idx / T;
        bool seen = false;
        for (int k = 0; k < cnt; ++k) seen |= (out[k] == t);
        if (!seen) out[cnt++] = t;
    }
    return cnt;
}

struct TileGeom {
    int N[3];
    int T[3];
    int nt[3];
    int P;
};

__global__ void k_tile_count(const int32_t *__restrict__ start, int64_t n, TileGeom tg, int32_t *__restrict__ tcount,
                             int64_t *__restrict__ pcount) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        int L[3][kMaxTileList];
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = axis_tiles(start[3 * a + d], tg.P, tg.N[d], tg.T[d], L[d]);
        for (int iz = 0; iz < c[2]; ++iz)
            for (int iy = 0; iy < c[1]; ++iy)
                for (int ix = 0; ix < c[0]; ++ix)
                    atomicAdd(&tcount[((int64_t)L[2][iz] * tg.nt[1] + L[1][iy]) * tg.nt[0] + L[0][ix]], 1);
        pcount[a] = (int64_t)c[0] * c[1] * c[2];
    }
}

__global__ void k_tile_fill(const int32_t *__restrict__ start, int64_t n, TileGeom tg,
                            const int64_t *__restrict__ tstart, int32_t *__restrict__ cursor,
                            int32_t *__restrict__ unsorted) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        int L[3][kMaxTileList];
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = axis_tiles(start[3 * a + d], tg.P, tg.N[d], tg.T[d], L[d]);
        for (int iz = 0; iz < c[2]; ++iz)
            for (int iy = 0; iy < c[1]; ++iy)
                for (int ix = 0; ix < c[0]; ++ix) {
                    const int64_t t = ((int64_t)L[2][iz] * tg.nt[1] + L[1][iy]) * tg.nt[0] + L[0][ix];
                    unsorted[tstart[t] + atomicAdd(&cursor[t], 1)] = (int32_t)a;
                }
    }
}

// One block per tile: order the tile's particles by id (bitonic sort in shared
// memory for up to kSortCap entries, else a rank count over the whole list).  The
// atomics of k_tile_fill leave the unsorted order arbitrary; the sorted order makes
// every tiled kernel's sums deterministic.
constexpr int kSortCap = 4096;

// Where particle v's entry for tile (tx, ty, tzi) landed: pentry[pstart[v] + its index in v's tile order] = pos.
__device__ __forceinline__ void tile_pentry_out(int32_t v, int64_t pos, int tx, int ty, int tzi,
                                                const int32_t *__restrict__ start, const TileGeom &tg,
                                                const int64_t *__restrict__ pstart, int32_t *__restrict__ pentry) {
    int L[3][kMaxTileList];
    int c[3];
    for (int d = 0; d < 3; ++d) c[d] = axis_tiles(start[3 * (int64_t)v + d], tg.P, tg.N[d], tg.T[d], L[d]);
    int ix = 0, iy = 0, iz = 0;
    while (ix < c[0] && L[0][ix] != tx) ++ix;
    while (iy < c[1] && L[1][iy] != ty) ++iy;
    while (iz < c[2] && L[2][iz] != tzi) ++iz;
    pentry[pstart[v] + ((int64_t)iz * c[1] + iy) * c[0] + ix] = (int32_t)pos;
}

template <int TPB>
__global__ void __launch_bounds__(TPB) k_tile_sort(const int32_t *__restrict__ unsorted,
                                                   const int64_t *__restrict__ tstart, int64_t ntiles,
                                                   int32_t *__restrict__ entries) {
    __shared__ int32_t key[kSortCap];
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t s0 = tstart[t];
        const int len = (int)(tstart[t + 1] - s0);
        if (len == 0) continue;
        if (len <= kSortCap) {
            int L = 1;
            while (L < len) L <<= 1;
            __syncthreads();   // the previous tile's reads of key are done
            for (int i = threadIdx.x; i < L; i += blockDim.x) key[i] = i < len ? unsorted[s0 + i] : INT_MAX;
            __syncthreads();
            for (int k = 2; k <= L; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = threadIdx.x; i < L; i += blockDim.x) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const int32_t a = key[i], b = key[ixj];
                            if ((a > b) == ((i & k) == 0)) {
                                key[i] = b;
                                key[ixj] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            for (int e = threadIdx.x; e < len; e += blockDim.x) entries[s0 + e] = key[e];
        } else {
            // ids are distinct within a tile: an entry's rank is the count of smaller ids
            for (int e = threadIdx.x; e < len; e += blockDim.x) {
                const int32_t v = unsorted[s0 + e];
                int rank = 0;
                for (int j = 0; j < len; ++j) rank += (unsorted[s0 + j] < v);
                entries[s0 + rank] = v;
            }
        }
    }
}

// out[n] = out[n - 1] + in[n - 1]: the total after an exclusive scan of n >= 1 counts.
template <typename Tin>
__global__ void k_scan_total(const Tin *__restrict__ in, int64_t *__restrict__ out, int64_t n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = out[n - 1] + (int64_t)in[n - 1];
}

static char *carve_t(char *&p, size_t bytes) {
    uintptr_t u = ((uintptr_t)p + 255) & ~(uintptr_t)255;
    p = (char *)(u + bytes);
    return (char *)u;
}

// Upper bound of the distinct tiles along one axis that P consecutive nodes (mod N) touch: a window of P nodes
// spans at most (P - 1) / T + 2 tiles of T, one more where it wraps past a partial last tile.
static int64_t axis_tile_bound(int N, int T, int P) {
    const int64_t nt = (N + T - 1) / T;
    return std::min<int64_t>(nt, (P - 1) / T + 2 + (N % T != 0 ? 1 : 0));
}

// Tile lists without a host round trip: the entry arrays are sized by the per-particle bound (nentries holds that
// capacity), the offsets and totals stay on the device.
int tile_bins_build(const int32_t *start, int64_t n, const GridParams &gp, int tz, TileBins &tb, cudaStream_t s) {
    tile_bins_free(tb, s);
    if (!tiles_supported(gp, tz) || n < 1) return MPS_BAD_ARG;
    TileGeom tg;
    tg.P = gp.P;
    tg.T[0] = kTileX;
    tg.T[1] = kTileY;
    tg.T[2] = tz;
    int64_t per = 1;
    for (int d = 0; d < 3; ++d) {
        tg.N[d] = gp.N[d];
        tg.nt[d] = (gp.N[d] + tg.T[d] - 1) / tg.T[d];
        per *= axis_tile_bound(gp.N[d], tg.T[d], gp.P);
    }
    tb.tz = tz;
    tb.ntx = tg.nt[0];
    tb.nty = tg.nt[1];
    tb.ntz = tg.nt[2];
    tb.ntiles = (int64_t)tg.nt[0] * tg.nt[1] * tg.nt[2];
    const int64_t T = tb.ntiles;
    const int64_t Emax = n * per;
    tb.nentries = Emax;
    // temporaries: tile counts and cursors, per-particle counts, scan scratch, the unsorted lists
    size_t tmp_bytes = 256 * 5 + (size_t)T * 4 * 2 + (size_t)n * 8 + scan_workspace(std::max(T, n) + 1) +
                       (size_t)Emax * 4;
    char *tmp = nullptr;
    MPS_CUDA_TRY(cudaMallocAsync((void **)&tmp, tmp_bytes, s));
    char *p = tmp;
    int32_t *tcount = (int32_t *)carve_t(p, (size_t)T * 4);
    int32_t *cursor = (int32_t *)carve_t(p, (size_t)T * 4);
    int64_t *pcount = (int64_t *)carve_t(p, (size_t)n * 8);
    void *scan_tmp = carve_t(p, scan_workspace(std::max(T, n) + 1));
    int32_t *unsorted = (int32_t *)carve_t(p, (size_t)Emax * 4);
    // persistent arrays
    size_t bytes = 256 * 4 + (size_t)(T + 1) * 8 + (size_t)Emax * 4 + (size_t)(n + 1) * 8 + (size_t)Emax * 4;
    MPS_CUDA_TRY(cudaMallocAsync(&tb.mem, bytes, s));
    p = (char *)tb.mem;
    tb.tile_start = (int64_t *)carve_t(p, (size_t)(T + 1) * 8);
    tb.entries = (int32_t *)carve_t(p, (size_t)Emax * 4);
    tb.pstart = (int64_t *)carve_t(p, (size_t)(n + 1) * 8);
    tb.pentry = (int32_t *)carve_t(p, (size_t)Emax * 4);
    MPS_CUDA_TRY(cudaMemsetAsync(tcount, 0, (size_t)T * 4, s));
    MPS_CUDA_TRY(cudaMemsetAsync(cursor, 0, (size_t)T * 4, s));
    k_tile_count<<<grid_for(n, 256), 256, 0, s>>>(start, n, tg, tcount, pcount);
    MPS_LAUNCH_CHECK();
    int r = exclusive_scan_i32_to_i64(tcount, tb.tile_start, T, scan_tmp, s);
    if (r) return r;
    k_scan_total<int32_t><<<1, 32, 0, s>>>(tcount, tb.tile_start, T);
    MPS_LAUNCH_CHECK();
    r = exclusive_scan_i64(pcount, tb.pstart, n, scan_tmp, s);
    if (r) return r;
    k_scan_total<int64_t><<<1, 32, 0, s>>>(pcount, tb.pstart, n);
    MPS_LAUNCH_CHECK();
    k_tile_fill<<<grid_for(n, 256), 256, 0, s>>>(start, n, tg, tb.tile_start, cursor, unsorted);
    MPS_LAUNCH_CHECK();
    // one block per tile; 128 threads where the tiles average a few hundred entries (depth-4 tiles), 256 for longer
    const unsigned tblocks = (unsigned)std::min<int64_t>(T, INT32_MAX);
    if (Emax / T <= 512)
        k_tile_sort<128><<<tblocks, 128, 0, s>>>(unsorted, tb.tile_start, T, tb.entries);
    else
        k_tile_sort<256><<<tblocks, 256, 0, s>>>(unsorted, tb.tile_start, T, tb.entries);
    MPS_LAUNCH_CHECK();
    cudaFreeAsync(tmp, s);
    return MPS_OK;
}

// A warp per tile: for each of its (sorted) entries, where it sits in the particle's own list.
__global__ void k_tile_pentry(const int64_t *__restrict__ tstart, int64_t ntiles, const int32_t *__restrict__ entries,
                              const int32_t *__restrict__ start, TileGeom tg, const int64_t *__restrict__ pstart,
                              int32_t *__restrict__ pentry) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nw) {
        const int tx = (int)(t % tg.nt[0]), ty = (int)((t / tg.nt[0]) % tg.nt[1]),
                  tzi = (int)(t / ((int64_t)tg.nt[0] * tg.nt[1]));
        for (int64_t e = tstart[t] + lane; e < tstart[t + 1]; e += 32)
            tile_pentry_out(entries[e], e, tx, ty, tzi, start, tg, pstart, pentry);
    }
}

int tile_bins_pentry(const int32_t *start, const GridParams &gp, TileBins &tb, cudaStream_t s) {
    if (tb.has_pentry || !tb.mem) return MPS_OK;
    TileGeom tg;
    tg.P = gp.P;
    tg.T[0] = kTileX;
    tg.T[1] = kTileY;
    tg.T[2] = tb.tz;
    for (int d = 0; d < 3; ++d) {
        tg.N[d] = gp.N[d];
        tg.nt[d] = (gp.N[d] + tg.T[d] - 1) / tg.T[d];
    }
    k_tile_pentry<<<grid_for(tb.ntiles * 32, 256), 256, 0, s>>>(tb.tile_start, tb.ntiles, tb.entries, start, tg,
                                                               tb.pstart, tb.pentry);
    MPS_LAUNCH_CHECK();
    tb.has_pentry = true;
    return MPS_OK;
}

__device__ __forceinline__ int64_t home_block(const int32_t *__restrict__ start, int64_t a, int nbx, int nby) {
    return ((int64_t)(start[3 * a + 2] / kHomeBlock) * nby + start[3 * a + 1] / kHomeBlock) * nbx +
           start[3 * a] / kHomeBlock;
}

__global__ void k_home_count(const int32_t *__restrict__ start, int64_t n, int nbx, int nby,
                             int32_t *__restrict__ count) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&count[home_block(start, a, nbx, nby)], 1);
}

// The order inside a block is that of the atomics; each particle's sum does not depend on it.
__global__ void k_home_fill(const int32_t *__restrict__ start, int64_t n, int nbx, int nby,
                            const int64_t *__restrict__ hstart, int32_t *__restrict__ cursor,
                            int32_t *__restrict__ hentries) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = home_block(start, a, nbx, nby);
        hentries[hstart[b] + atomicAdd(&cursor[b], 1)] = (int32_t)a;
    }
}

int tile_bins_home(const int32_t *start, int64_t n, const GridParams &gp, TileBins &tb, cudaStream_t s) {
    if (tb.has_home) return MPS_OK;
    if (n < 1) return MPS_BAD_ARG;
    int64_t H = 1;
    for (int d = 0; d < 3; ++d) {
        tb.nhb[d] = (int)((gp.N[d] + kHomeBlock - 1) / kHomeBlock);
        H *= tb.nhb[d];
    }
    tb.nhome = H;
    size_t tmp_bytes = 256 * 3 + (size_t)H * 4 * 2 + scan_workspace(H + 1);
    char *tmp = nullptr;
    MPS_CUDA_TRY(cudaMallocAsync((void **)&tmp, tmp_bytes, s));
    char *p = tmp;
    int32_t *count = (int32_t *)carve_t(p, (size_t)H * 4);
    int32_t *cursor = (int32_t *)carve_t(p, (size_t)H * 4);
    void *scan_tmp = carve_t(p, scan_workspace(H + 1));
    MPS_CUDA_TRY(cudaMallocAsync(&tb.hmem, 256 * 2 + (size_t)(H + 1) * 8 + (size_t)n * 4, s));
    p = (char *)tb.hmem;
    tb.hstart = (int64_t *)carve_t(p, (size_t)(H + 1) * 8);
    tb.hentries = (int32_t *)carve_t(p, (size_t)n * 4);
    MPS_CUDA_TRY(cudaMemsetAsync(count, 0, (size_t)H * 4, s));
    MPS_CUDA_TRY(cudaMemsetAsync(cursor, 0, (size_t)H * 4, s));
    k_home_count<<<grid_for(n, 256), 256, 0, s>>>(start, n, tb.nhb[0], tb.nhb[1], count);
    MPS_LAUNCH_CHECK();
    int r = exclusive_scan_i32_to_i64(count, tb.hstart, H, scan_tmp, s);
    if (r) return r;
    k_scan_total<int32_t><<<1, 32, 0, s>>>(count, tb.hstart, H);
    MPS_LAUNCH_CHECK();
    k_home_fill<<<grid_for(n, 256), 256, 0, s>>>(start, n, tb.nhb[0], tb.nhb[1], tb.hstart, cursor, tb.hentries);
    MPS_LAUNCH_CHECK();
    cudaFreeAsync(tmp, s);
    tb.has_home = true;
    return MPS_OK;
}

void tile_bins_free(TileBins &tb, cudaStream_t s) {
    if (tb.mem) cudaFreeAsync(tb.mem, s);
    if (tb.hmem) cudaFreeAsync(tb.hmem, s);
    tb = TileBins();
}

// ---------------------------------------------------------------------------
// Spread
// ---------------------------------------------------------------------------
// T: accumulation arithmetic (float, double, or the double-float dfv);
// TW: stored weight type; TG: grid element type.
template <typename T, int TZ, int NR, typename TW = T, typename TG = T>
__global__ void __launch_bounds__(256) k_spread_tiled(const double *__restrict__ m, int64_t n, int r0,
                                                      const int32_t *__restrict__ start, const TW *__restrict__ w,
                                                      GridParams gp, const int64_t *__restrict__ tstart,
                                                      const int32_t *__restrict__ entries, int ntx, int nty,
                                                      TG *__restrict__ grid) {
    constexpr int C = 3 * NR;
    __shared__ int3 s_off[kChunk];
    __shared__ T s_w[kChunk][3 * kMaxP];
    __shared__ T s_m[kChunk][C];
    const int64_t t = blockIdx.x;
    const int bx = (int)(t % ntx), by = (int)((t / ntx) % nty), bz = (int)(t / ((int64_t)ntx * nty));
    const int X0 = bx * kTileX, Y0 = by * kTileY, Z0 = bz * TZ;
    // warp w owns the 8 x 4 patch (columns 8 (w & 1) .. +8, rows 4 (w >> 1) .. +4) of the 16 x 16 tile: a particle
    // whose stencil misses the patch costs the warp one uniform branch (with two full 16-wide rows per warp, every
    // warp whose rows the particle reaches would run it, however few of the columns it covers)
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tx = 8 * (wid & 1) + (lane & 7), ty = 4 * (wid >> 1) + (lane >> 3);
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    ProdAcc<T> acc[TZ][C];
#pragma unroll
    for (int z = 0; z < TZ; ++z)
#pragma unroll
        for (int c = 0; c < C; ++c) acc[z][c].zero();
    const int64_t e0 = tstart[t], e1 = tstart[t + 1];
    for (int64_t cb = e0; cb < e1; cb += kChunk) {
        const int cnt = (int)min((int64_t)kChunk, e1 - cb);
        if (threadIdx.x < cnt) {
            const int32_t a = entries[cb + threadIdx.x];
            int ox = X0 - start[3 * a], oy = Y0 - start[3 * a + 1], oz = Z0 - start[3 * a + 2];
            if (ox < 0) ox += Nx;
            if (oy < 0) oy += Ny;
            if (oz < 0) oz += Nz;
            s_off[threadIdx.x] = make_int3(ox, oy, oz);
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const double *ma = m + ((int64_t)(r0 + r) * n + a) * 3;
                s_m[threadIdx.x][3 * r + 0] = (T)ma[0];
                s_m[threadIdx.x][3 * r + 1] = (T)ma[1];
                s_m[threadIdx.x][3 * r + 2] = (T)ma[2];
            }
        }
        for (int q = threadIdx.x; q < cnt * 3 * P; q += blockDim.x) {
            const int pp = q / (3 * P), k = q % (3 * P);
            const int32_t a = entries[cb + pp];
            s_w[pp][(k / P) * kMaxP + (k % P)] = (T)w[(int64_t)a * 3 * P + k];
        }
        __syncthreads();
        for (int pp = 0; pp < cnt; ++pp) {
            const int3 o = s_off[pp];
            int dx = o.x + tx;
            if (dx >= Nx) dx -= Nx;
            int dy = o.y + ty;
            if (dy >= Ny) dy -= Ny;
            if (dx < P && dy < P) {
                const T wxy = s_w[pp][dx] * s_w[pp][kMaxP + dy];
                T mv[C];
#pragma unroll
                for (int c = 0; c < C; ++c) mv[c] = s_m[pp][c];
#pragma unroll
                for (int z = 0; z < TZ; ++z) {
                    int dz = o.z + z;
                    if (dz >= Nz) dz -= Nz;
                    if (dz < P) {
                        const T wv = wxy * s_w[pp][2 * kMaxP + dz];
#pragma unroll
                        for (int c = 0; c < C; ++c) acc[z][c].add(wv, mv[c]);
                    }
                }
            }
        }
        __syncthreads();
    }
    const int gx = X0 + tx, gy = Y0 + ty;
    if (gx < Nx && gy < Ny) {
        const int64_t G = gp.G;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            const int gz = Z0 + z;
            if (gz < Nz) {
                const int64_t node = ((int64_t)gz * Ny + gy) * Nx + gx;
#pragma unroll
                for (int c = 0; c < C; ++c) grid[(int64_t)(3 * r0 + c) * G + node] = (TG)acc[z][c].get();
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Contract
// ---------------------------------------------------------------------------
constexpr int kRowPad = kTileX + 1;  // padded tile row: rows y and y+2 no longer share banks

// T: accumulation arithmetic; TG: grid element type; TP: partial type; TW: weight type.
template <typename T, int TZ, int NR, typename TG = T, typename TP = T, typename TW = TG>
__global__ void __launch_bounds__(256) k_contract_tiled(const TG *__restrict__ grid, int r0,
                                                        const int32_t *__restrict__ start, const TW *__restrict__ w,
                                                        GridParams gp, const int64_t *__restrict__ tstart,
                                                        const int32_t *__restrict__ entries, int ntx, int nty,
                                                        TP *__restrict__ partial) {
    constexpr int C = 3 * NR;
    constexpr int kPlane = kTileY * kRowPad;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tile = (T *)smem_raw;                                  // [C][TZ][16][17]
    T *wbuf = tile + C * TZ * kPlane;                         // [8 warps][3*kMaxP]
    const int64_t t = blockIdx.x;
    const int bx = (int)(t % ntx), by = (int)((t / ntx) % nty), bz = (int)(t / ((int64_t)ntx * nty));
    const int X0 = bx * kTileX, Y0 = by * kTileY, Z0 = bz * TZ;
    const int tx = threadIdx.x & (kTileX - 1), ty = threadIdx.x >> 4;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    const int64_t e0 = tstart[t], e1 = tstart[t + 1];
    if (e0 == e1) return;
    {
        const int gx = X0 + tx, gy = Y0 + ty;
        const bool in = gx < Nx && gy < Ny;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            const int gz = Z0 + z;
            const int64_t node = ((int64_t)gz * Ny + gy) * Nx + gx;
#pragma unroll
            for (int c = 0; c < C; ++c)
                tile[(c * TZ + z) * kPlane + ty * kRowPad + tx] =
                    (in && gz < Nz) ? (T)grid[(int64_t)(3 * r0 + c) * G + node] : (T)0;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T *wb = wbuf + wid * 3 * kMaxP;
    for (int64_t e = e0 + wid; e < e1; e += 8) {
        const int32_t a = entries[e];
        int ox = X0 - start[3 * a], oy = Y0 - start[3 * a + 1], oz = Z0 - start[3 * a + 2];
        if (ox < 0) ox += Nx;
        if (oy < 0) oy += Ny;
        if (oz < 0) oz += Nz;
        for (int k = lane; k < 3 * P; k += 32) wb[(k / P) * kMaxP + (k % P)] = (T)w[(int64_t)a * 3 * P + k];
        // stencil columns / rows / planes of this particle that fall inside the tile (and the grid)
        int xr = lane - ox, yr = lane - oy, zr = lane - oz;
        if (xr < 0) xr += Nx;
        if (yr < 0) yr += Ny;
        if (zr < 0) zr += Nz;
        const unsigned mx = __ballot_sync(0xffffffffu, lane < P && xr < kTileX && X0 + xr < Nx);
        const unsigned my = __ballot_sync(0xffffffffu, lane < P && yr < kTileY && Y0 + yr < Ny);
        unsigned mz = __ballot_sync(0xffffffffu, lane < P && zr < TZ && Z0 + zr < Nz);
        __syncwarp();
        const int nx = __popc(mx), ny = __popc(my);
        T acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = (T)0;
        for (int q = lane; q < nx * ny; q += 32) {
            const unsigned jxu = __fns(mx, 0, q % nx + 1), jyu = __fns(my, 0, q / nx + 1);
            if (jxu >= (unsigned)P || jyu >= (unsigned)P) continue;  // (cannot happen: q < nx*ny)
            const int jx = (int)jxu, jy = (int)jyu;
            int x = jx - ox, y = jy - oy;
            if (x < 0) x += Nx;
            if (y < 0) y += Ny;
            const T wxy = wb[jx] * wb[kMaxP + jy];
            unsigned mzz = mz;
            while (mzz) {
                const int jz = __ffs(mzz) - 1;
                mzz &= mzz - 1;
                int z = jz - oz;
                if (z < 0) z += Nz;
                const T wv = wxy * wb[2 * kMaxP + jz];
                const T *tp = tile + z * kPlane + y * kRowPad + x;
#pragma unroll
                for (int c = 0; c < C; ++c) acc[c] += wv * tp[c * TZ * kPlane];
            }
        }
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < C; ++c) partial[e * C + c] = (TP)acc[c];
        }
        __syncwarp();
    }
}

template <typename T, int NR>
__global__ void k_contract_gather(const T *__restrict__ partial, int64_t n, int r0, const int64_t *__restrict__ pstart,
                                  const int32_t *__restrict__ pentry, double hprod, double *__restrict__ out) {
    constexpr int C = 3 * NR;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        double acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = 0.0;
        for (int64_t k = pstart[a]; k < pstart[a + 1]; ++k) {
            const T *pp = partial + (int64_t)pentry[k] * C;
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] += (double)pp[c];
        }
#pragma unroll
        for (int r = 0; r < NR; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) out[((int64_t)(r0 + r) * n + a) * 3 + c] = acc[3 * r + c] * hprod;
    }
}

template <typename T, int TZ, int NR, typename TW, typename TG>
static int spread_launch(const double *m, int64_t n, int r0, const int32_t *start, const TW *w, const GridParams &gp,
                         const TileBins &tb, TG *grid, cudaStream_t s) {
    k_spread_tiled<T, TZ, NR, TW, TG><<<(unsigned)tb.ntiles, 256, 0, s>>>(m, n, r0, start, w, gp, tb.tile_start,
                                                                           tb.entries, tb.ntx, tb.nty, grid);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T, int TZ, typename TW, typename TG>
static int spread_dispatch(const double *m, int64_t n, int nrhs, const int32_t *start, const TW *w,
                           const GridParams &gp, const TileBins &tb, TG *grid, cudaStream_t s, int per = 3) {
    for (int r0 = 0; r0 < nrhs; r0 += per) {
        const int nr = min(per, nrhs - r0);
        int rc = nr == 3 ? spread_launch<T, TZ, 3, TW, TG>(m, n, r0, start, w, gp, tb, grid, s)
                 : nr == 2 ? spread_launch<T, TZ, 2, TW, TG>(m, n, r0, start, w, gp, tb, grid, s)
                           : spread_launch<T, TZ, 1, TW, TG>(m, n, r0, start, w, gp, tb, grid, s);
        if (rc) return rc;
    }
    return MPS_OK;
}

template <typename T>
int spread_tiled(const double *m, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp,
                 const TileBins &tb, T *grid, cudaStream_t s) {
    if (tb.tz == 8) return spread_dispatch<T, 8, T, T>(m, n, nrhs, start, w, gp, tb, grid, s);
    if (tb.tz == 4) return spread_dispatch<T, 4, T, T>(m, n, nrhs, start, w, gp, tb, grid, s);
    return MPS_BAD_ARG;
}

int spread_tiled_df(const double *m, int64_t n, int nrhs, const int32_t *start, const dfv *w, const GridParams &gp,
                    const TileBins &tb, dfv *grid, cudaStream_t s) {
    // three vectors per launch: one vector per launch (a third of the registers) measured slower, the
    // per-particle staging and w products then being repeated for every vector
    if (tb.tz == 8) return spread_dispatch<dfv, 8, dfv, dfv>(m, n, nrhs, start, w, gp, tb, grid, s);
    if (tb.tz == 4) return spread_dispatch<dfv, 4, dfv, dfv>(m, n, nrhs, start, w, gp, tb, grid, s);
    return MPS_BAD_ARG;
}

template <typename T, int TZ, int NR, typename TG, typename TP, typename TW>
static int contract_launch(const TG *grid, int64_t n, int r0, const int32_t *start, const TW *w,
                           const GridParams &gp, const TileBins &tb, TP *partial, double *out, cudaStream_t s) {
    constexpr int C = 3 * NR;
    const size_t smem = sizeof(T) * ((size_t)C * TZ * kTileY * kRowPad + 8 * 3 * kMaxP);
    static std::atomic<bool> attr_set{false};  // one attribute call per instantiation (a repeat is harmless)
    if (!attr_set.load(std::memory_order_acquire)) {
        MPS_CUDA_TRY(cudaFuncSetAttribute(k_contract_tiled<T, TZ, NR, TG, TP, TW>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set.store(true, std::memory_order_release);
    }
    k_contract_tiled<T, TZ, NR, TG, TP, TW><<<(unsigned)tb.ntiles, 256, smem, s>>>(
        grid, r0, start, w, gp, tb.tile_start, tb.entries, tb.ntx, tb.nty, partial);
    MPS_LAUNCH_CHECK();
    k_contract_gather<TP, NR><<<grid_for(n, 256), 256, 0, s>>>(partial, n, r0, tb.pstart, tb.pentry, gp.hprod, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T, int TZ, typename TG, typename TP, typename TW>
static int contract_dispatch(const TG *grid, int64_t n, int nrhs, const int32_t *start, const TW *w,
                             const GridParams &gp, const TileBins &tb, TP *partial, double *out, cudaStream_t s) {
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = min(3, nrhs - r0);
        int rc = nr == 3   ? contract_launch<T, TZ, 3, TG, TP, TW>(grid, n, r0, start, w, gp, tb, partial, out, s)
                 : nr == 2 ? contract_launch<T, TZ, 2, TG, TP, TW>(grid, n, r0, start, w, gp, tb, partial, out, s)
                           : contract_launch<T, TZ, 1, TG, TP, TW>(grid, n, r0, start, w, gp, tb, partial, out, s);
        if (rc) return rc;
    }
    return MPS_OK;
}

template <typename T>
int contract_tiled(const T *grid, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp,
                   const TileBins &tb, T *partial, double *out, cudaStream_t s) {
    if (tb.tz == 8) return contract_dispatch<T, 8, T, T, T>(grid, n, nrhs, start, w, gp, tb, partial, out, s);
    if (tb.tz == 4) return contract_dispatch<T, 4, T, T, T>(grid, n, nrhs, start, w, gp, tb, partial, out, s);
    return MPS_BAD_ARG;
}

int contract_tiled_df(const dfv *grid, int64_t n, int nrhs, const int32_t *start, const double *w,
                      const GridParams &gp, const TileBins &tb, double *partial, double *out, cudaStream_t s) {
    if (tb.tz == 8)
        return contract_dispatch<dfv, 8, dfv, double, double>(grid, n, nrhs, start, w, gp, tb, partial, out, s);
    if (tb.tz == 4)
        return contract_dispatch<dfv, 4, dfv, double, double>(grid, n, nrhs, start, w, gp, tb, partial, out, s);
    return MPS_BAD_ARG;
}

// Contraction of double-float grids, one warp per particle, particles visited in
// `order` (cell order: the warps of a CTA read overlapping stencils).  Lanes take
// the stencil's (x, y) columns; each column's z sum over the 3*NR grids runs in
// a ProdAcc<dfv> (exact leading products, two-sum, unnormalised within the
// column), then the column sums are weighted by wx*wy in double-float.  Fixed
// summation order: deterministic.  Bounds of 3 blocks per SM let ptxas keep more
// loads in flight (72 registers for one vector; 1.19 ms per residual matvec at the
// bench workload against 1.30 ms with 56 registers under the default heuristic).
template <int NR>
__global__ void __launch_bounds__(256, 3) k_contract_df_warp(const dfv *__restrict__ grid, int64_t n, int r0,
                                                          const int32_t *__restrict__ order,
                                                          const int32_t *__restrict__ start,
                                                          const dfv *__restrict__ w, GridParams gp,
                                                          double *__restrict__ out) {
    constexpr int C = 3 * NR;
    __shared__ dfv s_w[8][3 * kMaxP];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    const int64_t NxNy = (int64_t)Nx * Ny;
    dfv *wb = s_w[wid];
    for (int64_t i = warp; i < n; i += nw) {
        const int64_t a = order ? order[i] : i;
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        __syncwarp();
        for (int k = lane; k < 3 * P; k += 32) wb[k] = w[a * 3 * P + k];
        __syncwarp();
        dfv acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = dfv(0.f, 0.f);
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            ProdAcc<dfv> col[C];
#pragma unroll
            for (int c = 0; c < C; ++c) col[c].zero();
#pragma unroll 2
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const int64_t node = rowb + NxNy * iz;
                const dfv wz = wb[2 * P + jz];
#pragma unroll
                for (int c = 0; c < C; ++c) col[c].add(wz, grid[(int64_t)(3 * r0 + c) * G + node]);
            }
            const dfv wxy = wb[jx] * wb[P + jy];
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] += wxy * col[c].get();
        }
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < C; ++c) out[((int64_t)r0 * n + a) * 3 + (c / 3) * n * 3 + c % 3] = (double)acc[c] * gp.hprod;
    }
}

int contract_df_warp(const dfv *grid, int64_t n, int nrhs, const int32_t *order, const int32_t *start, const dfv *w,
                     const GridParams &gp, double *out, cudaStream_t s) {
    if (gp.P > kMaxP) return MPS_BAD_ARG;
    const unsigned blocks = grid_for(n * 32, 256, 152 * 64);
    // one vector per launch by default: a third of the registers (102 -> ~50), so three times the warps in flight
    // to cover the L2 latency of the grid reads; MPS_DF_CONTRACT_NR=3 batches three vectors per launch
    const char *e = getenv("MPS_DF_CONTRACT_NR");
    const int per = (e && strcmp(e, "3") == 0) ? 3 : 1;
    for (int r0 = 0; r0 < nrhs; r0 += per) {
        const int nr = min(per, nrhs - r0);
        if (nr == 3)
            k_contract_df_warp<3><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, gp, out);
        else if (nr == 2)
            k_contract_df_warp<2><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, gp, out);
        else
            k_contract_df_warp<1><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, gp, out);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

__global__ void k_weights_df(const double *__restrict__ w, int64_t total, dfv *__restrict__ wd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        wd[i] = dfv(w[i]);
}

int weights_df(const double *w, int64_t total, dfv *wd, cudaStream_t s) {
    k_weights_df<<<grid_for(total, 256), 256, 0, s>>>(w, total, wd);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

// In-place reinterpretation of a grid between float64 values and (hi, lo) pairs
// (same 8 bytes per value; each thread reads and writes only its own element).
__global__ void k_f64_to_dfv(double *__restrict__ g, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const dfv v(g[i]);
        reinterpret_cast<dfv *>(g)[i] = v;
    }
}
__global__ void k_dfv_to_f64(double *__restrict__ g, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const dfv v = reinterpret_cast<const dfv *>(g)[i];
        g[i] = (double)v;
    }
}

int f64_to_dfv_inplace(double *g, int64_t total, cudaStream_t s) {
    k_f64_to_dfv<<<grid_for(total, 256), 256, 0, s>>>(g, total);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int dfv_to_f64_inplace(double *g, int64_t total, cudaStream_t s) {
    k_dfv_to_f64<<<grid_for(total, 256), 256, 0, s>>>(g, total);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template int spread_tiled<float>(const double *, int64_t, int, const int32_t *, const float *, const GridParams &,
                                 const TileBins &, float *, cudaStream_t);
template int spread_tiled<double>(const double *, int64_t, int, const int32_t *, const double *, const GridParams &,
                                  const TileBins &, double *, cudaStream_t);
template int contract_tiled<float>(const float *, int64_t, int, const int32_t *, const float *, const GridParams &,
                                   const TileBins &, float *, double *, cudaStream_t);
template int contract_tiled<double>(const double *, int64_t, int, const int32_t *, const double *,
                                    const GridParams &, const TileBins &, double *, double *, cudaStream_t);

}  // namespace mps
