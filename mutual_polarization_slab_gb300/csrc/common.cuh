// Shared helpers for the GB300 spectral-Ewald kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mps_gb300.h"

#define MPS_PI 3.14159265358979323846

namespace mps {

constexpr int kWarp = 32;

// Status plumbing: CUDA errors become MPS_CUDA_ERR, never exceptions.
#define MPS_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) {                             \
            mps::set_last_error(_e, #expr, __FILE__, __LINE__); \
            return MPS_CUDA_ERR;                             \
        }                                                    \
    } while (0)

#define MPS_LAUNCH_CHECK()                                   \
    do {                                                     \
        mps::count_launch();                                 \
        cudaError_t _e = cudaGetLastError();                 \
        if (_e != cudaSuccess) {                             \
            mps::set_last_error(_e, "kernel launch", __FILE__, __LINE__); \
            return MPS_CUDA_ERR;                             \
        }                                                    \
    } while (0)

void set_last_error(cudaError_t e, const char *what, const char *file, int line);
void count_launch();
// Kernels enqueued while this thread captures a CUDA graph are not launches:
// between capture_count_begin and capture_count_end count_launch counts them
// for the caller (the launches per graph execution) instead of the process total.
void capture_count_begin();
long long capture_count_end();
void add_launches(long long k);

inline unsigned grid_for(int64_t work, int block, int64_t cap = 152 * 32) {
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// numpy float mod: result carries the sign of the divisor.
__device__ __forceinline__ double np_mod(double a, double b) {
    double r = fmod(a, b);
    if (r != 0.0) {
        if ((b < 0.0) != (r < 0.0)) r = __dadd_rn(r, b);
    } else {
        r = copysign(0.0, b);
    }
    return r;
}

// Integer frequency of unshifted FFT index i with the fftshift convention
// k in [-ceil((n-1)/2), floor((n-1)/2)] (the Nyquist bin of an even axis is negative).
__device__ __forceinline__ int fft_freq(int i, int n) {
    int c = n / 2;
    int p = i + c;
    if (p >= n) p -= n;
    return p - c;
}

// Quarter of an R2C half spectrum (Nx/2+1, Ny, Nz; x fastest): the points with
// iy <= Ny/2 and iz <= Nz/2.  Index N - i has frequency -fft_freq(i, N), so a
// coefficient that depends on k only through kx^2, ky^2, kz^2 is the same at
// (ix, +-iy, +-iz); mirror_points calls f(linear index, sy, sz) once for each
// distinct such point, sy / sz = -1 where the y / z index was mirrored.
struct HalfQuarter {
    int Nxh, Ny, Nz, Nyq, Nzq;
    __host__ __device__ explicit HalfQuarter(const int N[3])
        : Nxh(N[0] / 2 + 1), Ny(N[1]), Nz(N[2]), Nyq(N[1] / 2 + 1), Nzq(N[2] / 2 + 1) {}
    __host__ __device__ int64_t size() const { return (int64_t)Nxh * Nyq * Nzq; }
    __device__ void point(int64_t t, int *ix, int *iy, int *iz) const {
        *ix = (int)(t % Nxh);
        *iy = (int)((t / Nxh) % Nyq);
        *iz = (int)(t / ((int64_t)Nxh * Nyq));
    }
};

template <class F>
__device__ __forceinline__ void mirror_points(const HalfQuarter &q, int ix, int iy, int iz, F &&f) {
    const int my = (q.Ny - iy) % q.Ny, mz = (q.Nz - iz) % q.Nz;
    const int na = my == iy ? 1 : 2, nb = mz == iz ? 1 : 2;
    for (int a = 0; a < na; ++a)
        for (int b = 0; b < nb; ++b)
            f(((int64_t)(b ? mz : iz) * q.Ny + (a ? my : iy)) * q.Nxh + ix, a ? -1 : 1, b ? -1 : 1);
}

__device__ __forceinline__ int64_t wrap_index(int64_t i, int64_t n) {
    int64_t r = i % n;
    return r < 0 ? r + n : r;
}

// Exclusive scan of int64 counts (n may be large); tmp is scan_workspace() bytes.
size_t scan_workspace(int64_t n);
int exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, void *tmp, cudaStream_t s);
int exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, void *tmp, cudaStream_t s);

}  // namespace mps
