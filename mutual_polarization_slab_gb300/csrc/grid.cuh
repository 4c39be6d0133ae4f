#pragma once

#include "common.cuh"

namespace mps {

struct GridParams {
    int N[3];          // nodes per axis
    int P;             // Gaussian support
    int64_t G;         // N[0] N[1] N[2]
    double h[3];       // spacing
    double eta[3];     // spectral splitting
    double inv_eta[3];
    double kfac[3];    // 2 pi / L
    double xi;
    double wconst;     // (2 xi^2/pi)^{3/2} / sqrt(prod eta)
    double hprod;      // trapezoid factor of the contraction
    // optional visiting order of the particles (ids sorted by cell, n entries):
    // per-particle gather kernels read overlapping stencils from neighbouring warps
    const int32_t *order = nullptr;
};

// The P x P (x, y) rows of a particle's stencil, handed to the lanes of a warp
// 32 at a time.  In a full pass lane l takes row row0 + l and its whole z run; in
// the last, partial pass the z run of each of the rem remaining rows is split over
// lpp = 32 / rem lanes (lane sub of a row takes z = sub, sub + lpp, ...), so no
// lane idles.  Returns false for a lane left without a row.
__device__ __forceinline__ bool stencil_row(int row0, int P, int lane, int *idx, int *sub, int *lpp) {
    const int rem = P * P - row0;
    const int l = rem >= 32 ? 1 : 32 / rem;
    const int q = lane / l;
    *idx = row0 + q;
    *sub = lane - q * l;
    *lpp = l;
    return row0 + q < P * P;
}

GridParams make_grid_params(const int64_t *Ngrid, const double *box, double xi, const double *eta, int P);
int grid_geometry(const double *x, int64_t n, const GridParams &gp, int32_t *start, double *w64, float *w32,
                  cudaStream_t s);
int green_half(const GridParams &gp, double *h64, float *h32, cudaStream_t s);
template <typename T>
int spread(const double *m, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp, T *grid,
           cudaStream_t s);
template <typename T>
int contract(const T *grid, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp, double *out,
             cudaStream_t s);
template <typename T>
int scale_half(void *spec, int nrhs, const GridParams &gp, const T *Hh, cudaStream_t s);
int scale_full_c2c(void *spec, const GridParams &gp, cudaStream_t s);
int pack_complex(const double *re_im, int64_t G, void *c, cudaStream_t s);
int unpack_complex(const void *c, int64_t G, double *re_im, cudaStream_t s);

}  // namespace mps
