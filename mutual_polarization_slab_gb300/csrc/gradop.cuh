// Gradient form of the float32 wave-space operator (see gradop.cu).
#pragma once

#include "grid.cuh"
#include "tiles.cuh"

namespace mps {

int grad_factors(const double *x, int64_t n, const GridParams &gp, const double *w64, float *g32, cudaStream_t s);
int grad_scale_coef(const GridParams &gp, const double *H, float *hs, cudaStream_t s);
// grid[r][G] for r < nrhs (one scalar grid per vector), written completely.
int spread_grad_tiled(const double *m, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                      const GridParams &gp, const TileBins &tb, float *grid, cudaStream_t s);
// out[r][a][c] = h^3 sum_n grad w_a(n) grid[r](n) (overwrites); partial: nentries * 3 * min(nrhs, 3) floats.
int contract_grad_tiled(const float *grid, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                        const GridParams &gp, const TileBins &tb, float *partial, double *out, cudaStream_t s);

// The same contraction as one warp per particle gathering from the grids (no tiles).
int contract_grad_warp(const float *grid, int64_t n, int nrhs, const int32_t *order, const int32_t *start,
                       const float *w, const float *g, const GridParams &gp, double *out, cudaStream_t s);
// The same sums (bit-identical) with each home block's reachable nodes staged in shared memory first; tb must hold
// home bins (tile_bins_home) of the same start.
bool contract_grad_home_supported(const GridParams &gp);
int contract_grad_home(const float *grid, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                       const GridParams &gp, const TileBins &tb, double *out, cudaStream_t s);

}  // namespace mps
