// Tile binning of particles and the tiled spread / contract kernels.
#pragma once

#include "grid.cuh"
#include "dfloat.cuh"

namespace mps {

constexpr int kTileX = 16;
constexpr int kTileY = 16;
constexpr int kMaxP = 16;       // largest support handled by the tiled kernels
constexpr int kMaxTilesPerDim = 4;

// Particles binned into every grid tile their P^3 stencil touches.
struct TileBins {
    int tz = 0;                 // tile depth (z)
    int ntx = 0, nty = 0, ntz = 0;
    int64_t ntiles = 0;
    int64_t nentries = 0;
    int64_t *tile_start = nullptr;   // ntiles + 1
    int32_t *entries = nullptr;      // particle id per (tile, particle) entry, tiles in order, ids ascending
    int64_t *pstart = nullptr;       // n + 1: each particle's entries ...
    int32_t *pentry = nullptr;       // ... listed here (entry indices), in the particle's tile order
    bool has_pentry = false;         // pentry filled (the tiled contractions' gathers need it; spreads do not)
    void *mem = nullptr;             // single allocation backing the arrays above
    // Home bins (on demand, tile_bins_home): every particle once, under the kHomeBlock^3 block of grid nodes that
    // holds the first node of its stencil; the stencil then lies inside the block grown by P - 1 nodes per axis.
    bool has_home = false;
    int nhb[3] = {0, 0, 0};          // home blocks per axis
    int64_t nhome = 0;
    int64_t *hstart = nullptr;       // nhome + 1
    int32_t *hentries = nullptr;     // n particle ids, grouped by home block
    void *hmem = nullptr;
};

constexpr int kHomeBlock = 8;

bool tiles_supported(const GridParams &gp, int tz);
int tile_bins_build(const int32_t *start, int64_t n, const GridParams &gp, int tz, TileBins &tb, cudaStream_t s);
// Fills tb.pentry (once) for the gathers of the tiled contractions.
int tile_bins_pentry(const int32_t *start, const GridParams &gp, TileBins &tb, cudaStream_t s);
// Fills the home bins (once) for the staged contractions.
int tile_bins_home(const int32_t *start, int64_t n, const GridParams &gp, TileBins &tb, cudaStream_t s);
void tile_bins_free(TileBins &tb, cudaStream_t s);

// grid[(r*3+c)][G] for r < nrhs, written completely (no zeroing needed).
template <typename T>
int spread_tiled(const double *m, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp,
                 const TileBins &tb, T *grid, cudaStream_t s);

// out[r][a][c] = hprod * sum over the stencil (overwrites); partial: nentries * 3 * min(nrhs,3) of T.
template <typename T>
int contract_tiled(const T *grid, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp,
                   const TileBins &tb, T *partial, double *out, cudaStream_t s);

// The same kernels with double-float accumulation (float-pair arithmetic) on
// double-float weights, the grids stored as (hi, lo) float pairs: the float64-accurate
// matvec without float64 issue (no conversion to or from float64 between stages).
int spread_tiled_df(const double *m, int64_t n, int nrhs, const int32_t *start, const dfv *w, const GridParams &gp,
                    const TileBins &tb, dfv *grid, cudaStream_t s);
// Warp-per-particle contraction of double-float grids (particles in `order`, null =
// input order); out[r][a][c] = hprod * sum (overwrites).  w: double-float weights.
int contract_df_warp(const dfv *grid, int64_t n, int nrhs, const int32_t *order, const int32_t *start, const dfv *w,
                     const GridParams &gp, double *out, cudaStream_t s);
// Double-float copy of float64 weights.
int weights_df(const double *w, int64_t total, dfv *wd, cudaStream_t s);
int contract_tiled_df(const dfv *grid, int64_t n, int nrhs, const int32_t *start, const double *w,
                      const GridParams &gp, const TileBins &tb, double *partial, double *out, cudaStream_t s);
// Grid storage conversions in place (float64 <-> (hi, lo) pairs), for the untiled kernels.
int f64_to_dfv_inplace(double *g, int64_t total, cudaStream_t s);
int dfv_to_f64_inplace(double *g, int64_t total, cudaStream_t s);

}  // namespace mps
