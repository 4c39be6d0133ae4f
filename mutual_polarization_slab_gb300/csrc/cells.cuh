// Cell binning and pair-list builders shared by the stateless entry points
// and the system object.
#pragma once

#include "common.cuh"

namespace mps {

struct CellBins {
    int64_t n = 0;
    int64_t ncell[3] = {0, 0, 0};
    int64_t ncells = 0;
    int32_t *lin = nullptr;       // linear cell index per particle
    int32_t *counts = nullptr;    // particles per cell
    int64_t *starts = nullptr;    // exclusive scan of counts
    int32_t *cursor = nullptr;
    int32_t *sorted = nullptr;    // particle ids sorted by (cell, id)
    int32_t *unsorted = nullptr;
};

// Structure-of-arrays pair data of the filtered per-particle CSR list.
template <typename T>
struct PairData {
    int32_t *nbr;   // source particle b of pair (a <- b)
    T *A;           // interpolated I - rr coupling
    T *BA;          // rr coupling minus A
    T *rx, *ry, *rz;  // unit vector from b to a (minimum image)
    T *dist;          // separation (only kept when an operator interpolates more tables)
};

void compute_ncell(const double *box, double rmax, int64_t *ncell);
size_t cell_bins_bytes(int64_t n, int64_t ncells);
int cell_assign(const double *x, int64_t n, const double *box, const int64_t *ncell, int64_t *cell3, cudaStream_t s);
int cell_bins_build(const int64_t *cell3, int64_t n, const int64_t *ncell, void *ws, CellBins &cb, cudaStream_t s);
int positions_f32(const double *x, int64_t n, float *xf, unsigned *maxbits, double *maxabs, cudaStream_t s);
int csr_pairs_count(const double *x, const float *xf, double maxabs, const double *box, double rc, const CellBins &cb,
                    int64_t *cnt27, int64_t *off27, void *scan_tmp, int64_t *total_host, cudaStream_t s);
int csr_pairs_fill(const double *x, const float *xf, double maxabs, const double *box, double rc, const CellBins &cb,
                   const int64_t *cnt27,
                   const int64_t *off27, const double *perp, const double *para, const double *rv, int64_t ntab,
                   int64_t *row_ptr, PairData<double> p64, PairData<float> p32, int *err, cudaStream_t s);

}  // namespace mps
