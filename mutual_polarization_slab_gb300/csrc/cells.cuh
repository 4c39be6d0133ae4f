// Cell binning and pair-list builders shared by the stateless entry points
// and the system object.
#pragma once

#include "common.cuh"
#include "dfloat.cuh"

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
// Enqueues the pair count on s and the copies of the last offset and count into last2 (two int64 in page-locked
// host memory): once s is synchronised the number of pairs is last2[0] + last2[1].
int csr_pairs_count(const double *x, const float *xf, double maxabs, const double *box, double rc, const CellBins &cb,
                    int64_t *cnt27, int64_t *off27, void *scan_tmp, int64_t *last2, cudaStream_t s);
int csr_pairs_fill(const double *x, const float *xf, double maxabs, const double *box, double rc, const CellBins &cb,
                   const int64_t *cnt27,
                   const int64_t *off27, const double *perp, const double *para, const double *rv, int64_t ntab,
                   int64_t *row_ptr, PairData<double> p64, PairData<float> p32, int *err, cudaStream_t s);

// Double-float form of the solver's pair list (the dipole operator): positions as
// float pairs, the interpolation table per segment as double-float values.
struct DfTab {
    const float *rvf = nullptr;       // ntab table separations (float, for the index search)
    const float4 *seg_r = nullptr;    // segment i: (r_{i-1}, 1/(r_i - r_{i-1})) double-float
    const float4 *seg_perp = nullptr; // (perp_{i-1}, perp_i - perp_{i-1})
    const float4 *seg_para = nullptr; // (para_{i-1}, para_i - para_{i-1})
    int64_t ntab = 0;
    float inv_dr = 0.f;               // (ntab - 1) / r_last: uniform-spacing index guess
};
size_t df_tab_bytes(int64_t ntab);
int df_tab_build(const double *perp, const double *para, const double *rv, int64_t ntab, void *buf, DfTab &t,
                 cudaStream_t s);
int positions_df(const double *x, int64_t n, float2 *xdf, cudaStream_t s);
// Same pair set and order as csr_pairs_fill; couplings, unit vectors and
// separations in double-float (pdf) and float32 (p32); float64 only for the
// keep decision of pairs in the screen's margin band.
int csr_pairs_fill_df(const double *x, const float *xf, const float2 *xdf, double maxabs, const double *box, double rc,
                      const CellBins &cb, const int64_t *cnt27, const int64_t *off27, const DfTab &tab,
                      int64_t *row_ptr, PairData<dfv> pdf, PairData<float> p32, int *err, cudaStream_t s);
// p64 = pdf converted to float64 (the float64 operator's pair data, built on demand).
int pairs_df_to_f64(const PairData<dfv> &pdf, int64_t np, PairData<double> p64, cudaStream_t s);

// Real-space field at ne probe points from np source dipoles within rc (Compute_Field/RealSpace.m
// over the probe/source pairs of Compute_Field/FieldMap.m:46-52); out: ne x 3 (overwrites).
int probe_real_space(const double *xe, int64_t ne, const double *xp, const double *p, int64_t np, const double *box,
                     double rc, const double *perp, const double *para, const double *rv, int64_t ntab, double *out,
                     cudaStream_t s);

// Field and gradient (ne x 8: E then G xx xy xz yy yz) at probes from source dipoles + quadrupoles
// sq (np x 8) within rc; tab9: the 9 coupling tables (9 x ntab) on rv (Compute_Field_Quadrupole/RealSpace.m).
int probe_real_space_quad(const double *xe, int64_t ne, const double *xp, const double *sq, int64_t np,
                          const double *box, double rc, const double *tab9, const double *rv, int64_t ntab,
                          double *out, cudaStream_t s);

// Real-space field (ne x 3) at probes of radius class cmin from source dipoles p (np x 3) of classes cls
// within rc; perp/para: M(M+1)/2 columns of ntab rows on rv (Compute_Field_Sizes/RealSpace.m).
int probe_real_space_cs(const double *xe, int64_t ne, const double *xp, const double *p, const int32_t *cls,
                        int32_t cmin, int32_t M, int64_t np, const double *box, double rc, const double *perp,
                        const double *para, const double *rv, int64_t ntab, double *out, cudaStream_t s);

}  // namespace mps
