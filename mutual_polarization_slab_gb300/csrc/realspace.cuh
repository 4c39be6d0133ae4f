#pragma once

#include "cells.cuh"

namespace mps {

template <typename T>
int real_space_csr(const double *m, double *out, int64_t n, int nrhs, const int64_t *row_ptr, PairData<T> pd,
                   const double *diag, const int32_t *diag_of_rhs, const double *slab, bool accumulate,
                   cudaStream_t s);
// The same pair sum in double-float arithmetic on double-float pair data; mdf is
// scratch for the double-float copy of m (nrhs x n x 3).
int real_space_csr_df(const double *m, dfv *mdf, double *out, int64_t n, int nrhs, const int64_t *row_ptr,
                      PairData<dfv> pd, const double *diag, const int32_t *diag_of_rhs, const double *slab,
                      bool accumulate, const int32_t *order, cudaStream_t s);
// Float32 pair sum on a float copy m32 of the moments (scratch of m32_floats(n, nrhs) floats or more: per particle
// its nrhs x 3 components side by side, padded to a multiple of 4).
size_t m32_floats(int64_t n, int nrhs);
int real_space_csr_f32(const double *m, float *m32, double *out, int64_t n, int nrhs, const int64_t *row_ptr,
                       PairData<float> pd, const double *diag, const int32_t *diag_of_rhs, const double *slab,
                       bool accumulate, const int32_t *order, cudaStream_t s);
int build_diag(const double *lam, int64_t total, const double *perp, double *diag, cudaStream_t s);
// Real and imaginary parts of the diagonal for complex permittivities (lr + i li).
int build_diag_complex(const double *lr, const double *li, int64_t total, const double *perp, double *dr, double *di,
                       cudaStream_t s);
int slab_terms(const double *m, int64_t n, int nrhs, double scale, double *slab, cudaStream_t s);
void table_self_terms(double xi, double *s_pc, double *s_fd);

}  // namespace mps
