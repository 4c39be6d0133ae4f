#pragma once

#include "grid.cuh"

namespace mps {

template <typename T>
int spread_gen(const double *m, int64_t n, int nrhs, int ncomp, const int32_t *start, const T *w,
               const GridParams &gp, T *grid, cudaStream_t s);
template <typename T>
int contract_gen(const T *grid, int64_t n, int nrhs, int ncomp, const int32_t *start, const T *w,
                 const GridParams &gp, double *out, cudaStream_t s);
int quad_diag(const double *lam, int64_t total, const double *gq2, double *diag, cudaStream_t s);
int quad_kcoef(const GridParams &gp, double *c64, float *c32, cudaStream_t s);
template <typename T>
int scale_quad(void *spec, int nrhs, const GridParams &gp, const T *coef, cudaStream_t s);
int quad_pair_coefs(const double *dist, int64_t np, const double *perp, const double *para, const double *qt,
                    const double *rv, int64_t ntab, double *c64, float *c32, int *err, cudaStream_t s);
template <typename T>
int real_space_quad(const double *m, double *out, int64_t n, int nrhs, const int64_t *row_ptr, const int32_t *nbr,
                    const T *rx, const T *ry, const T *rz, const T *coef, const double *diagS, const double *diagQ,
                    const int32_t *diag_of_rhs, cudaStream_t s);

}  // namespace mps
