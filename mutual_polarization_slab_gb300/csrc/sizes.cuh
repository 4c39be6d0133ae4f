#pragma once

#include "cells.cuh"
#include "grid.cuh"

namespace mps {

int cs_pair_coefs(const int64_t *row_ptr, const int32_t *nbr, const double *dist, int64_t n, const double *radius,
                  const int32_t *cls, int64_t M, const double *tab, const double *rv, int64_t ntab, double xi,
                  PairData<double> p64, PairData<float> p32, int *err, cudaStream_t s);
int cs_diag(const double *lam, int64_t n, int64_t nsets, const double *radius, const int32_t *cls, int64_t M,
            const double *tab, int64_t ntab, double xi, double *diag, cudaStream_t s);
int cs_geometry(const double *x, int64_t n, const GridParams &gp, const double *radius, double xi, double eta,
                int32_t *start, double *base, double *g64, float *g32, cudaStream_t s);
int cs_green(const GridParams &gp, double eta, double xi, double *c64, float *c32, cudaStream_t s);
template <typename T>
int spread_cs(const double *m, int64_t n, int nrhs, const int32_t *start, const double *base, const T *g,
              const GridParams &gp, T *grid, cudaStream_t s);
template <typename T>
int scale_cs(void *spec, int nrhs, const GridParams &gp, const T *coef, cudaStream_t s);
template <typename T>
int contract_cs(const T *grid, int64_t n, int nrhs, const int32_t *start, const double *base, const T *g,
                const GridParams &gp, double *out, cudaStream_t s);

}  // namespace mps
