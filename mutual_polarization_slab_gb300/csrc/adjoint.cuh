#pragma once

#include "cells.cuh"
#include "grid.cuh"

namespace mps {

int rs_force(const double *m, int64_t n, const int64_t *row_ptr, const PairData<double> &pd, const double *perp,
             const double *para, const double *rv, int64_t ntab, double *F, int *err, cudaStream_t s);
int wave_force(const double *phi, const double *x, const double *m, int64_t n, const int32_t *start, const double *w,
               const GridParams &gp, double *F, cudaStream_t s);
int eps_grad(const double *m, const double *diag, double self, int64_t n, double *dE, cudaStream_t s);

}  // namespace mps
