// Adjoint forces of the polarisation energy E = -1/2 m . H0 with A(x) m = H0.
//
// Because the operator is symmetric, dE/dx_k = 1/2 m^T (dA/dx_k) m with the
// converged moments held fixed (no second solve), so
//   F_k = -dE/dx_k = -sum_j grad_r [m_k . M(r) m_j]            (real space)
//                    - h^3 sum_n grad_x w_k(n) (m_k . phi(n))  (wave space)
// with M(r) = A(r)(I - r r) + B(r) r r, r = x_k - x_j (minimum image), A and B
// the linearly interpolated tables (their derivatives are the segment slopes,
// i.e. the exact derivative of the operator that was solved), w_k the Gaussian
// spreading weight and phi the convolved grid the contraction reads
// (IFFT(scale(FFT(spread(m))))).  The dielectric, self and slab terms do not
// depend on positions.  dE/d eps_k = 1/2 |m_k|^2 dD_k/d eps_k with
// D_k = 3 / (4 pi (eps_k - 1)) + self.
#include <math.h>

#include "cells.cuh"
#include "grid.cuh"

namespace mps {

__device__ __forceinline__ int64_t seg_index(const double *__restrict__ rv, int64_t n, double d) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (rv[mid] < d)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// One group of 8 lanes per particle over its CSR row.
__global__ void __launch_bounds__(256) k_rs_force(const double *__restrict__ m, int64_t n,
                                                  const int64_t *__restrict__ row_ptr, PairData<double> pd,
                                                  const double *__restrict__ perp, const double *__restrict__ para,
                                                  const double *__restrict__ rv, int64_t ntab,
                                                  double *__restrict__ F, int *__restrict__ err) {
    constexpr int G = 8;
    const int lane = threadIdx.x % G;
    const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t a = grp; a < n; a += ngrp) {
        const double amx = m[3 * a], amy = m[3 * a + 1], amz = m[3 * a + 2];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int64_t e = row_ptr[a] + lane; e < row_ptr[a + 1]; e += G) {
            const int32_t b = pd.nbr[e];
            const double d = pd.dist[e];
            const int64_t i = seg_index(rv, ntab, d);
            if (i <= 0 || i >= ntab) {
                atomicExch(err, 1);
                continue;
            }
            const double dr = rv[i] - rv[i - 1];
            const double Ap = (perp[i] - perp[i - 1]) / dr;
            const double Bp = (para[i] - para[i - 1]) / dr;
            const double A = pd.A[e], BA = pd.BA[e];
            const double rx = pd.rx[e], ry = pd.ry[e], rz = pd.rz[e];
            const double mbx = m[3 * b], mby = m[3 * b + 1], mbz = m[3 * b + 2];
            const double ar = amx * rx + amy * ry + amz * rz;
            const double br = mbx * rx + mby * ry + mbz * rz;
            const double ab = amx * mbx + amy * mby + amz * mbz;
            const double s = BA / d;
            // grad_r [A (ma.mb) + (B - A)(ma.r)(mb.r)]
            const double cr = Ap * ab + (Bp - Ap) * ar * br - 2.0 * s * ar * br;
            fx -= cr * rx + s * (br * amx + ar * mbx);
            fy -= cr * ry + s * (br * amy + ar * mby);
            fz -= cr * rz + s * (br * amz + ar * mbz);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o, G);
            fy += __shfl_xor_sync(0xffffffffu, fy, o, G);
            fz += __shfl_xor_sync(0xffffffffu, fz, o, G);
        }
        if (lane == 0) {
            F[3 * a] = fx;
            F[3 * a + 1] = fy;
            F[3 * a + 2] = fz;
        }
    }
}

// Half-away-from-zero rounding, as the grid geometry uses.
__device__ __forceinline__ double round_half_away(double v) {
    const double a = floor(fabs(v) + 0.5);
    return v > 0 ? a : (v < 0 ? -a : 0.0 * a);
}

// Wave-space part: warp per particle over its P^3 stencil; phi = the three
// convolved component grids of one vector.
__global__ void __launch_bounds__(256) k_wave_force(const double *__restrict__ phi, const double *__restrict__ x,
                                                    const double *__restrict__ m, int64_t n,
                                                    const int32_t *__restrict__ start, const double *__restrict__ w,
                                                    GridParams gp, double *__restrict__ F) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    const double kx = 4.0 * gp.xi * gp.xi / gp.eta[0], ky = 4.0 * gp.xi * gp.xi / gp.eta[1],
                 kz = 4.0 * gp.xi * gp.xi / gp.eta[2];
    for (int64_t a = warp; a < n; a += nw) {
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const double *wa = w + a * 3 * P;
        double base[3];
        for (int d = 0; d < 3; ++d) {
            const double xv = x[3 * a + d];
            base[d] = __dsub_rn(__dmul_rn(round_half_away(__ddiv_rn(xv, gp.h[d])), gp.h[d]), xv);
        }
        const double mx = m[3 * a], my = m[3 * a + 1], mz = m[3 * a + 2];
        double gx = 0.0, gy = 0.0, gz = 0.0;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const double rx = base[0] + (double)(jx - lo) * gp.h[0];
            const double ry = base[1] + (double)(jy - lo) * gp.h[1];
            const double wxy = wa[jx] * wa[P + jy];
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const double rz = base[2] + (double)(jz - lo) * gp.h[2];
                const double wv = wxy * wa[2 * P + jz];
                const int64_t node = rowb + (int64_t)Nx * Ny * iz;
                const double val = wv * (mx * phi[node] + my * phi[G + node] + mz * phi[2 * G + node]);
                gx += kx * rx * val;
                gy += ky * ry * val;
                gz += kz * rz * val;
            }
        }
        gx = warp_sum(gx);
        gy = warp_sum(gy);
        gz = warp_sum(gz);
        if (lane == 0) {
            F[3 * a] -= gp.hprod * gx;
            F[3 * a + 1] -= gp.hprod * gy;
            F[3 * a + 2] -= gp.hprod * gz;
        }
    }
}

// dD/d eps = -3 / (4 pi (eps - 1)^2) = -(4 pi / 3) (D - self)^2, from the stored diagonal.
__global__ void k_eps_grad(const double *__restrict__ m, const double *__restrict__ diag, double self, int64_t n,
                           double *__restrict__ dE) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const double m2 = m[3 * a] * m[3 * a] + m[3 * a + 1] * m[3 * a + 1] + m[3 * a + 2] * m[3 * a + 2];
        const double dl = diag[a] - self;
        dE[a] = 0.5 * m2 * (-(4.0 * MPS_PI / 3.0) * dl * dl);
    }
}

int rs_force(const double *m, int64_t n, const int64_t *row_ptr, const PairData<double> &pd, const double *perp,
             const double *para, const double *rv, int64_t ntab, double *F, int *err, cudaStream_t s) {
    k_rs_force<<<grid_for(n * 8, 256, 152 * 64), 256, 0, s>>>(m, n, row_ptr, pd, perp, para, rv, ntab, F, err);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int wave_force(const double *phi, const double *x, const double *m, int64_t n, const int32_t *start, const double *w,
               const GridParams &gp, double *F, cudaStream_t s) {
    k_wave_force<<<grid_for(n * 32, 256, 152 * 64), 256, 0, s>>>(phi, x, m, n, start, w, gp, F);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int eps_grad(const double *m, const double *diag, double self, int64_t n, double *dE, cudaStream_t s) {
    k_eps_grad<<<grid_for(n, 256), 256, 0, s>>>(m, diag, self, n, dE);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

}  // namespace mps
