// Dipole + quadrupole operator: 8 moments per sphere, S (x, y, z) and the
// traceless quadrupole Q stored as (xx, xy, xz, yy, yz), zz = -(xx + yy)
// (Capacitance_Quadrupole/MatrixVectorMultiply.m:31-77).
//
//   spread / contract   the dipole path's Gaussian on 8 component grids
//                       (CQ/Spread.m:41-71, CQ/Contract.m:49-77)
//   scale               E~ = (HES k.fS + HEQ Qd.fQ) k,  G~ = (HGS k.fS + HGQ Qd.fQ) Qf
//                       with HES = 9 j1^2, HEQ = -45/2 i j1 j2, HGS = 45 i j2 j1,
//                       HGQ = 225/2 j2^2, times exp(-sum(1-eta)k^2/4xi^2)/k^2
//                       (CQ/Scale.m:19-72); on the half spectrum of real grids
//                       the unpaired Nyquist bins get the average of the
//                       coupling at k and at its conjugate partner (the real
//                       part of the reference's complex pipeline)
//   real space          nine interpolated couplings per pair (CQ/RealSpace.m:27-100)
#include <math.h>

#include "quad.cuh"

namespace mps {

// ---------------------------------------------------------------------------
// Spread / contract for ncomp (<= 8) moment components per particle.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_spread_gen(const double *__restrict__ m, int64_t n, int nrhs, int ncomp,
                                                    const int32_t *__restrict__ start, const T *__restrict__ w,
                                                    GridParams gp, T *__restrict__ grid) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    for (int64_t t = warp; t < n * nrhs; t += nw) {
        const int64_t a = gp.order ? (int64_t)gp.order[t % n] : t % n;
        const int r = (int)(t / n);
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const T *wa = w + a * 3 * P;
        T mv[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) mv[c] = c < ncomp ? (T)m[((int64_t)r * n + a) * ncomp + c] : (T)0;
        T *g0 = grid + (int64_t)r * ncomp * G;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const T wxy = wa[jx] * wa[P + jy];
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const T wv = wxy * wa[2 * P + jz];
                const int64_t node = rowb + (int64_t)Nx * Ny * iz;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (c < ncomp) atomicAdd(g0 + c * G + node, wv * mv[c]);
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_contract_gen(const T *__restrict__ grid, int64_t n, int nrhs, int ncomp,
                                                      const int32_t *__restrict__ start, const T *__restrict__ w,
                                                      GridParams gp, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    for (int64_t t = warp; t < n * nrhs; t += nw) {
        const int64_t a = gp.order ? (int64_t)gp.order[t % n] : t % n;
        const int r = (int)(t / n);
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const T *wa = w + a * 3 * P;
        const T *g0 = grid + (int64_t)r * ncomp * G;
        T acc[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = (T)0;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const T wxy = wa[jx] * wa[P + jy];
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const T wv = wxy * wa[2 * P + jz];
                const int64_t node = rowb + (int64_t)Nx * Ny * iz;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (c < ncomp) acc[c] += wv * g0[c * G + node];
            }
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0)
            for (int c = 0; c < ncomp; ++c) out[((int64_t)r * n + a) * ncomp + c] = (double)acc[c] * gp.hprod;
    }
}

// ---------------------------------------------------------------------------
// Wave space
// ---------------------------------------------------------------------------
__global__ void k_quad_kcoef(GridParams gp, double *__restrict__ c64, float *__restrict__ c32) {
    const int Nxh = gp.N[0] / 2 + 1;
    const int64_t Gc = (int64_t)Nxh * gp.N[1] * gp.N[2];
    const double invG = 1.0 / (double)gp.G;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gc; t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t % Nxh);
        const int iy = (int)((t / Nxh) % gp.N[1]);
        const int iz = (int)(t / ((int64_t)Nxh * gp.N[1]));
        const double kx = fft_freq(ix, gp.N[0]) * gp.kfac[0];
        const double ky = fft_freq(iy, gp.N[1]) * gp.kfac[1];
        const double kz = fft_freq(iz, gp.N[2]) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        double v[4] = {0, 0, 0, 0};
        if (k2 > 0) {
            const double k = sqrt(k2);
            const double s = sin(k), c = cos(k);
            const double j1 = s / k2 - c / k;
            const double j2 = (3.0 / k2 - 1.0) * s / k - 3.0 * c / k2;
            const double etak2 = (1 - gp.eta[0]) * kx * kx + (1 - gp.eta[1]) * ky * ky + (1 - gp.eta[2]) * kz * kz;
            const double g = exp(-etak2 / (4 * gp.xi * gp.xi)) / k2 * invG;
            v[0] = 9.0 * j1 * j1 * g;        // HES
            v[1] = -22.5 * j1 * j2 * g;      // HEQ / i
            v[2] = 45.0 * j2 * j1 * g;       // HGS / i
            v[3] = 112.5 * j2 * j2 * g;      // HGQ
            for (int q = 0; q < 4; ++q)
                if (!isfinite(v[q])) v[q] = 0.0;
        }
        for (int q = 0; q < 4; ++q) {
            c64[4 * t + q] = v[q];
            if (c32) c32[4 * t + q] = (float)v[q];
        }
    }
}

template <typename T>
struct C2T;
template <>
struct C2T<float> {
    using type = float2;
};
template <>
struct C2T<double> {
    using type = double2;
};

// out = M(q) f for unit wave vector q; cconj flips the imaginary couplings.
template <typename T, typename C>
__device__ __forceinline__ void quad_couple(const T q[3], const T cf[4], bool cconj, const C f[8], C out[8]) {
    const T qd[5] = {q[0] * q[0] - q[2] * q[2], 2 * q[0] * q[1], 2 * q[0] * q[2], q[1] * q[1] - q[2] * q[2],
                     2 * q[1] * q[2]};
    const T qf[5] = {q[0] * q[0] - (T)(1.0 / 3.0), q[0] * q[1], q[0] * q[2], q[1] * q[1] - (T)(1.0 / 3.0),
                     q[1] * q[2]};
    C dS, dQ;
    dS.x = q[0] * f[0].x + q[1] * f[1].x + q[2] * f[2].x;
    dS.y = q[0] * f[0].y + q[1] * f[1].y + q[2] * f[2].y;
    dQ.x = dQ.y = (T)0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        dQ.x += qd[k] * f[3 + k].x;
        dQ.y += qd[k] * f[3 + k].y;
    }
    const T eq = cconj ? -cf[1] : cf[1];
    const T gs = cconj ? -cf[2] : cf[2];
    // a = HES dS + i eq dQ ; b = i gs dS + HGQ dQ
    C a, b;
    a.x = cf[0] * dS.x - eq * dQ.y;
    a.y = cf[0] * dS.y + eq * dQ.x;
    b.x = -gs * dS.y + cf[3] * dQ.x;
    b.y = gs * dS.x + cf[3] * dQ.y;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        out[k].x = a.x * q[k];
        out[k].y = a.y * q[k];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        out[3 + k].x = b.x * qf[k];
        out[3 + k].y = b.y * qf[k];
    }
}

template <typename T>
__global__ void k_scale_quad(typename C2T<T>::type *__restrict__ spec, int nrhs, GridParams gp,
                             const T *__restrict__ coef) {
    using C = typename C2T<T>::type;
    const int Nxh = gp.N[0] / 2 + 1;
    const int64_t Gc = (int64_t)Nxh * gp.N[1] * gp.N[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gc; t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t % Nxh);
        const int iy = (int)((t / Nxh) % gp.N[1]);
        const int iz = (int)(t / ((int64_t)Nxh * gp.N[1]));
        const double kx = fft_freq(ix, gp.N[0]) * gp.kfac[0];
        const double ky = fft_freq(iy, gp.N[1]) * gp.kfac[1];
        const double kz = fft_freq(iz, gp.N[2]) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        T q[3] = {0, 0, 0};
        if (k2 > 0) {
            const double inv = 1.0 / sqrt(k2);
            q[0] = (T)(kx * inv);
            q[1] = (T)(ky * inv);
            q[2] = (T)(kz * inv);
        }
        const bool ny[3] = {(gp.N[0] % 2 == 0) && ix == gp.N[0] / 2, (gp.N[1] % 2 == 0) && iy == gp.N[1] / 2,
                            (gp.N[2] % 2 == 0) && iz == gp.N[2] / 2};
        const bool nyq = ny[0] || ny[1] || ny[2];
        // conjugate partner: non-Nyquist components flip sign
        const T qp[3] = {ny[0] ? q[0] : -q[0], ny[1] ? q[1] : -q[1], ny[2] ? q[2] : -q[2]};
        const T cf[4] = {coef[4 * t], coef[4 * t + 1], coef[4 * t + 2], coef[4 * t + 3]};
        for (int r = 0; r < nrhs; ++r) {
            C *s = spec + (int64_t)(8 * r) * Gc + t;
            C f[8], o1[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) f[c] = s[c * Gc];
            quad_couple<T, C>(q, cf, false, f, o1);
            if (nyq) {
                C o2[8];
                quad_couple<T, C>(qp, cf, true, f, o2);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    o1[c].x = (T)0.5 * (o1[c].x + o2[c].x);
                    o1[c].y = (T)0.5 * (o1[c].y + o2[c].y);
                }
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c * Gc] = o1[c];
        }
    }
}

// ---------------------------------------------------------------------------
// Real space
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t qsearch(const double *__restrict__ rv, int64_t n, double d, double inv_dr) {
    double gf = d * inv_dr;
    int64_t g = gf < 0 ? 0 : (gf > (double)(n - 1) ? n - 1 : (int64_t)gf);
    for (int it = 0; it < 64; ++it) {
        if (g < n && rv[g] < d) {
            ++g;
            continue;
        }
        if (g > 0 && rv[g - 1] >= d) {
            --g;
            continue;
        }
        return g;
    }
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

// coef[p][9] = (A, B, C, D, E, F, G, H, I) interpolated at the pair separation.
__global__ void k_quad_pair_coefs(const double *__restrict__ dist, int64_t np, const double *__restrict__ perp,
                                  const double *__restrict__ para, const double *__restrict__ qt,
                                  const double *__restrict__ rv, int64_t ntab, double inv_dr,
                                  double *__restrict__ c64, float *__restrict__ c32, int *__restrict__ err) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const double d = dist[p];
        const int64_t i = qsearch(rv, ntab, d, inv_dr);
        double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (i <= 0 || i >= ntab) {
            atomicExch(err, 1);
        } else {
            const double t = (d - rv[i - 1]) / (rv[i] - rv[i - 1]);
            const double u = 1.0 - t;
            v[0] = perp[i - 1] * u + perp[i] * t;
            v[1] = para[i - 1] * u + para[i] * t;
            for (int k = 0; k < 7; ++k) v[2 + k] = qt[k * ntab + i - 1] * u + qt[k * ntab + i] * t;
        }
        for (int k = 0; k < 9; ++k) {
            c64[9 * p + k] = v[k];
            if (c32) c32[9 * p + k] = (float)v[k];
        }
    }
}

template <typename T, int G>
__global__ void __launch_bounds__(256) k_rs_quad(const double *__restrict__ m, double *__restrict__ out, int64_t n,
                                                 int nrhs, const int64_t *__restrict__ row_ptr,
                                                 const int32_t *__restrict__ nbr, const T *__restrict__ rxs,
                                                 const T *__restrict__ rys, const T *__restrict__ rzs,
                                                 const T *__restrict__ coef, const double *__restrict__ diagS,
                                                 const double *__restrict__ diagQ,
                                                 const int32_t *__restrict__ diag_of_rhs) {
    const int lane = threadIdx.x % G;
    const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t t = grp; t < n * nrhs; t += ngrp) {
        const int64_t a = t % n;
        const int r = (int)(t / n);
        T acc[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = (T)0;
        for (int64_t e = row_ptr[a] + lane; e < row_ptr[a + 1]; e += G) {
            const int32_t b = nbr[e];
            const T rx = rxs[e], ry = rys[e], rz = rzs[e];
            const T *cf = coef + 9 * e;
            const T A = cf[0], B = cf[1], Cc = cf[2], D = cf[3], E = cf[4], F = cf[5], Gg = cf[6], H = cf[7],
                    I = cf[8];
            const double *mb = m + ((int64_t)r * n + b) * 8;
            const T Sx = (T)mb[0], Sy = (T)mb[1], Sz = (T)mb[2];
            const T Q0 = (T)mb[3], Q1 = (T)mb[4], Q2 = (T)mb[5], Q3 = (T)mb[6], Q4 = (T)mb[7];
            const T sr = Sx * rx + Sy * ry + Sz * rz;
            const T Qr0 = Q0 * rx + Q1 * ry + Q2 * rz;
            const T Qr1 = Q1 * rx + Q3 * ry + Q4 * rz;
            const T Qr2 = Q2 * rx + Q4 * ry - (Q0 + Q3) * rz;
            const T rQr = Q0 * (rx * rx - rz * rz) + 2 * Q1 * rx * ry + 2 * Q2 * rx * rz + Q3 * (ry * ry - rz * rz) +
                          2 * Q4 * ry * rz;
            // field: A S + (B-A)(S.r) r - (C rQr r)/2 - D Q.r
            const T sE = (B - A) * sr - (T)0.5 * Cc * rQr;
            acc[0] += A * Sx + sE * rx - D * Qr0;
            acc[1] += A * Sy + sE * ry - D * Qr1;
            acc[2] += A * Sz + sE * rz - D * Qr2;
            // gradient, 5-component (xx, xy, xz, yy, yz)
            const T q5[5] = {rx * rx, rx * ry, rx * rz, ry * ry, ry * rz};
            const T srs[5] = {2 * Sx * rx, Sx * ry + rx * Sy, Sx * rz + rx * Sz, 2 * Sy * ry, Sy * rz + ry * Sz};
            const T qq[5] = {4 * Qr0 * rx, 2 * (Qr0 * ry + rx * Qr1), 2 * (Qr0 * rz + rx * Qr2), 4 * Qr1 * ry,
                             2 * (Qr1 * rz + ry * Qr2)};
            const T Qv[5] = {Q0, Q1, Q2, Q3, Q4};
            const T cq = Cc * sr + (T)0.5 * I * rQr;
            const T di = (D + E) * sr + (T)0.5 * (F + H) * rQr;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                T v = cq * q5[k] + D * srs[k] + (T)0.5 * (Gg * Qv[k] + H * qq[k]);
                if (k == 0 || k == 3) v += di;
                acc[3 + k] += v;
            }
        }
#pragma unroll
        for (int c = 0; c < 8; ++c)
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o, G);
        if (lane == 0) {
            const int64_t di0 = (int64_t)(diag_of_rhs ? diag_of_rhs[r] : 0) * n + a;
            const double ds = diagS[di0], dq = diagQ[di0];
            const double *ma = m + ((int64_t)r * n + a) * 8;
            double *o = out + ((int64_t)r * n + a) * 8;
            for (int c = 0; c < 3; ++c) o[c] += ds * ma[c] + (double)acc[c];
            for (int c = 3; c < 8; ++c) o[c] += dq * ma[c] + (double)acc[c];
        }
    }
}

// Gradient/quadrupole diagonal: 15 / (8 pi (eps - 1)) + grad_quad_2(0) / 2
// (CQ/MatrixVectorMultiply.m and CQ/RealSpace.m self terms).
__global__ void k_quad_diag(const double *__restrict__ lam, int64_t total, double self_q, double *__restrict__ diag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        diag[i] = 15.0 / (8.0 * MPS_PI * (lam[i] - 1.0)) + 0.5 * self_q;
}

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
template <typename T>
int spread_gen(const double *m, int64_t n, int nrhs, int ncomp, const int32_t *start, const T *w,
               const GridParams &gp, T *grid, cudaStream_t s) {
    MPS_CUDA_TRY(cudaMemsetAsync(grid, 0, sizeof(T) * (size_t)ncomp * nrhs * gp.G, s));
    k_spread_gen<T><<<grid_for(n * nrhs * 32, 256, 152 * 64), 256, 0, s>>>(m, n, nrhs, ncomp, start, w, gp, grid);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int contract_gen(const T *grid, int64_t n, int nrhs, int ncomp, const int32_t *start, const T *w,
                 const GridParams &gp, double *out, cudaStream_t s) {
    k_contract_gen<T><<<grid_for(n * nrhs * 32, 256, 152 * 64), 256, 0, s>>>(grid, n, nrhs, ncomp, start, w, gp, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int quad_diag(const double *lam, int64_t total, const double *gq2, double *diag, cudaStream_t s) {
    double self_q = 0.0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&self_q, gq2, sizeof(double), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_TRY(cudaStreamSynchronize(s));
    k_quad_diag<<<grid_for(total, 256), 256, 0, s>>>(lam, total, self_q, diag);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int quad_kcoef(const GridParams &gp, double *c64, float *c32, cudaStream_t s) {
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    k_quad_kcoef<<<grid_for(Gc, 256), 256, 0, s>>>(gp, c64, c32);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int scale_quad(void *spec, int nrhs, const GridParams &gp, const T *coef, cudaStream_t s) {
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    k_scale_quad<T><<<grid_for(Gc, 256), 256, 0, s>>>((typename C2T<T>::type *)spec, nrhs, gp, coef);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int quad_pair_coefs(const double *dist, int64_t np, const double *perp, const double *para, const double *qt,
                    const double *rv, int64_t ntab, double *c64, float *c32, int *err, cudaStream_t s) {
    if (np == 0) return MPS_OK;
    double rv_last = 0.0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&rv_last, rv + ntab - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_TRY(cudaStreamSynchronize(s));
    const double inv_dr = rv_last > 0 ? (double)(ntab - 1) / rv_last : 0.0;
    k_quad_pair_coefs<<<grid_for(np, 256), 256, 0, s>>>(dist, np, perp, para, qt, rv, ntab, inv_dr, c64, c32, err);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int real_space_quad(const double *m, double *out, int64_t n, int nrhs, const int64_t *row_ptr, const int32_t *nbr,
                    const T *rx, const T *ry, const T *rz, const T *coef, const double *diagS, const double *diagQ,
                    const int32_t *diag_of_rhs, cudaStream_t s) {
    constexpr int G = 8;
    k_rs_quad<T, G><<<grid_for(n * nrhs * G, 256, 152 * 64), 256, 0, s>>>(m, out, n, nrhs, row_ptr, nbr, rx, ry, rz,
                                                                          coef, diagS, diagQ, diag_of_rhs);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template int spread_gen<float>(const double *, int64_t, int, int, const int32_t *, const float *, const GridParams &,
                               float *, cudaStream_t);
template int spread_gen<double>(const double *, int64_t, int, int, const int32_t *, const double *,
                                const GridParams &, double *, cudaStream_t);
template int contract_gen<float>(const float *, int64_t, int, int, const int32_t *, const float *, const GridParams &,
                                 double *, cudaStream_t);
template int contract_gen<double>(const double *, int64_t, int, int, const int32_t *, const double *,
                                  const GridParams &, double *, cudaStream_t);
template int scale_quad<float>(void *, int, const GridParams &, const float *, cudaStream_t);
template int scale_quad<double>(void *, int, const GridParams &, const double *, cudaStream_t);
template int real_space_quad<float>(const double *, double *, int64_t, int, const int64_t *, const int32_t *,
                                    const float *, const float *, const float *, const float *, const double *,
                                    const double *, const int32_t *, cudaStream_t);
template int real_space_quad<double>(const double *, double *, int64_t, int, const int64_t *, const int32_t *,
                                     const double *, const double *, const double *, const double *, const double *,
                                     const double *, const int32_t *, cudaStream_t);

}  // namespace mps
