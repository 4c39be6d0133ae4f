// Wave-space part: Gaussian grid weights, spread (K4), Green's-function scale
// (K5) and contract (K6) (EW/ewald.py:205-599).
#include <math.h>

#include "grid.cuh"

namespace mps {

// Half-away-from-zero rounding (EW/ewald.py:71-78).
__device__ __forceinline__ double matlab_round_d(double v) {
    double a = floor(fabs(v) + 0.5);
    return v > 0 ? a : (v < 0 ? -a : 0.0 * a);
}

// ---------------------------------------------------------------------------
// Separable geometry: per particle the wrapped index of stencil column 0 and the
// three 1-D Gaussian factors (the x factor carries the normalisation constant).
// Weight of node (jx,jy,jz) = w[0][jx] w[1][jy] w[2][jz]; it equals the
// reference's const*exp(-2 xi^2 sum_d r_d^2/eta_d) evaluated at (node0+off)h - x.
// ---------------------------------------------------------------------------
__global__ void k_grid_geom(const double *__restrict__ x, int64_t n, GridParams gp, int32_t *__restrict__ start,
                            double *__restrict__ w64, float *__restrict__ w32) {
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * 3; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t / 3;
        const int d = (int)(t % 3);
        const double h = gp.h[d];
        const double xv = x[3 * a + d];
        const double node0 = matlab_round_d(__ddiv_rn(xv, h));
        const int64_t n0 = (int64_t)node0;
        start[t] = (int32_t)wrap_index(n0 - lo - 1, gp.N[d]);
        const double base = __dsub_rn(__dmul_rn(node0, h), xv);
        const double c = (d == 0) ? gp.wconst : 1.0;
        // exp(-q r_j^2) at r_j = r_0 + j h by the recurrence w_{j+1} = w_j g_j, g_j = exp(-q (2 r_0 h + (2j+1) h^2)),
        // g_{j+1} = g_j exp(-2 q h^2): three exponentials per axis instead of P (float64 exp and division are slow
        // on GB300); the weights agree with the direct exponentials to 2e-14 relative at P = 10 (3.5e-14 at P = 16)
        const double q = 2.0 * gp.xi * gp.xi * gp.inv_eta[d];
        const double r0 = base - (double)lo * h;
        double v = c * exp(-q * (r0 * r0));
        double g = exp(-q * (2.0 * r0 * h + h * h));
        const double g2 = exp(-2.0 * q * (h * h));
        for (int j = 0; j < P; ++j) {
            w64[(a * 3 + d) * P + j] = v;
            if (w32) w32[(a * 3 + d) * P + j] = (float)v;
            v *= g;
            g *= g2;
        }
    }
}

// ---------------------------------------------------------------------------
// Spread: one warp per particle; lanes walk the P x P (x,y) footprint and the z
// column; float or double atomics into planar grids [vec*3 + comp][G].
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_spread(const double *__restrict__ m, int64_t n, int nrhs,
                                                const int32_t *__restrict__ start, const T *__restrict__ w,
                                                GridParams gp, T *__restrict__ grid) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    for (int64_t a = warp; a < n; a += nw) {
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const T *wa = w + a * 3 * P;
        for (int r = 0; r < nrhs; ++r) {
            const double *ma = m + ((int64_t)r * n + a) * 3;
            const T m0 = (T)ma[0], m1 = (T)ma[1], m2 = (T)ma[2];
            T *g0 = grid + (int64_t)(3 * r) * G;
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
                    atomicAdd(g0 + node, wv * m0);
                    atomicAdd(g0 + G + node, wv * m1);
                    atomicAdd(g0 + 2 * G + node, wv * m2);
                }
            }
        }
    }
}

// Contract: one warp per particle, gather + warp reduction; out = Hk (overwrites).
template <typename T>
__global__ void __launch_bounds__(256) k_contract(const T *__restrict__ grid, int64_t n, int nrhs,
                                                  const int32_t *__restrict__ start, const T *__restrict__ w,
                                                  GridParams gp, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    for (int64_t a = warp; a < n; a += nw) {
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const T *wa = w + a * 3 * P;
        for (int r = 0; r < nrhs; ++r) {
            const T *g0 = grid + (int64_t)(3 * r) * G;
            T a0 = 0, a1 = 0, a2 = 0;
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
                    a0 += wv * g0[node];
                    a1 += wv * g0[G + node];
                    a2 += wv * g0[2 * G + node];
                }
            }
            a0 = warp_sum(a0);
            a1 = warp_sum(a1);
            a2 = warp_sum(a2);
            if (lane == 0) {
                double *o = out + ((int64_t)r * n + a) * 3;
                o[0] = (double)a0 * gp.hprod;
                o[1] = (double)a1 * gp.hprod;
                o[2] = (double)a2 * gp.hprod;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Green's coefficient over the R2C half spectrum (Nz, Ny, Nx/2+1), including the
// 1/G of the unnormalised inverse transform:
//   H(k) = 9 pi / (2|k|) J_{3/2}(|k|)^2 exp(-sum_d (1-eta_d) k_d^2 / (4 xi^2)) / |k|^2 / G
// With J_{3/2}(k) = sqrt(2 / (pi k)) (sin k / k - cos k) this is
//   9 (sin k - k cos k)^2 exp(...) / k^6,
// one sincos, one square root and one division per point (float64 issue is what this kernel costs).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double green_coef(double kx, double ky, double kz, const GridParams &gp) {
    const double k2 = kx * kx + ky * ky + kz * kz;
    if (k2 == 0.0) return 0.0;
    const double kk = sqrt(k2);
    double sk, ck;
    sincos(kk, &sk, &ck);
    const double u = sk - kk * ck;
    const double etak2 = (1.0 - gp.eta[0]) * kx * kx + (1.0 - gp.eta[1]) * ky * ky + (1.0 - gp.eta[2]) * kz * kz;
    double H = 9.0 * u * u * exp(-etak2 / (4.0 * gp.xi * gp.xi)) / (k2 * k2 * k2);
    if (!isfinite(H)) H = 0.0;
    return H;
}

// The Gaussian factor of H is separable, exp(-sum_d (1 - eta_d) k_d^2 / (4 xi^2)) =
// prod_d f_d(k_d): the per-axis factors of the spectrum's quarter, f[0 .. Nxh) for
// x, then Ny/2 + 1 for y and Nz/2 + 1 for z (one float64 exp per axis index
// instead of one per spectrum point).
__global__ void k_green_axes(GridParams gp, double *__restrict__ f) {
    const HalfQuarter q(gp.N);
    const int nx = q.Nxh, ny = q.Nyq, nz = q.Nzq;
    const double s = 1.0 / (4.0 * gp.xi * gp.xi);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx + ny + nz; i += gridDim.x * blockDim.x) {
        const int d = i < nx ? 0 : (i < nx + ny ? 1 : 2);
        const int idx = d == 0 ? i : (d == 1 ? i - nx : i - nx - ny);
        const double k = fft_freq(idx, gp.N[d]) * gp.kfac[d];
        f[i] = exp(-(1.0 - gp.eta[d]) * (k * k) * s);
    }
}

// One thread per point of the spectrum's quarter (iy <= Ny/2, iz <= Nz/2), written
// to its mirrored points as well: H depends on ky, kz only through their squares,
// and the mirrored frequencies are exact negations, so every copy is the value the
// point would compute itself (a quarter of the float64 sincos work).
//   H = 9 (sin k - k cos k)^2 f_x f_y f_z / k^6 / G.
__global__ void k_green_half(GridParams gp, const double *__restrict__ f, double *__restrict__ h64,
                             float *__restrict__ h32) {
    const HalfQuarter q(gp.N);
    const int64_t Gq = q.size();
    const double invG = 1.0 / (double)gp.G;
    const double *fy = f + q.Nxh, *fz = fy + q.Nyq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gq; t += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        q.point(t, &ix, &iy, &iz);
        const double kx = fft_freq(ix, gp.N[0]) * gp.kfac[0];
        const double ky = fft_freq(iy, gp.N[1]) * gp.kfac[1];
        const double kz = fft_freq(iz, gp.N[2]) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        double H = 0.0;
        if (k2 > 0.0) {
            const double kk = sqrt(k2);
            double sk, ck;
            sincos(kk, &sk, &ck);
            const double u = sk - kk * ck;
            H = 9.0 * u * u * (f[ix] * fy[iy] * fz[iz]) / (k2 * k2 * k2) * invG;
            if (!isfinite(H)) H = 0.0;
        }
        mirror_points(q, ix, iy, iz, [&](int64_t i, int, int) {
            h64[i] = H;
            if (h32) h32[i] = (float)H;
        });
    }
}

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
    using type = float2;
};
template <>
struct Cplx<double> {
    using type = double2;
};

// Scale on the half spectrum, in place, for 3*nrhs component spectra.
// Tensor H khat khat^T with the entries that couple an unpaired Nyquist axis to
// a non-Nyquist axis set to zero: the real part of the reference's operator.
template <typename T>
__global__ void k_scale_half(typename Cplx<T>::type *__restrict__ spec, int nrhs, GridParams gp,
                             const T *__restrict__ Hh) {
    using C = typename Cplx<T>::type;
    const int Nxh = gp.N[0] / 2 + 1;
    const int64_t Gc = (int64_t)Nxh * gp.N[1] * gp.N[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gc; t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t % Nxh);
        const int iy = (int)((t / Nxh) % gp.N[1]);
        const int iz = (int)(t / ((int64_t)Nxh * gp.N[1]));
        const T kx = (T)(fft_freq(ix, gp.N[0]) * gp.kfac[0]);
        const T ky = (T)(fft_freq(iy, gp.N[1]) * gp.kfac[1]);
        const T kz = (T)(fft_freq(iz, gp.N[2]) * gp.kfac[2]);
        const T k2 = kx * kx + ky * ky + kz * kz;
        const T H = Hh[t];
        const bool nx = (gp.N[0] % 2 == 0) && (ix == gp.N[0] / 2);
        const bool ny = (gp.N[1] % 2 == 0) && (iy == gp.N[1] / 2);
        const bool nz = (gp.N[2] % 2 == 0) && (iz == gp.N[2] / 2);
        T q[3] = {0, 0, 0};
        if (k2 > (T)0) {
            const T inv = (T)1 / sqrt(k2);
            q[0] = kx * inv;
            q[1] = ky * inv;
            q[2] = kz * inv;
        }
        const bool ny3[3] = {nx, ny, nz};
        T Tm[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Tm[i][j] = (ny3[i] == ny3[j]) ? H * q[i] * q[j] : (T)0;
        for (int r = 0; r < nrhs; ++r) {
            C *s = spec + (int64_t)(3 * r) * Gc + t;
            const C f0 = s[0], f1 = s[Gc], f2 = s[2 * Gc];
            C g[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                g[i].x = Tm[i][0] * f0.x + Tm[i][1] * f1.x + Tm[i][2] * f2.x;
                g[i].y = Tm[i][0] * f0.y + Tm[i][1] * f1.y + Tm[i][2] * f2.y;
            }
            s[0] = g[0];
            s[Gc] = g[1];
            s[2 * Gc] = g[2];
        }
    }
}

// Full-spectrum complex scale in unshifted order (the reference's own pipeline).
__global__ void k_scale_full_c2c(double2 *__restrict__ spec, GridParams gp) {
    const int64_t G = gp.G;
    const double invG = 1.0 / (double)G;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < G; t += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(t % gp.N[0]);
        const int iy = (int)((t / gp.N[0]) % gp.N[1]);
        const int iz = (int)(t / ((int64_t)gp.N[0] * gp.N[1]));
        const double kx = fft_freq(ix, gp.N[0]) * gp.kfac[0];
        const double ky = fft_freq(iy, gp.N[1]) * gp.kfac[1];
        const double kz = fft_freq(iz, gp.N[2]) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        double2 *s = spec + t;
        if (k2 == 0.0) {
            s[0] = make_double2(0, 0);
            s[G] = make_double2(0, 0);
            s[2 * G] = make_double2(0, 0);
            continue;
        }
        const double H = green_coef(kx, ky, kz, gp) * invG;
        const double inv = 1.0 / sqrt(k2);
        const double q0 = kx * inv, q1 = ky * inv, q2 = kz * inv;
        const double2 f0 = s[0], f1 = s[G], f2 = s[2 * G];
        const double dr = H * (q0 * f0.x + q1 * f1.x + q2 * f2.x);
        const double di = H * (q0 * f0.y + q1 * f1.y + q2 * f2.y);
        s[0] = make_double2(dr * q0, di * q0);
        s[G] = make_double2(dr * q1, di * q1);
        s[2 * G] = make_double2(dr * q2, di * q2);
    }
}

__global__ void k_pack_c(const double *__restrict__ re_im, int64_t G, double2 *__restrict__ c) {
    // re_im: [2][3][G] -> c: [3][G]
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * G; t += (int64_t)gridDim.x * blockDim.x)
        c[t] = make_double2(re_im[t], re_im[3 * G + t]);
}

__global__ void k_unpack_c(const double2 *__restrict__ c, int64_t G, double *__restrict__ re_im) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * G; t += (int64_t)gridDim.x * blockDim.x) {
        re_im[t] = c[t].x;
        re_im[3 * G + t] = c[t].y;
    }
}

// ---------------------------------------------------------------------------
// Drop-in kernels working on the reference's dense (N, P^3) weight arrays.
// ---------------------------------------------------------------------------
__global__ void k_precalc(int P, double hx, double hy, double hz, int64_t *__restrict__ off, double *__restrict__ offxyz) {
    const int lo = (P - 1) / 2;
    const int64_t P3 = (int64_t)P * P * P;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < P3; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t o[3] = {j % P - lo, (j / P) % P - lo, j / ((int64_t)P * P) - lo};
        const double h[3] = {hx, hy, hz};
        for (int d = 0; d < 3; ++d) {
            off[3 * j + d] = o[d];
            offxyz[3 * j + d] = (double)o[d] * h[d];
        }
    }
}

__global__ void k_grid_dense(const double *__restrict__ x, int64_t n, GridParams gp, int64_t *__restrict__ lin,
                             double *__restrict__ ws, double *__restrict__ wc) {
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    const int64_t P3 = (int64_t)P * P * P;
    const double c2 = __dmul_rn(-2.0, __dmul_rn(gp.xi, gp.xi));
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * P3; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t / P3;
        const int64_t j = t % P3;
        const int64_t o[3] = {j % P - lo, (j / P) % P - lo, j / ((int64_t)P * P) - lo};
        int64_t node[3];
        double s = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double h = gp.h[d];
            const double n0 = matlab_round_d(__ddiv_rn(x[3 * a + d], h));
            node[d] = wrap_index((int64_t)n0 + o[d] - 1, gp.N[d]);
            const double base = __dsub_rn(__dmul_rn(n0, h), x[3 * a + d]);
            const double r = __dadd_rn(base, __dmul_rn((double)o[d], h));
            const double term = __dmul_rn(__dmul_rn(r, r), gp.inv_eta[d]);
            s = (d == 0) ? term : __dadd_rn(s, term);
        }
        lin[t] = node[0] + (int64_t)gp.N[0] * node[1] + (int64_t)gp.N[0] * gp.N[1] * node[2];
        const double wv = __dmul_rn(gp.wconst, exp(__dmul_rn(c2, s)));
        ws[t] = wv;
        wc[t] = __dmul_rn(wv, gp.hprod);
    }
}

__global__ void k_spread_dense(const double *__restrict__ m, int64_t n, int64_t nvec, const int64_t *__restrict__ lin,
                               const double *__restrict__ w, int64_t P3, int64_t G, double *__restrict__ grid) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * P3; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t / P3;
        const int64_t node = lin[t];
        const double wv = w[t];
        for (int64_t v = 0; v < nvec; ++v)
            for (int c = 0; c < 3; ++c) atomicAdd(grid + (v * 3 + c) * G + node, wv * m[(v * n + a) * 3 + c]);
    }
}

__global__ void k_contract_dense(const double *__restrict__ grid, int64_t n, int64_t nvec,
                                 const int64_t *__restrict__ lin, const double *__restrict__ w, int64_t P3, int64_t G,
                                 double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a = warp; a < n; a += nw) {
        for (int64_t v = 0; v < nvec; ++v) {
            double acc[3] = {0, 0, 0};
            for (int64_t j = lane; j < P3; j += 32) {
                const int64_t node = lin[a * P3 + j];
                const double wv = w[a * P3 + j];
                for (int c = 0; c < 3; ++c) acc[c] += wv * grid[(v * 3 + c) * G + node];
            }
            for (int c = 0; c < 3; ++c) {
                double s = warp_sum(acc[c]);
                if (lane == 0) out[(v * n + a) * 3 + c] = s;
            }
        }
    }
}

// fftshift-ordered k-space arrays in the reference's (Nx,Ny,Nz[,3]) C layout.
__global__ void k_kspace_shifted(GridParams gp, double *__restrict__ khat, double *__restrict__ Hc) {
    const int64_t G = gp.G;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < G; t += (int64_t)gridDim.x * blockDim.x) {
        const int iz = (int)(t % gp.N[2]);
        const int iy = (int)((t / gp.N[2]) % gp.N[1]);
        const int ix = (int)(t / ((int64_t)gp.N[2] * gp.N[1]));
        const double kx = (double)(ix - gp.N[0] / 2) * gp.kfac[0];
        const double ky = (double)(iy - gp.N[1] / 2) * gp.kfac[1];
        const double kz = (double)(iz - gp.N[2] / 2) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        double den = sqrt(k2);
        if (den == 0.0) den = 1.0;
        khat[3 * t + 0] = kx / den;
        khat[3 * t + 1] = ky / den;
        khat[3 * t + 2] = kz / den;
        Hc[t] = green_coef(kx, ky, kz, gp);
    }
}

__global__ void k_scale_dense(const double2 *__restrict__ fH, const double *__restrict__ khat,
                              const double *__restrict__ Hc, int64_t G, double2 *__restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < G; t += (int64_t)gridDim.x * blockDim.x) {
        const double q0 = khat[3 * t], q1 = khat[3 * t + 1], q2 = khat[3 * t + 2];
        const double2 f0 = fH[3 * t], f1 = fH[3 * t + 1], f2 = fH[3 * t + 2];
        const double dr = Hc[t] * (q0 * f0.x + q1 * f1.x + q2 * f2.x);
        const double di = Hc[t] * (q0 * f0.y + q1 * f1.y + q2 * f2.y);
        out[3 * t + 0] = make_double2(dr * q0, di * q0);
        out[3 * t + 1] = make_double2(dr * q1, di * q1);
        out[3 * t + 2] = make_double2(dr * q2, di * q2);
    }
}

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
GridParams make_grid_params(const int64_t *Ngrid, const double *box, double xi, const double *eta_in, int P) {
    GridParams gp;
    gp.P = P;
    gp.xi = xi;
    gp.G = 1;
    double etaprod = 1.0;
    gp.hprod = 1.0;
    for (int d = 0; d < 3; ++d) {
        gp.N[d] = (int)Ngrid[d];
        gp.G *= Ngrid[d];
        gp.h[d] = box[d] / (double)Ngrid[d];
        gp.eta[d] = (eta_in && eta_in[d] > 0) ? eta_in[d] : P * (gp.h[d] * xi) * (gp.h[d] * xi) / MPS_PI;
        gp.inv_eta[d] = 1.0 / gp.eta[d];
        gp.kfac[d] = 2.0 * MPS_PI / box[d];
        etaprod *= gp.eta[d];
        gp.hprod *= gp.h[d];
    }
    gp.wconst = pow(2.0 * xi * xi / MPS_PI, 1.5) * sqrt(1.0 / etaprod);
    return gp;
}

int grid_geometry(const double *x, int64_t n, const GridParams &gp, int32_t *start, double *w64, float *w32,
                  cudaStream_t s) {
    if (n == 0) return MPS_OK;
    k_grid_geom<<<grid_for(3 * n, 256), 256, 0, s>>>(x, n, gp, start, w64, w32);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int green_half(const GridParams &gp, double *h64, float *h32, cudaStream_t s) {
    const HalfQuarter q(gp.N);
    const int nf = q.Nxh + q.Nyq + q.Nzq;
    double *f = nullptr;
    MPS_CUDA_TRY(cudaMallocAsync((void **)&f, sizeof(double) * nf, s));
    k_green_axes<<<grid_for(nf, 128), 128, 0, s>>>(gp, f);
    MPS_LAUNCH_CHECK();
    k_green_half<<<grid_for(q.size(), 256), 256, 0, s>>>(gp, f, h64, h32);
    MPS_LAUNCH_CHECK();
    MPS_CUDA_TRY(cudaFreeAsync(f, s));
    return MPS_OK;
}

template <typename T>
int spread(const double *m, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp, T *grid,
           cudaStream_t s) {
    MPS_CUDA_TRY(cudaMemsetAsync(grid, 0, sizeof(T) * 3 * nrhs * gp.G, s));
    if (n == 0) return MPS_OK;
    k_spread<T><<<grid_for(n * 32, 256, 152 * 64), 256, 0, s>>>(m, n, nrhs, start, w, gp, grid);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int contract(const T *grid, int64_t n, int nrhs, const int32_t *start, const T *w, const GridParams &gp, double *out,
             cudaStream_t s) {
    if (n == 0) return MPS_OK;
    k_contract<T><<<grid_for(n * 32, 256, 152 * 64), 256, 0, s>>>(grid, n, nrhs, start, w, gp, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int scale_half(void *spec, int nrhs, const GridParams &gp, const T *Hh, cudaStream_t s) {
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    k_scale_half<T><<<grid_for(Gc, 256), 256, 0, s>>>((typename Cplx<T>::type *)spec, nrhs, gp, Hh);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int scale_full_c2c(void *spec, const GridParams &gp, cudaStream_t s) {
    k_scale_full_c2c<<<grid_for(gp.G, 256), 256, 0, s>>>((double2 *)spec, gp);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int pack_complex(const double *re_im, int64_t G, void *c, cudaStream_t s) {
    k_pack_c<<<grid_for(3 * G, 256), 256, 0, s>>>(re_im, G, (double2 *)c);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int unpack_complex(const void *c, int64_t G, double *re_im, cudaStream_t s) {
    k_unpack_c<<<grid_for(3 * G, 256), 256, 0, s>>>((const double2 *)c, G, re_im);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template int spread<float>(const double *, int64_t, int, const int32_t *, const float *, const GridParams &, float *,
                           cudaStream_t);
template int spread<double>(const double *, int64_t, int, const int32_t *, const double *, const GridParams &,
                            double *, cudaStream_t);
template int contract<float>(const float *, int64_t, int, const int32_t *, const float *, const GridParams &, double *,
                             cudaStream_t);
template int contract<double>(const double *, int64_t, int, const int32_t *, const double *, const GridParams &,
                              double *, cudaStream_t);
template int scale_half<float>(void *, int, const GridParams &, const float *, cudaStream_t);
template int scale_half<double>(void *, int, const GridParams &, const double *, cudaStream_t);

}  // namespace mps

using namespace mps;

static bool valid3(const int64_t *N) { return N && N[0] > 0 && N[1] > 0 && N[2] > 0; }

extern "C" int mps_pre_calculations(int P, const double *h, int64_t *offset, double *offsetxyz, mps_stream_t stream) {
    if (P < 1 || !h || !offset || !offsetxyz) return MPS_BAD_ARG;
    int64_t P3 = (int64_t)P * P * P;
    k_precalc<<<grid_for(P3, 256), 256, 0, (cudaStream_t)stream>>>(P, h[0], h[1], h[2], offset, offsetxyz);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_grid_kernel(const double *x, int64_t n, const int64_t *Ngrid, const double *h, double xi,
                               const double *eta, int P, int64_t *linnode, double *w_spread, double *w_contract,
                               mps_stream_t stream) {
    if (n < 0 || P < 1 || !valid3(Ngrid) || !h || !eta) return MPS_BAD_ARG;
    if (n == 0) return MPS_OK;
    double box[3] = {h[0] * Ngrid[0], h[1] * Ngrid[1], h[2] * Ngrid[2]};
    GridParams gp = make_grid_params(Ngrid, box, xi, eta, P);
    for (int d = 0; d < 3; ++d) {
        gp.h[d] = h[d];
        gp.eta[d] = eta[d];
        gp.inv_eta[d] = 1.0 / eta[d];
    }
    gp.hprod = h[0] * h[1] * h[2];
    gp.wconst = pow(2.0 * xi * xi / MPS_PI, 1.5) * sqrt(1.0 / (eta[0] * eta[1] * eta[2]));
    int64_t P3 = (int64_t)P * P * P;
    k_grid_dense<<<grid_for(n * P3, 256), 256, 0, (cudaStream_t)stream>>>(x, n, gp, linnode, w_spread, w_contract);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_spread_fast(const double *m, int64_t n, int64_t nvec, const int64_t *Ngrid, const int64_t *linnode,
                               const double *w_spread, int64_t P3, double *grid, mps_stream_t stream) {
    if (n < 0 || nvec < 1 || !valid3(Ngrid) || P3 < 1) return MPS_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int64_t G = Ngrid[0] * Ngrid[1] * Ngrid[2];
    MPS_CUDA_TRY(cudaMemsetAsync(grid, 0, sizeof(double) * 3 * nvec * G, s));
    if (n == 0) return MPS_OK;
    k_spread_dense<<<grid_for(n * P3, 256), 256, 0, s>>>(m, n, nvec, linnode, w_spread, P3, G, grid);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_contract_fast(const double *grid, int64_t n, int64_t nvec, const int64_t *Ngrid,
                                 const int64_t *linnode, const double *w_contract, int64_t P3, double *out,
                                 mps_stream_t stream) {
    if (n < 0 || nvec < 1 || !valid3(Ngrid) || P3 < 1) return MPS_BAD_ARG;
    if (n == 0) return MPS_OK;
    int64_t G = Ngrid[0] * Ngrid[1] * Ngrid[2];
    k_contract_dense<<<grid_for(n * 32, 256), 256, 0, (cudaStream_t)stream>>>(grid, n, nvec, linnode, w_contract, P3,
                                                                             G, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_precompute_kspace(const int64_t *Ngrid, const double *box, double xi, const double *eta,
                                     double *khat, double *Hcoef, mps_stream_t stream) {
    if (!valid3(Ngrid) || !box || !eta || !khat || !Hcoef) return MPS_BAD_ARG;
    GridParams gp = make_grid_params(Ngrid, box, xi, eta, 1);
    k_kspace_shifted<<<grid_for(gp.G, 256), 256, 0, (cudaStream_t)stream>>>(gp, khat, Hcoef);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_scale_fast(const double *fH, const double *khat, const double *Hcoef, int64_t G, double *out,
                              mps_stream_t stream) {
    if (G < 0 || (G > 0 && (!fH || !khat || !Hcoef || !out))) return MPS_BAD_ARG;
    if (G == 0) return MPS_OK;
    k_scale_dense<<<grid_for(G, 256), 256, 0, (cudaStream_t)stream>>>((const double2 *)fH, khat, Hcoef, G,
                                                                       (double2 *)out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}
