// Polydisperse dipole operator (spheres of different radii; the MATLAB variant
// Capacitance_Sizes, cited CS/).
//
//   real space   dielectric 3/(4 pi a^3 (eps - 1)), self value of the (a_i, a_i)
//                coupling, pair couplings of the two radii (CS/RealSpace.m:18-76)
//                either interpolated from the per-radius-pair tables of
//                CS/RealSpaceTable.m or evaluated in closed form at the exact
//                separation (continuous radii)
//   wave space   the dipoles are spread as charges onto ONE scalar grid with the
//                sphere kernel K(d) r-hat.p (CS/Spread.m:39-72), scaled by
//                exp(-(1-eta) q^2 / 4 xi^2) / q^2 (CS/Scale.m:16-21; even in q, so
//                the half-spectrum real transforms are exact), and contracted with
//                prod(h) sum K(d) r-hat (CS/Contract.m:39-73)
//
// The kernel values K(d)/d of every particle's P^3 stencil are computed once
// per system; the spread and contract rebuild r = node - x from the particle's
// base offset.
#include <math.h>

#include <cstdlib>

#include "sizes.cuh"

namespace mps {

// ---------------------------------------------------------------------------
// Couplings (CS/RealSpaceTable.m:34-146), written with shared subexpressions.
// ---------------------------------------------------------------------------
__host__ __device__ inline void cs_couplings(double r, double ai, double aj, double xi, double *perp, double *para) {
    const double pi = MPS_PI;
    const double sp3 = pi * sqrt(pi);
    const double x2 = xi * xi, x4 = x2 * x2, x6 = x4 * x2;
    const double s = ai + aj, d = ai - aj;
    const double ai2 = ai * ai, aj2 = aj * aj, ai3 = ai2 * ai, aj3 = aj2 * aj;
    const double A3 = ai3 * aj3;
    const double c1 = 4 * ai3 - 3 * ai2 * aj - 3 * ai * aj2 + 4 * aj3;
    const double c2 = 4 * ai3 + 3 * ai2 * aj - 3 * ai * aj2 - 4 * aj3;
    const double c3 = ai3 - 3 * ai2 * aj - 3 * ai * aj2 + aj3;
    const double c4 = ai3 + 3 * ai2 * aj - 3 * ai * aj2 - aj3;
    const double q1 = ai2 - 4 * ai * aj + aj2;
    const double q2 = ai2 + 4 * ai * aj + aj2;
    const double sq = ai2 + aj2;
    const double dq = (ai2 - aj2) * (ai2 - aj2);
    const double s2 = s * s, d2 = d * d;
    const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r, r6 = r3 * r3;
    const double e1 = exp(-(r + s) * (r + s) * x2), e2 = exp(-(r - s) * (r - s) * x2);
    const double e3 = exp(-(r - d) * (r - d) * x2), e4 = exp(-(r + d) * (r + d) * x2);
    const double g1 = erfc((r + s) * xi), g2 = erfc((r - s) * xi), g3 = erfc((r - d) * xi), g4 = erfc((r + d) * xi);
    const double base_s = r * (3 - 12 * (ai2 - ai * aj + aj2) * x2 - 4 * s2 * q1 * x4);
    const double tail_s = 3 * s + 4 * c1 * x2 + 4 * s2 * s * q1 * x4;
    const double base_d = r * (-3 + 12 * (ai2 + ai * aj + aj2) * x2 + 4 * d2 * q2 * x4);
    const double tail_d = 3 * d + 4 * c2 * x2 + 4 * d2 * d * q2 * x4;
    // I - rr part
    {
        const double k5 = 1.0 / (1024 * sp3 * A3 * r3 * xi * x4);
        const double mid_s = r3 * (16 * x2 + 8 * (-4 * ai2 + ai * aj - 4 * aj2) * x4);
        const double mid_d = r3 * (-16 * x2 + 8 * (4 * ai2 + ai * aj + 4 * aj2) * x4);
        const double f1 = k5 * (4 * r5 * x4 - 4 * s * r4 * x4 + mid_s + r2 * (-12 * s * x2 - 8 * c1 * x4) + base_s + tail_s);
        const double f2 = k5 * (4 * r5 * x4 + 4 * s * r4 * x4 + mid_s + r2 * (12 * s * x2 + 8 * c1 * x4) + base_s - tail_s);
        const double f3 = k5 * (-4 * r5 * x4 - 4 * d * r4 * x4 + mid_d + r2 * (-12 * d * x2 - 8 * c2 * x4) + base_d + tail_d);
        const double f4 = k5 * (-4 * r5 * x4 + 4 * d * r4 * x4 + mid_d + r2 * (12 * d * x2 + 8 * c2 * x4) + base_d - tail_d);
        const double k6 = 1.0 / (2048 * pi * A3 * r3 * x6);
        const double gs = r2 * (-18 * x2 + 72 * sq * x4 + 72 * dq * x6) + 3 - 18 * sq * x2 - 36 * dq * x4;
        const double t4 = 36 * r4 * x4 * (-1 + 2 * sq * x2);
        const double f5 = k6 * (-8 * r6 * x6 + t4 + 128 * (ai3 + aj3) * r3 * x6 + gs - 8 * s2 * s2 * q1 * x6);
        const double f6 = k6 * (-8 * r6 * x6 + t4 - 128 * (ai3 + aj3) * r3 * x6 + gs - 8 * s2 * s2 * q1 * x6);
        const double f7 = k6 * (8 * r6 * x6 - t4 + 128 * (ai3 - aj3) * r3 * x6 - gs + 8 * d2 * d2 * q2 * x6);
        const double f8 = k6 * (8 * r6 * x6 - t4 - 128 * (ai3 - aj3) * r3 * x6 - gs + 8 * d2 * d2 * q2 * x6);
        double reg = 0.0;
        if (r < s && r >= d && r >= -d)
            reg = (s - r) * (s - r) * (s - r) / (128 * pi * A3 * r3) * (-r3 - 3 * s * r2 + 3 * q1 * r + c3);
        else if (r < -d && r > d)
            reg = (r3 - aj3) / (4 * pi * aj3 * r3);
        else if (r < d && r > -d)
            reg = (r3 - ai3) / (4 * pi * ai3 * r3);
        *perp = f1 * e1 + f2 * e2 + f3 * e3 + f4 * e4 + f5 * g1 + f6 * g2 + f7 * g3 + f8 * g4 + reg;
    }
    // rr part
    {
        const double k5 = 1.0 / (512 * sp3 * A3 * r3 * xi * x4);
        const double mid_s = r3 * (14 * x2 - 4 * (7 * ai2 - 4 * ai * aj + 7 * aj2) * x4);
        const double mid_d = r3 * (-14 * x2 + 4 * (7 * ai2 + 4 * ai * aj + 7 * aj2) * x4);
        const double f1 = k5 * (8 * r5 * x4 - 8 * s * r4 * x4 + mid_s + r2 * (-6 * s * x2 - 4 * c3 * x4) - base_s - tail_s);
        const double f2 = k5 * (8 * r5 * x4 + 8 * s * r4 * x4 + mid_s + r2 * (6 * s * x2 + 4 * c3 * x4) - base_s + tail_s);
        const double f3 = k5 * (-8 * r5 * x4 - 8 * d * r4 * x4 + mid_d + r2 * (-6 * d * x2 - 4 * c4 * x4) - base_d - tail_d);
        const double f4 = k5 * (-8 * r5 * x4 + 8 * d * r4 * x4 + mid_d + r2 * (6 * d * x2 + 4 * c4 * x4) - base_d + tail_d);
        const double k6 = 1.0 / (1024 * pi * A3 * r3 * x6);
        const double hs = -3 + 18 * sq * x2 + 36 * dq * x4;
        const double t4 = 36 * r4 * x4 * (-1 + 2 * sq * x2);
        const double f5 = k6 * (-16 * r6 * x6 + t4 + 64 * (ai3 + aj3) * r3 * x6 + hs + 8 * s2 * s2 * q1 * x6);
        const double f6 = k6 * (-16 * r6 * x6 + t4 - 64 * (ai3 + aj3) * r3 * x6 + hs + 8 * s2 * s2 * q1 * x6);
        const double f7 = k6 * (16 * r6 * x6 - t4 + 64 * (ai3 - aj3) * r3 * x6 - hs - 8 * d2 * d2 * q2 * x6);
        const double f8 = k6 * (16 * r6 * x6 - t4 - 64 * (ai3 - aj3) * r3 * x6 - hs - 8 * d2 * d2 * q2 * x6);
        double reg = 0.0;
        if (r < s && r >= d && r >= -d)
            reg = -1.0 / (64 * pi * A3 * r3) * (s2 * s2 * q1 - 8 * (ai3 + aj3) * r3 + 9 * sq * r4 - 2 * r6);
        else if (r < -d && r > d)
            reg = (r3 + 2 * aj3) / (4 * pi * aj3 * r3);
        else if (r < d && r > -d)
            reg = (r3 + 2 * ai3) / (4 * pi * ai3 * r3);
        *para = f1 * e1 + f2 * e2 + f3 * e3 + f4 * e4 + f5 * g1 + f6 * g2 + f7 * g3 + f8 * g4 + reg;
    }
}

// r -> 0 value of both parts (CS/RealSpaceTable.m:87-89).
__host__ __device__ inline double cs_self(double ai, double aj, double xi) {
    const double pi = MPS_PI;
    const double x2 = xi * xi;
    const double ai3 = ai * ai * ai, aj3 = aj * aj * aj;
    return 1.0 / (16 * pi * sqrt(pi) * ai3 * aj3 * xi * x2) *
               ((1 - 2 * ai * ai * x2 + 2 * ai * aj * x2 - 2 * aj * aj * x2) * exp(-(ai + aj) * (ai + aj) * x2) +
                (-1 + 2 * ai * ai * x2 + 2 * ai * aj * x2 + 2 * aj * aj * x2) * exp(-(ai - aj) * (ai - aj) * x2)) +
           1.0 / (8 * pi * ai3 * aj3) * ((ai3 - aj3) * erf((ai - aj) * xi) - (ai3 + aj3) * erf((ai + aj) * xi)) +
           fmin(ai3, aj3) / (4 * pi * ai3 * aj3);
}

// Column of the radius pair (i, j): upper triangle in row order.
__host__ __device__ inline int64_t cs_column(int64_t i, int64_t j, int64_t M) {
    if (i > j) {
        const int64_t t = i;
        i = j;
        j = t;
    }
    return i * M - i * (i - 1) / 2 + (j - i);
}

__global__ void k_cs_table(const double *__restrict__ r, int64_t n, const double *__restrict__ a, int64_t M,
                           double xi, double *__restrict__ perp, double *__restrict__ para) {
    const int64_t m = M * (M + 1) / 2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * m; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, col = t / n;
        // invert the column index
        int64_t ci = 0, rem = col;
        while (rem >= M - ci) {
            rem -= M - ci;
            ++ci;
        }
        const int64_t cj = ci + rem;
        double pp, pa;
        if (i == 0) {
            pp = pa = cs_self(a[ci], a[cj], xi);
        } else {
            cs_couplings(r[i], a[ci], a[cj], xi, &pp, &pa);
        }
        perp[col * n + i] = pp;
        para[col * n + i] = pa;
    }
}

// First table entry >= d (search from a uniform-spacing guess).
__device__ __forceinline__ int64_t cs_search(const double *__restrict__ rv, int64_t n, double d) {
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

// Per-pair couplings of the CSR list: A (I - rr) and B - A, float64 and float32.
__global__ void k_cs_pair_coefs(const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ nbr,
                                const double *__restrict__ dist, int64_t n, const double *__restrict__ radius,
                                const int32_t *__restrict__ cls, int64_t M, const double *__restrict__ tab,
                                const double *__restrict__ rv, int64_t ntab, double xi, double *__restrict__ A64,
                                double *__restrict__ BA64, float *__restrict__ A32, float *__restrict__ BA32,
                                int *__restrict__ err) {
    const int64_t m = M * (M + 1) / 2;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t e = row_ptr[a]; e < row_ptr[a + 1]; ++e) {
            const int32_t b = nbr[e];
            const double d = dist[e];
            double A = 0.0, B = 0.0;
            if (tab) {
                const int64_t col = cs_column(cls[a], cls[b], M);
                const int64_t i = cs_search(rv, ntab, d);
                if (i <= 0 || i >= ntab) {
                    atomicExch(err, 1);
                } else {
                    const double rl = rv[i - 1], rh = rv[i];
                    const double *pp = tab + col * ntab, *pa = tab + (m + col) * ntab;
                    A = pp[i - 1] * (rh - d) / (rh - rl) + pp[i] * (d - rl) / (rh - rl);
                    B = pa[i - 1] * (rh - d) / (rh - rl) + pa[i] * (d - rl) / (rh - rl);
                }
            } else {
                cs_couplings(d, radius[a], radius[b], xi, &A, &B);
            }
            A64[e] = A;
            BA64[e] = B - A;
            A32[e] = (float)A;
            BA32[e] = (float)(B - A);
        }
    }
}

__global__ void k_cs_diag(const double *__restrict__ lam, int64_t n, int64_t nsets, const double *__restrict__ radius,
                          const int32_t *__restrict__ cls, int64_t M, const double *__restrict__ tab, int64_t ntab,
                          double xi, double *__restrict__ diag) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * nsets; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t % n;
        const double ra = radius[a];
        const double self = tab ? tab[cs_column(cls[a], cls[a], M) * ntab] : cs_self(ra, ra, xi);
        diag[t] = 3.0 / (4.0 * MPS_PI * ra * ra * ra * (lam[t] - 1.0)) + self;
    }
}

// Half-away-from-zero rounding of x / h (the MATLAB round of CS/Spread.m:37).
__device__ __forceinline__ double cs_round(double v) {
    const double a = floor(fabs(v) + 0.5);
    return v > 0 ? a : (v < 0 ? -a : 0.0 * a);
}

// Per particle: wrapped index of stencil column 0, base = node0 h - x, and the
// kernel K(d)/d at every node of the P^3 stencil (x fastest).
__global__ void k_cs_geom(const double *__restrict__ x, int64_t n, GridParams gp, const double *__restrict__ radius,
                          double xi, double eta, int32_t *__restrict__ start, double *__restrict__ base,
                          double *__restrict__ g64, float *__restrict__ g32) {
    const int P = gp.P;
    const int64_t P3 = (int64_t)P * P * P;
    const int lo = (P - 1) / 2;
    const double pi = MPS_PI;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * P3; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t / P3;
        const int64_t l = t % P3;
        const int o[3] = {(int)(l % P) - lo, (int)((l / P) % P) - lo, (int)(l / ((int64_t)P * P)) - lo};
        double r[3];
        for (int k = 0; k < 3; ++k) {
            const double xv = x[3 * a + k];
            const double node0 = cs_round(__ddiv_rn(xv, gp.h[k]));
            if (l == 0) {
                start[3 * a + k] = (int32_t)wrap_index((int64_t)node0 - lo - 1, gp.N[k]);
                base[3 * a + k] = node0 * gp.h[k] - xv;
            }
            r[k] = (node0 * gp.h[k] + (double)o[k] * gp.h[k]) - xv;
        }
        const double d = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double ra = radius[a];
        double v;
        if (d < 1e-6) {
            // small-d form as the reference writes it (CS/Spread.m:60-61)
            v = 8 * sqrt(2.0) * pow(xi, 5) * exp(-2 * ra * xi * xi / eta) / (pi * sqrt(pi) * pow(eta, 2.5));
        } else {
            const double K = 3.0 / (8 * sqrt(2.0) * pi * sqrt(pi) * ra * ra * ra * sqrt(eta) * xi * d * d) *
                             ((eta + 4 * ra * xi * xi * d) * exp(-2 * (d + ra) * (d + ra) * xi * xi / eta) -
                              (eta - 4 * ra * xi * xi * d) * exp(-2 * (d - ra) * (d - ra) * xi * xi / eta));
            v = K / d;
        }
        g64[t] = v;
        if (g32) g32[t] = (float)v;
    }
}

__global__ void k_cs_green(GridParams gp, double eta, double xi, double *__restrict__ c64, float *__restrict__ c32) {
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
        const double q2 = kx * kx + ky * ky + kz * kz;
        const double v = q2 > 0 ? exp(-(1 - eta) * q2 / (4 * xi * xi)) / q2 * invG : 0.0;
        c64[t] = v;
        if (c32) c32[t] = (float)v;
    }
}

// Spread: a warp per (particle, block of RB vectors); lanes walk the (x, y)
// footprint.  The particle's node weights K(d)/d (P^3 per particle) are read once
// per block of vectors instead of once per vector: with a spectrum batch (3 fields x
// K contrasts) they were the dominant read.
template <typename T, int RB, int MB = 1>
__global__ void __launch_bounds__(256, MB) k_spread_cs(const double *__restrict__ m, int64_t n, int nrhs,
                                                   const int32_t *__restrict__ start, const double *__restrict__ base,
                                                   const T *__restrict__ g, GridParams gp, T *__restrict__ grid) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t P3 = (int64_t)P * P * P;
    const int nblk = (nrhs + RB - 1) / RB;
    for (int64_t t = warp; t < n * nblk; t += nw) {
        const int64_t a = gp.order ? (int64_t)gp.order[t % n] : t % n;
        const int r0 = (int)(t / n) * RB;
        const int cnt = min(RB, nrhs - r0);
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        T px[RB], py[RB], pz[RB];
#pragma unroll
        for (int q = 0; q < RB; ++q) {
            const double *ma = m + ((int64_t)(r0 + (q < cnt ? q : 0)) * n + a) * 3;
            px[q] = (T)ma[0];
            py[q] = (T)ma[1];
            pz[q] = (T)ma[2];
        }
        const T bx = (T)(base[3 * a] - lo * gp.h[0]), by = (T)(base[3 * a + 1] - lo * gp.h[1]),
                bz = (T)(base[3 * a + 2] - lo * gp.h[2]);
        const T hx = (T)gp.h[0], hy = (T)gp.h[1], hz = (T)gp.h[2];
        const T *ga = g + a * P3;
        T *gr = grid + (int64_t)r0 * gp.G;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const T rx = bx + (T)jx * hx, ry = by + (T)jy * hy;
            T pxy[RB];
#pragma unroll
            for (int q = 0; q < RB; ++q) pxy[q] = rx * px[q] + ry * py[q];
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const T rz = bz + (T)jz * hz;
                const T wv = ga[jx + P * (jy + P * jz)];
                T *node = gr + rowb + (int64_t)Nx * Ny * iz;
#pragma unroll
                for (int q = 0; q < RB; ++q)
                    if (q < cnt) atomicAdd(node + (int64_t)q * gp.G, wv * (pxy[q] + rz * pz[q]));
            }
        }
    }
}

template <typename T>
struct CsCplx;
template <>
struct CsCplx<float> {
    using type = float2;
};
template <>
struct CsCplx<double> {
    using type = double2;
};

// spec[r][k] *= coef[k]: one thread per spectrum point reads its coefficient once for every vector, with one
// complex (8 or 16 byte) load and store per value.
template <typename T>
__global__ void k_scale_cs(T *__restrict__ spec, int nrhs, int64_t Gc, const T *__restrict__ coef) {
    using C = typename CsCplx<T>::type;
    C *sp = reinterpret_cast<C *>(spec);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gc; t += (int64_t)gridDim.x * blockDim.x) {
        const T c = coef[t];
        for (int r = 0; r < nrhs; ++r) {
            C v = sp[(int64_t)r * Gc + t];
            v.x *= c;
            v.y *= c;
            sp[(int64_t)r * Gc + t] = v;
        }
    }
}

// Contract: out = prod(h) sum_nodes K(d)/d (node - x) E~(node)  (overwrites).
// A warp per (particle, block of RB vectors): the node weights are read once per
// block; each vector's sums run in the same order as with one vector per warp.
template <typename T, int RB, int MB = 1>
__global__ void __launch_bounds__(256, MB) k_contract_cs(const T *__restrict__ grid, int64_t n, int nrhs,
                                                     const int32_t *__restrict__ start,
                                                     const double *__restrict__ base, const T *__restrict__ g,
                                                     GridParams gp, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t P3 = (int64_t)P * P * P;
    const int nblk = (nrhs + RB - 1) / RB;
    for (int64_t t = warp; t < n * nblk; t += nw) {
        const int64_t a = gp.order ? (int64_t)gp.order[t % n] : t % n;
        const int r0 = (int)(t / n) * RB;
        const int cnt = min(RB, nrhs - r0);
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const T bx = (T)(base[3 * a] - lo * gp.h[0]), by = (T)(base[3 * a + 1] - lo * gp.h[1]),
                bz = (T)(base[3 * a + 2] - lo * gp.h[2]);
        const T hx = (T)gp.h[0], hy = (T)gp.h[1], hz = (T)gp.h[2];
        const T *ga = g + a * P3;
        const T *gr = grid + (int64_t)r0 * gp.G;
        T ax[RB], ay[RB], az[RB];
#pragma unroll
        for (int q = 0; q < RB; ++q) ax[q] = ay[q] = az[q] = 0;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const T rx = bx + (T)jx * hx, ry = by + (T)jy * hy;
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            T sxy[RB], szz[RB];
#pragma unroll
            for (int q = 0; q < RB; ++q) sxy[q] = szz[q] = 0;
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const T wv = ga[jx + P * (jy + P * jz)];
                const T rz = bz + (T)jz * hz;
                const T *node = gr + rowb + (int64_t)Nx * Ny * iz;
#pragma unroll
                for (int q = 0; q < RB; ++q) {
                    if (q < cnt) {
                        const T v = wv * node[(int64_t)q * gp.G];
                        sxy[q] += v;
                        szz[q] += v * rz;
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < RB; ++q) {
                ax[q] += rx * sxy[q];
                ay[q] += ry * sxy[q];
                az[q] += szz[q];
            }
        }
#pragma unroll
        for (int q = 0; q < RB; ++q) {
            const T sxq = warp_sum(ax[q]), syq = warp_sum(ay[q]), szq = warp_sum(az[q]);
            if (lane == 0 && q < cnt) {
                double *o = out + ((int64_t)(r0 + q) * n + a) * 3;
                o[0] = (double)sxq * gp.hprod;
                o[1] = (double)syq * gp.hprod;
                o[2] = (double)szq * gp.hprod;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
int cs_pair_coefs(const int64_t *row_ptr, const int32_t *nbr, const double *dist, int64_t n, const double *radius,
                  const int32_t *cls, int64_t M, const double *tab, const double *rv, int64_t ntab, double xi,
                  PairData<double> p64, PairData<float> p32, int *err, cudaStream_t s) {
    k_cs_pair_coefs<<<grid_for(n, 128), 128, 0, s>>>(row_ptr, nbr, dist, n, radius, cls, M, tab, rv, ntab, xi, p64.A,
                                                    p64.BA, p32.A, p32.BA, err);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int cs_diag(const double *lam, int64_t n, int64_t nsets, const double *radius, const int32_t *cls, int64_t M,
            const double *tab, int64_t ntab, double xi, double *diag, cudaStream_t s) {
    k_cs_diag<<<grid_for(n * nsets, 256), 256, 0, s>>>(lam, n, nsets, radius, cls, M, tab, ntab, xi, diag);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int cs_geometry(const double *x, int64_t n, const GridParams &gp, const double *radius, double xi, double eta,
                int32_t *start, double *base, double *g64, float *g32, cudaStream_t s) {
    const int64_t P3 = (int64_t)gp.P * gp.P * gp.P;
    k_cs_geom<<<grid_for(n * P3, 256), 256, 0, s>>>(x, n, gp, radius, xi, eta, start, base, g64, g32);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int cs_green(const GridParams &gp, double eta, double xi, double *c64, float *c32, cudaStream_t s) {
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    k_cs_green<<<grid_for(Gc, 256), 256, 0, s>>>(gp, eta, xi, c64, c32);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int spread_cs(const double *m, int64_t n, int nrhs, const int32_t *start, const double *base, const T *g,
              const GridParams &gp, T *grid, cudaStream_t s) {
    MPS_CUDA_TRY(cudaMemsetAsync(grid, 0, sizeof(T) * (size_t)nrhs * gp.G, s));
    if (n == 0) return MPS_OK;
    // 8 vectors per warp pass (the node weights read once per 8 vectors); 4 and 16 measured slower
    const int64_t items = n * ((nrhs + 7) / 8);
    // float: bounds of 4 blocks per SM (72.8 ms over the 16-configuration batch's float32 matvecs against 75.8
    // unbounded); double: unbounded (a 64-register cap spills it)
    constexpr int MB = sizeof(T) == 4 ? 4 : 1;
    k_spread_cs<T, 8, MB><<<grid_for(items * 32, 256, 152 * 64), 256, 0, s>>>(m, n, nrhs, start, base, g, gp, grid);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int scale_cs(void *spec, int nrhs, const GridParams &gp, const T *coef, cudaStream_t s) {
    const int64_t Gc = (int64_t)(gp.N[0] / 2 + 1) * gp.N[1] * gp.N[2];
    k_scale_cs<T><<<grid_for(Gc, 256), 256, 0, s>>>((T *)spec, nrhs, Gc, coef);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <typename T>
int contract_cs(const T *grid, int64_t n, int nrhs, const int32_t *start, const double *base, const T *g,
                const GridParams &gp, double *out, cudaStream_t s) {
    if (n == 0) return MPS_OK;
    // 4 vectors per warp pass (5 x 4 accumulators per lane): 99 ms against 104 for 8 over the 16-configuration
    // batch's float32 matvecs; 16 spills
    const int64_t items = n * ((nrhs + 3) / 4);
    // float: bounds of 3 blocks per SM (76 registers: 83 ms over the batch's float32 matvecs against 99 at 64)
    constexpr int MB = sizeof(T) == 4 ? 3 : 1;
    k_contract_cs<T, 4, MB><<<grid_for(items * 32, 256, 152 * 64), 256, 0, s>>>(grid, n, nrhs, start, base, g, gp, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template int spread_cs<float>(const double *, int64_t, int, const int32_t *, const double *, const float *,
                              const GridParams &, float *, cudaStream_t);
template int spread_cs<double>(const double *, int64_t, int, const int32_t *, const double *, const double *,
                               const GridParams &, double *, cudaStream_t);
template int scale_cs<float>(void *, int, const GridParams &, const float *, cudaStream_t);
template int scale_cs<double>(void *, int, const GridParams &, const double *, cudaStream_t);
template int contract_cs<float>(const float *, int64_t, int, const int32_t *, const double *, const float *,
                                const GridParams &, double *, cudaStream_t);
template int contract_cs<double>(const double *, int64_t, int, const int32_t *, const double *, const double *,
                                 const GridParams &, double *, cudaStream_t);

}  // namespace mps

using namespace mps;

extern "C" int mps_sizes_table(const double *r, int64_t n, const double *a_uniq, int64_t M, double xi, double *perp,
                               double *para, mps_stream_t stream) {
    if (n < 1 || M < 1 || !r || !a_uniq || !perp || !para || !(xi > 0)) return MPS_BAD_ARG;
    const int64_t m = M * (M + 1) / 2;
    k_cs_table<<<grid_for(n * m, 256), 256, 0, (cudaStream_t)stream>>>(r, n, a_uniq, M, xi, perp, para);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}
