// Real-space part: closed-form coupling tables (EW/ewald.py:604-931) and the
// pair sums (EW/ewald.py:1019-1072).
#include <math.h>

#include "realspace.cuh"

namespace mps {

// ---------------------------------------------------------------------------
// Tables.  Each table is
//   cE r^-pE [E+(r) e^{-xi^2 (r+2)^2} + E-(r) e^{-xi^2 (r-2)^2} + E0(r) e^{-xi^2 r^2}]
// + cF r^-pF [F+(r) erfc(xi (r+2)) + F-(r) erfc(xi (r-2)) + F0(r) erfc(xi r)]
// + [r < 2] reg(r)
// with polynomial coefficient sets (highest power first) built on the host.
// ---------------------------------------------------------------------------
struct TableSpec {
    double cE, cF;
    int pE, pF;
    int nE, nF;          // coefficients per polynomial
    double E[3][6];      // +, -, 0
    double F[3][7];
};

struct TableSet {
    TableSpec t[6];
};

static void build_specs(double xi, TableSet &S) {
    const double x2 = xi * xi, x4 = x2 * x2, x6 = x4 * x2;
    const double sp3 = pow(MPS_PI, 1.5);
    const double q = 3.0 - 12.0 * x2 + 32.0 * x4;
    const double s = 2.0 * (3.0 + 4.0 * x2 - 32.0 * x4);
    auto set = [](TableSpec &T, double cE, int pE, std::initializer_list<double> ep, std::initializer_list<double> em,
                  std::initializer_list<double> e0, double cF, int pF, std::initializer_list<double> fp,
                  std::initializer_list<double> fm, std::initializer_list<double> f0) {
        T.cE = cE;
        T.pE = pE;
        T.cF = cF;
        T.pF = pF;
        T.nE = (int)ep.size();
        T.nF = (int)fp.size();
        int i = 0;
        for (double v : ep) T.E[0][i++] = v;
        i = 0;
        for (double v : em) T.E[1][i++] = v;
        i = 0;
        for (double v : e0) T.E[2][i++] = v;
        i = 0;
        for (double v : fp) T.F[0][i++] = v;
        i = 0;
        for (double v : fm) T.F[1][i++] = v;
        i = 0;
        for (double v : f0) T.F[2][i++] = v;
    };
    // potential / charge
    set(S.t[0], 1.0 / (32.0 * sp3 * xi), 1, {-1.0, -2.0}, {-1.0, 2.0}, {2.0, 0.0}, 1.0 / (64.0 * MPS_PI * x2), 1,
        {2 * x2, 8 * x2, 8 * x2 + 1.0}, {2 * x2, -8 * x2, 8 * x2 + 1.0}, {-4 * x2, 0.0, -2.0});
    // potential / dipole
    set(S.t[1], 1.0 / (256.0 * sp3 * xi * x2), 2, {-6 * x2, -4 * x2, 8 * x2 - 3.0, 2.0 - 16 * x2},
        {-6 * x2, 4 * x2, 8 * x2 - 3.0, 16 * x2 - 2.0}, {12 * x2, 0.0, 6.0, 0.0}, 1.0 / (512.0 * MPS_PI * x4), 2,
        {12 * x4, 32 * x4, 12 * x2, 0.0, 64 * x4 - 3.0}, {12 * x4, -32 * x4, 12 * x2, 0.0, 64 * x4 - 3.0},
        {-24 * x4, 0.0, -24 * x2, 0.0, 6.0});
    // field / dipole (I - rr)
    set(S.t[2], 1.0 / (1024.0 * sp3 * xi * x4), 3,
        {4 * x4, -8 * x4, 8 * x2 * (2 - 7 * x2), -8 * x2 * (3 + 2 * x2), q, s},
        {4 * x4, 8 * x4, 8 * x2 * (2 - 7 * x2), 8 * x2 * (3 + 2 * x2), q, -s},
        {-8 * x4, 0.0, -16 * x2 * (2 - 9 * x2), 0.0, 2 * (36 * x2 - 3), 0.0}, 1.0 / (2048.0 * MPS_PI * x6), 3,
        {-8 * x6, 0.0, -36 * x4 * (1 - 4 * x2), 256 * x6, -18 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6},
        {-8 * x6, 0.0, -36 * x4 * (1 - 4 * x2), -256 * x6, -18 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6},
        {16 * x6, 0.0, 72 * x4 * (1 - 4 * x2), 0.0, 36 * x2 * (1 - 8 * x2), 0.0, 2 * (36 * x2 - 3)});
    // field / dipole (rr)
    set(S.t[3], 1.0 / (512.0 * sp3 * xi * x4), 3,
        {8 * x4, -16 * x4, 2 * x2 * (7 - 20 * x2), -4 * x2 * (3 - 4 * x2), -q, -s},
        {8 * x4, 16 * x4, 2 * x2 * (7 - 20 * x2), 4 * x2 * (3 - 4 * x2), -q, s},
        {-16 * x4, 0.0, -4 * x2 * (7 - 36 * x2), 0.0, 2 * (3 - 36 * x2), 0.0}, 1.0 / (1024.0 * MPS_PI * x6), 3,
        {-16 * x6, 0.0, -36 * x4 * (1 - 4 * x2), 128 * x6, 0.0, 0.0, -3 + 36 * x2 - 256 * x6},
        {-16 * x6, 0.0, -36 * x4 * (1 - 4 * x2), -128 * x6, 0.0, 0.0, -3 + 36 * x2 - 256 * x6},
        {32 * x6, 0.0, 72 * x4 * (1 - 4 * x2), 0.0, 0.0, 0.0, 2 * (3 - 36 * x2)});
    // force 1
    set(S.t[4], 3.0 / (1024.0 * sp3 * xi * x4), 4, {4 * x4, -8 * x4, 4 * x2 * (1 - 2 * x2), 16 * x4, -q, -s},
        {4 * x4, 8 * x4, 4 * x2 * (1 - 2 * x2), -16 * x4, -q, s},
        {-8 * x4, 0.0, -8 * x2 * (1 - 6 * x2), 0.0, 2 * (3 - 36 * x2), 0.0}, 3.0 / (2048.0 * MPS_PI * x6), 4,
        {-8 * x6, 0.0, -12 * x4 * (1 - 4 * x2), 0.0, 6 * x2 * (1 - 8 * x2), 0.0, -3 + 36 * x2 - 256 * x6},
        {-8 * x6, 0.0, -12 * x4 * (1 - 4 * x2), 0.0, 6 * x2 * (1 - 8 * x2), 0.0, -3 + 36 * x2 - 256 * x6},
        {16 * x6, 0.0, 24 * x4 * (1 - 4 * x2), 0.0, -12 * x2 * (1 - 8 * x2), 0.0, 2 * (3 - 36 * x2)});
    // force 2
    set(S.t[5], 9.0 / (1024.0 * sp3 * xi * x4), 4, {4 * x4, -8 * x4, 8 * x4, 8 * x2 * (1 - 2 * x2), q, s},
        {4 * x4, 8 * x4, 8 * x4, -8 * x2 * (1 - 2 * x2), q, -s},
        {-8 * x4, 0.0, 16 * x4, 0.0, 2 * (36 * x2 - 3), 0.0}, 9.0 / (2048.0 * MPS_PI * x6), 4,
        {-8 * x6, 0.0, -4 * x4 * (1 - 4 * x2), 0.0, -2 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6},
        {-8 * x6, 0.0, -4 * x4 * (1 - 4 * x2), 0.0, -2 * x2 * (1 - 8 * x2), 0.0, 3 - 36 * x2 + 256 * x6},
        {16 * x6, 0.0, 8 * x4 * (1 - 4 * x2), 0.0, 4 * x2 * (1 - 8 * x2), 0.0, 2 * (36 * x2 - 3)});
}

__device__ __forceinline__ double horner(const double *c, int nc, double r) {
    double v = c[0];
    for (int i = 1; i < nc; ++i) v = v * r + c[i];
    return v;
}

__device__ double overlap_poly(int t, double r) {
    const double pi = MPS_PI;
    switch (t) {
        case 0: return -1.0 / (4.0 * pi * r) + (4.0 - r) / (16.0 * pi);
        case 1: return -1.0 / (4.0 * pi * r * r) + r / (8.0 * pi) * (1.0 - 3.0 / 8.0 * r);
        case 2: return -1.0 / (4.0 * pi * r * r * r) + (1.0 - 9.0 * r / 16.0 + r * r * r / 32.0) / (4.0 * pi);
        case 3: return 1.0 / (2.0 * pi * r * r * r) + (1.0 - 9.0 * r / 8.0 + r * r * r / 8.0) / (4.0 * pi);
        case 4: return 3.0 / (4.0 * pi * r * r * r * r) - 3.0 / (64.0 * pi) * (3.0 - r * r / 2.0);
        default: return -9.0 / (4.0 * pi * r * r * r * r) - 9.0 / (64.0 * pi) * (1.0 - r * r / 2.0);
    }
}

// overlap: bit t set = row t carries the r < 2 overlap polynomial (all six in the solver's tables;
// Compute_Field/RealSpaceTable.m drops it from field_dip_1 and field_dip_2).
__global__ void k_tables(const double *__restrict__ r, int64_t n, double xi, TableSet S, double self_pc,
                         double self_fd, int overlap, double *__restrict__ out) {
    const int64_t row = n + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0) {
            out[0 * row] = self_pc;
            out[1 * row] = 0.0;
            out[2 * row] = self_fd;
            out[3 * row] = self_fd;
            out[4 * row] = 0.0;
            out[5 * row] = 0.0;
            continue;
        }
        const double rv = r[i - 1];
        const double ep = exp(-(rv + 2.0) * (rv + 2.0) * xi * xi);
        const double em = exp(-(rv - 2.0) * (rv - 2.0) * xi * xi);
        const double e0 = exp(-rv * rv * xi * xi);
        const double fp = erfc((rv + 2.0) * xi);
        const double fm = erfc((rv - 2.0) * xi);
        const double f0 = erfc(rv * xi);
        for (int t = 0; t < 6; ++t) {
            const TableSpec &T = S.t[t];
            double v = T.cE / pow(rv, (double)T.pE) *
                       (horner(T.E[0], T.nE, rv) * ep + horner(T.E[1], T.nE, rv) * em + horner(T.E[2], T.nE, rv) * e0);
            v += T.cF / pow(rv, (double)T.pF) *
                 (horner(T.F[0], T.nF, rv) * fp + horner(T.F[1], T.nF, rv) * fm + horner(T.F[2], T.nF, rv) * f0);
            if (rv < 2.0 && ((overlap >> t) & 1)) v += overlap_poly(t, rv);
            out[t * row + i] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// Pair-list form (drop-in real_space_fast): diagonal, then scatter with atomics.
// ---------------------------------------------------------------------------
__global__ void k_rs_diag(const double *__restrict__ m, int64_t n, int64_t nvec, const double *__restrict__ lam,
                          double self_perp, double *__restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nvec * n * 3; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = (t / 3) % n;
        double d = -3.0 / (4.0 * MPS_PI * (1.0 - lam[a]));
        out[t] = d * m[t] + m[t] * self_perp;
    }
}

__global__ void k_rs_pairs(const double *__restrict__ m, int64_t n, int64_t nvec, const int64_t *__restrict__ p1,
                           const int64_t *__restrict__ p2, const double *__restrict__ rhat,
                           const double *__restrict__ A, const double *__restrict__ B, int64_t np,
                           double *__restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = p1[k], b = p2[k];
        const double rx = rhat[3 * k], ry = rhat[3 * k + 1], rz = rhat[3 * k + 2];
        const double av = A[k], ba = B[k] - A[k];
        for (int64_t v = 0; v < nvec; ++v) {
            const double *mb = m + (v * n + b) * 3;
            double proj = mb[0] * rx + mb[1] * ry + mb[2] * rz;
            double s = ba * proj;
            double *o = out + (v * n + a) * 3;
            atomicAdd(o + 0, av * mb[0] + s * rx);
            atomicAdd(o + 1, av * mb[1] + s * ry);
            atomicAdd(o + 2, av * mb[2] + s * rz);
        }
    }
}

// ---------------------------------------------------------------------------
// CSR form used by the system matvec.  A group of G lanes owns one particle;
// pair data are read once and applied to every vector of the batch.
//   out[r][a] = beta*out[r][a] + diag[r][a] m[r][a] + sum_b [A m_b + (B-A)(m_b.rhat) rhat] + slab[r] z
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T group_xor(T v, int o, int G) {
    return __shfl_xor_sync(0xffffffffu, v, o, G);
}
template <>
__device__ __forceinline__ dfv group_xor<dfv>(dfv v, int o, int G) {
    return dfv(__shfl_xor_sync(0xffffffffu, v.hi, o, G), __shfl_xor_sync(0xffffffffu, v.lo, o, G));
}

// T: pair arithmetic (float, double or double-float dfv); mT: the moments read
// by the pair loop in type TM (float64 m itself, or its float / double-float copy).
// order: optional row visiting order (null = row index).
template <typename T, int G, int R, typename TM = double>
__global__ void __launch_bounds__(256) k_rs_csr(const double *__restrict__ m, double *__restrict__ out, int64_t n,
                                                int nrhs, int r0, const int64_t *__restrict__ row_ptr,
                                                PairData<T> pd, const double *__restrict__ diag,
                                                const int32_t *__restrict__ diag_of_rhs,
                                                const double *__restrict__ slab, int accumulate,
                                                const TM *__restrict__ mT, const int32_t *__restrict__ order) {
    const int lane = threadIdx.x % G;
    const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
    r0 += (int)blockIdx.y * R;   // several blocks of R vectors in one launch (grid y)
    const int nr = min(R, nrhs - r0);
    for (int64_t i = grp; i < n; i += ngrp) {
        // rows in `order` (cell order): neighbouring groups read overlapping neighbour moments
        const int64_t a = order ? (int64_t)order[i] : i;
        T acc[R][3];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r][0] = acc[r][1] = acc[r][2] = (T)0;
        const int64_t e0 = row_ptr[a], e1 = row_ptr[a + 1];
        // two entries per lane in flight: the loop waits on its neighbour gathers (same order of the sums)
#pragma unroll 2
        for (int64_t e = e0 + lane; e < e1; e += G) {
            const int32_t b = pd.nbr[e];
            const T av = pd.A[e], ba = pd.BA[e];
            const T rx = pd.rx[e], ry = pd.ry[e], rz = pd.rz[e];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r < nr) {
                    const TM *mb = mT + ((int64_t)(r0 + r) * n + b) * 3;
                    const T mx = (T)mb[0], my = (T)mb[1], mz = (T)mb[2];
                    const T s = ba * (mx * rx + my * ry + mz * rz);
                    acc[r][0] += av * mx + s * rx;
                    acc[r][1] += av * my + s * ry;
                    acc[r][2] += av * mz + s * rz;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) acc[r][c] += group_xor(acc[r][c], o, G);
        if (lane == 0) {
            for (int r = 0; r < nr; ++r) {
                const int rr = r0 + r;
                const double dg = diag[(int64_t)(diag_of_rhs ? diag_of_rhs[rr] : 0) * n + a];
                const double *ma = m + ((int64_t)rr * n + a) * 3;
                double *o = out + ((int64_t)rr * n + a) * 3;
                double v0 = dg * ma[0] + (double)acc[r][0];
                double v1 = dg * ma[1] + (double)acc[r][1];
                double v2 = dg * ma[2] + (double)acc[r][2] + slab[rr];
                if (accumulate) {
                    v0 += o[0];
                    v1 += o[1];
                    v2 += o[2];
                }
                o[0] = v0;
                o[1] = v1;
                o[2] = v2;
            }
        }
    }
}

template <typename T>
int real_space_csr(const double *m, double *out, int64_t n, int nrhs, const int64_t *row_ptr, PairData<T> pd,
                   const double *diag, const int32_t *diag_of_rhs, const double *slab, bool accumulate,
                   cudaStream_t s) {
    constexpr int G = 8;
    const int block = 256;
    unsigned grid = grid_for(n * G, block, 152 * 64);
    for (int r0 = 0; r0 < nrhs; r0 += 4) {
        int nr = nrhs - r0;
        if (nr >= 4) {
            const int nb = nr / 4;   // every full block of 4 vectors in one launch (grid y)
            k_rs_csr<T, G, 4><<<dim3(grid, nb), block, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs,
                                                               slab, accumulate, m, nullptr);
            r0 += 4 * (nb - 1);
        }
        else if (nr == 3)
            k_rs_csr<T, G, 3><<<grid, block, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab, accumulate, m, nullptr);
        else if (nr == 2)
            k_rs_csr<T, G, 2><<<grid, block, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab, accumulate, m, nullptr);
        else
            k_rs_csr<T, G, 1><<<grid, block, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab, accumulate, m, nullptr);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

template int real_space_csr<double>(const double *, double *, int64_t, int, const int64_t *, PairData<double>,
                                    const double *, const int32_t *, const double *, bool, cudaStream_t);
template int real_space_csr<float>(const double *, double *, int64_t, int, const int64_t *, PairData<float>,
                                   const double *, const int32_t *, const double *, bool, cudaStream_t);

__global__ void k_to_dfv(const double *__restrict__ m, int64_t total, dfv *__restrict__ md) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        md[i] = dfv(m[i]);
}

int real_space_csr_df(const double *m, dfv *mdf, double *out, int64_t n, int nrhs, const int64_t *row_ptr,
                      PairData<dfv> pd, const double *diag, const int32_t *diag_of_rhs, const double *slab,
                      bool accumulate, const int32_t *order, cudaStream_t s) {
    k_to_dfv<<<grid_for((int64_t)nrhs * n * 3, 256), 256, 0, s>>>(m, (int64_t)nrhs * n * 3, mdf);
    MPS_LAUNCH_CHECK();
    constexpr int G = 8;
    const unsigned grid = grid_for(n * G, 256, 152 * 64);
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = nrhs - r0;
        if (nr >= 3)
            k_rs_csr<dfv, G, 3, dfv><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                          accumulate, mdf, order);
        else if (nr == 2)
            k_rs_csr<dfv, G, 2, dfv><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                          accumulate, mdf, order);
        else
            k_rs_csr<dfv, G, 1, dfv><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                          accumulate, mdf, order);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

// Float copy of the moments with each particle's nrhs x 3 components side by side (stride S floats, a multiple of
// 4): the pair loop gathers a neighbour's block of vectors with 16-byte loads from one place instead of one
// 4-byte load per vector and component from nrhs planes.
__global__ void k_to_f32_rows(const double *__restrict__ m, int64_t n, int nrhs, int S, float *__restrict__ mf) {
    const int64_t total = (int64_t)nrhs * n * 3;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / (n * 3), rem = t - r * n * 3;
        const int64_t a = rem / 3;
        const int c = (int)(rem - a * 3);
        mf[a * S + r * 3 + c] = (float)m[t];
    }
}

size_t m32_floats(int64_t n, int nrhs) { return (size_t)n * (size_t)((3 * nrhs + 3) & ~3); }

// The float32 pair sum of k_rs_csr (same sums, same order) on the row copy of k_to_f32_rows: a neighbour's R
// vectors are ceil(3R / 4) float4 loads at a 16-byte aligned offset (r0 is a multiple of 4 and S of 4, so
// 3 r0 + 4 ceil(3R / 4) <= S: a read past the block's last component stays inside the particle's row).
template <int G, int R>
__global__ void __launch_bounds__(256) k_rs_csr_f32(const double *__restrict__ m, double *__restrict__ out, int64_t n,
                                                    int nrhs, int r0, const int64_t *__restrict__ row_ptr,
                                                    PairData<float> pd, const double *__restrict__ diag,
                                                    const int32_t *__restrict__ diag_of_rhs,
                                                    const double *__restrict__ slab, int accumulate,
                                                    const float *__restrict__ mf, int S,
                                                    const int32_t *__restrict__ order) {
    constexpr int NQ = (3 * R + 3) / 4;   // float4 loads per neighbour
    const int lane = threadIdx.x % G;
    const int64_t grp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ngrp = ((int64_t)gridDim.x * blockDim.x) / G;
    r0 += (int)blockIdx.y * R;
    const int nr = min(R, nrhs - r0);
    const float *mb0 = mf + 3 * r0;
    for (int64_t i = grp; i < n; i += ngrp) {
        const int64_t a = order ? (int64_t)order[i] : i;
        float acc[R][3];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.f;
        const int64_t e0 = row_ptr[a], e1 = row_ptr[a + 1];
#pragma unroll 2
        for (int64_t e = e0 + lane; e < e1; e += G) {
            const int32_t b = pd.nbr[e];
            const float av = pd.A[e], ba = pd.BA[e];
            const float rx = pd.rx[e], ry = pd.ry[e], rz = pd.rz[e];
            const float4 *q = reinterpret_cast<const float4 *>(mb0 + (int64_t)b * S);
            float v[4 * NQ];
#pragma unroll
            for (int k = 0; k < NQ; ++k) {
                const float4 t = __ldg(q + k);
                v[4 * k] = t.x;
                v[4 * k + 1] = t.y;
                v[4 * k + 2] = t.z;
                v[4 * k + 3] = t.w;
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r < nr) {
                    const float mx = v[3 * r], my = v[3 * r + 1], mz = v[3 * r + 2];
                    const float s = ba * (mx * rx + my * ry + mz * rz);
                    acc[r][0] += av * mx + s * rx;
                    acc[r][1] += av * my + s * ry;
                    acc[r][2] += av * mz + s * rz;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) acc[r][c] += __shfl_xor_sync(0xffffffffu, acc[r][c], o, G);
        if (lane == 0) {
            for (int r = 0; r < nr; ++r) {
                const int rr = r0 + r;
                const double dg = diag[(int64_t)(diag_of_rhs ? diag_of_rhs[rr] : 0) * n + a];
                const double *ma = m + ((int64_t)rr * n + a) * 3;
                double *o = out + ((int64_t)rr * n + a) * 3;
                double v0 = dg * ma[0] + (double)acc[r][0];
                double v1 = dg * ma[1] + (double)acc[r][1];
                double v2 = dg * ma[2] + (double)acc[r][2] + slab[rr];
                if (accumulate) {
                    v0 += o[0];
                    v1 += o[1];
                    v2 += o[2];
                }
                o[0] = v0;
                o[1] = v1;
                o[2] = v2;
            }
        }
    }
}

// Float32 pair sum on a float copy of the moments (converted once per matvec, not
// once per pair: float64 -> float32 conversions run on GB300's narrow float64
// pipe), rows in `order`, up to 8 right-hand sides per pass over the pair data.
template <int G>
static int rs_f32_launches(const double *m, float *m32, double *out, int64_t n, int nrhs, int S,
                           const int64_t *row_ptr, PairData<float> pd, const double *diag, const int32_t *diag_of_rhs,
                           const double *slab, bool accumulate, const int32_t *order, cudaStream_t s) {
    const unsigned grid = grid_for(n * G, 256, 152 * 64);
    // blocks of 8 vectors, then one of 4, then the last 3, 2 or 1: every block starts at a multiple of 4
    for (int r0 = 0; r0 < nrhs;) {
        const int nr = nrhs - r0;
        if (nr >= 8) {
            // every full block of 8 vectors in one launch (grid y): small systems fill the GPU with all of them
            const int nb = nr / 8;
            k_rs_csr_f32<G, 8><<<dim3(grid, nb), 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs,
                                                              slab, accumulate, m32, S, order);
            r0 += 8 * nb;
        } else if (nr >= 4) {
            k_rs_csr_f32<G, 4><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                    accumulate, m32, S, order);
            r0 += 4;
        } else if (nr == 3) {
            k_rs_csr_f32<G, 3><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                    accumulate, m32, S, order);
            r0 += 3;
        } else if (nr == 2) {
            k_rs_csr_f32<G, 2><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                    accumulate, m32, S, order);
            r0 += 2;
        } else {
            k_rs_csr_f32<G, 1><<<grid, 256, 0, s>>>(m, out, n, nrhs, r0, row_ptr, pd, diag, diag_of_rhs, slab,
                                                    accumulate, m32, S, order);
            r0 += 1;
        }
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

// Float32 pair sum on a float copy of the moments (converted once per matvec, not
// once per pair: float64 -> float32 conversions run on GB300's narrow float64
// pipe), rows in `order`, up to 8 right-hand sides per pass over the pair data.
int real_space_csr_f32(const double *m, float *m32, double *out, int64_t n, int nrhs, const int64_t *row_ptr,
                       PairData<float> pd, const double *diag, const int32_t *diag_of_rhs, const double *slab,
                       bool accumulate, const int32_t *order, cudaStream_t s) {
    const int S = (3 * nrhs + 3) & ~3;
    k_to_f32_rows<<<grid_for((int64_t)nrhs * n * 3, 256), 256, 0, s>>>(m, n, nrhs, S, m32);
    MPS_LAUNCH_CHECK();
    // 4 lanes per particle: the polydisperse batch (48 vectors, configurations of 500..20,000 spheres) took 7.14 s
    // against 7.27 s with 8 lanes, the headline step 18.74 against 18.75 ms; 16 lanes took 19.08 ms
    return rs_f32_launches<4>(m, m32, out, n, nrhs, S, row_ptr, pd, diag, diag_of_rhs, slab, accumulate, order, s);
}

// Diagonal (dielectric + self) per particle and permittivity set.
__global__ void k_diag(const double *__restrict__ lam, int64_t total, double self_perp, double *__restrict__ diag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        diag[i] = -3.0 / (4.0 * MPS_PI * (1.0 - lam[i])) + self_perp;
}

int build_diag(const double *lam, int64_t total, const double *perp, double *diag, cudaStream_t s) {
    double self_perp = 0.0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&self_perp, perp, sizeof(double), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_TRY(cudaStreamSynchronize(s));
    k_diag<<<grid_for(total, 256), 256, 0, s>>>(lam, total, self_perp, diag);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

// Complex permittivity eps = a + i b: D = -3 / (4 pi (1 - eps)) + self_perp, split
// into its real and imaginary parts (EW/ewald.py:1058 with complex lambda, as the
// MATLAB spectrum drivers allow).
__global__ void k_diag_cplx(const double *__restrict__ lr, const double *__restrict__ li, int64_t total,
                            double self_perp, double *__restrict__ dr, double *__restrict__ di) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const double u = 1.0 - lr[i], v = -li[i];   // 1 - eps = u + i v
        const double q = u * u + v * v;
        dr[i] = -3.0 * u / (4.0 * MPS_PI * q) + self_perp;
        di[i] = 3.0 * v / (4.0 * MPS_PI * q);
    }
}

int build_diag_complex(const double *lr, const double *li, int64_t total, const double *perp, double *dr, double *di,
                       cudaStream_t s) {
    double self_perp = 0.0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&self_perp, perp, sizeof(double), cudaMemcpyDeviceToHost, s));
    MPS_CUDA_TRY(cudaStreamSynchronize(s));
    k_diag_cplx<<<grid_for(total, 256), 256, 0, s>>>(lr, li, total, self_perp, dr, di);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

// Slab term per vector: slab_factor * sum_a m_z(a) / V (deterministic two-stage sum).
__global__ void k_slab(const double *__restrict__ m, int64_t n, double scale, double *__restrict__ slab) {
    __shared__ double sm[32];
    const int r = blockIdx.x;
    double acc = 0.0;
    for (int64_t a = threadIdx.x; a < n; a += blockDim.x) acc += m[((int64_t)r * n + a) * 3 + 2];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) slab[r] = scale * v;
    }
}

int slab_terms(const double *m, int64_t n, int nrhs, double scale, double *slab, cudaStream_t s) {
    k_slab<<<nrhs, 1024, 0, s>>>(m, n, scale, slab);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

void table_self_terms(double xi, double *s_pc, double *s_fd) {
    double e4 = exp(-4.0 * xi * xi);
    double ec = erfc(2.0 * xi);
    *s_pc = (1.0 - e4) / (8.0 * pow(MPS_PI, 1.5) * xi) + ec / (4.0 * MPS_PI);
    *s_fd = (-1.0 + 6.0 * xi * xi + (1.0 - 2.0 * xi * xi) * e4) / (16.0 * pow(MPS_PI, 1.5) * xi * xi * xi) +
            ec / (4.0 * MPS_PI);
}

}  // namespace mps

using namespace mps;

extern "C" int mps_real_space_table(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream) {
    if (n < 0 || !(xi > 0) || !tables || (n > 0 && !r)) return MPS_BAD_ARG;
    TableSet S;
    build_specs(xi, S);
    double spc, sfd;
    table_self_terms(xi, &spc, &sfd);
    cudaStream_t s = (cudaStream_t)stream;
    k_tables<<<grid_for(n + 1, 128), 128, 0, s>>>(r, n, xi, S, spc, sfd, 0x3f, tables);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_real_space_table_probe(const double *r, int64_t n, double xi, double *tables,
                                          mps_stream_t stream) {
    if (n < 0 || !(xi > 0) || !tables || (n > 0 && !r)) return MPS_BAD_ARG;
    TableSet S;
    build_specs(xi, S);
    double spc, sfd;
    table_self_terms(xi, &spc, &sfd);
    cudaStream_t s = (cudaStream_t)stream;
    k_tables<<<grid_for(n + 1, 128), 128, 0, s>>>(r, n, xi, S, spc, sfd, 0x33, tables);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_real_space_fast(const double *m, int64_t n, int64_t nvec, const double *lambdap, const int64_t *p1,
                                   const int64_t *p2, const double *rhat, const double *A, const double *B,
                                   int64_t n_pairs, double self_perp, double *out, mps_stream_t stream) {
    if (n < 0 || nvec < 1 || n_pairs < 0) return MPS_BAD_ARG;
    if (n == 0) return MPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    k_rs_diag<<<grid_for(nvec * n * 3, 256), 256, 0, s>>>(m, n, nvec, lambdap, self_perp, out);
    MPS_LAUNCH_CHECK();
    if (n_pairs > 0) {
        k_rs_pairs<<<grid_for(n_pairs, 256), 256, 0, s>>>(m, n, nvec, p1, p2, rhat, A, B, n_pairs, out);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}
