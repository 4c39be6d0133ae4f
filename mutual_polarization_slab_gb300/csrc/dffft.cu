// Double-float 3-D real FFT pipeline (see dffft.cuh).
//
// Arithmetic: a value is hi + lo (two floats).  Sums use the two-sum error-free
// transformation, products the FMA-based two-product; every step is written
// with __fadd_rn/__fmul_rn/__fmaf_rn so the compiler cannot contract or reorder
// it.  A complex value is a float4 (re.hi, re.lo, im.hi, im.lo).
//
// Transforms: one warp owns one 1-D line in shared memory and runs a
// mixed-radix (4, 3, 5, 2) Stockham FFT on it (stage s reads in[j + r N/R],
// multiplies by the twiddle w^(r (j mod Ns)) of the Ns R-point DFT and writes
// out[(j / Ns) Ns R + j mod Ns + r Ns]; the output is in natural order).
// Inverse transforms use conj(FFT(conj(x))).
//   x pass   two real rows y, y+1 form one complex line; the half spectra are
//            separated with X0[k] = (Z[k] + conj Z[N-k]) / 2,
//            X1[k] = -i (Z[k] - conj Z[N-k]) / 2 (and the reverse on the way back)
//   y pass   tiles of 8 consecutive kx columns, coalesced along kx
//   z pass   forward FFT, the dipole Green's scale H k k^T (float64 coefficient,
//            Nyquist rule of the float64 path) and the inverse FFT in one kernel,
//            for the three components of one vector together
#include <math.h>

#include <map>
#include <mutex>
#include <vector>

#include "dffft.cuh"

namespace mps {

#define MPS_TRY_STATUS(expr)          \
    do {                              \
        int _r = (expr);              \
        if (_r != MPS_OK) return _r;  \
    } while (0)

struct dfr {
    float hi, lo;
};
struct dfc {
    dfr re, im;
};

__device__ __forceinline__ dfr fts(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfr dadd(dfr a, dfr b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return fts(s, e);
}
__device__ __forceinline__ dfr dneg(dfr a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfr dsub(dfr a, dfr b) { return dadd(a, dneg(b)); }
__device__ __forceinline__ dfr dmul(dfr a, dfr b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fts(p, e);
}
__device__ __forceinline__ dfr dhalf(dfr a) { return {__fmul_rn(a.hi, 0.5f), __fmul_rn(a.lo, 0.5f)}; }
__device__ __forceinline__ dfr dfrom(double v) {
    const float h = __double2float_rn(v);
    return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double dto(dfr a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dfc cadd(dfc a, dfc b) { return {dadd(a.re, b.re), dadd(a.im, b.im)}; }
__device__ __forceinline__ dfc csub(dfc a, dfc b) { return {dsub(a.re, b.re), dsub(a.im, b.im)}; }
__device__ __forceinline__ dfc cmul(dfc a, dfc w) {
    return {dsub(dmul(a.re, w.re), dmul(a.im, w.im)), dadd(dmul(a.re, w.im), dmul(a.im, w.re))};
}
__device__ __forceinline__ dfc cscale(dfc a, dfr c) { return {dmul(a.re, c), dmul(a.im, c)}; }
__device__ __forceinline__ dfc chalf(dfc a) { return {dhalf(a.re), dhalf(a.im)}; }
__device__ __forceinline__ dfc mul_i(dfc a) { return {dneg(a.im), a.re}; }
__device__ __forceinline__ dfc mul_mi(dfc a) { return {a.im, dneg(a.re)}; }
__device__ __forceinline__ dfc cconj(dfc a) { return {a.re, dneg(a.im)}; }
__device__ __forceinline__ dfc ld4(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ float4 st4(dfc a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ dfc czero() { return {{0.f, 0.f}, {0.f, 0.f}}; }

// Small DFTs, forward sign (w = exp(-2 pi i / R)).
template <int R>
__device__ __forceinline__ void dft(dfc *v);

template <>
__device__ __forceinline__ void dft<2>(dfc *v) {
    const dfc a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<3>(dfc *v) {
    const dfr s3 = dfrom(0.86602540378443864676372317075294);
    const dfc a = cadd(v[1], v[2]), b = csub(v[1], v[2]);
    const dfc m = csub(v[0], chalf(a));
    const dfc tb = cscale(b, s3);
    v[0] = cadd(v[0], a);
    v[1] = cadd(m, mul_mi(tb));
    v[2] = cadd(m, mul_i(tb));
}

template <>
__device__ __forceinline__ void dft<4>(dfc *v) {
    const dfc a = cadd(v[0], v[2]), b = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, mul_mi(d));
    v[3] = cadd(b, mul_i(d));
}

template <>
__device__ __forceinline__ void dft<5>(dfc *v) {
    const dfr c1 = dfrom(0.30901699437494742410229341718282), c2 = dfrom(-0.80901699437494742410229341718282);
    const dfr s1 = dfrom(0.95105651629515357211643933337938), s2 = dfrom(0.58778525229247312916870595463907);
    const dfc a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]), a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    const dfc m1 = cadd(v[0], cadd(cscale(a1, c1), cscale(a2, c2)));
    const dfc m2 = cadd(v[0], cadd(cscale(a1, c2), cscale(a2, c1)));
    const dfc t1 = cadd(cscale(b1, s1), cscale(b2, s2));
    const dfc t2 = csub(cscale(b1, s2), cscale(b2, s1));
    v[0] = cadd(v[0], cadd(a1, a2));
    v[1] = cadd(m1, mul_mi(t1));
    v[2] = cadd(m2, mul_mi(t2));
    v[3] = cadd(m2, mul_i(t2));
    v[4] = cadd(m1, mul_i(t1));
}

template <int R>
__device__ __forceinline__ void df_stage(const float4 *__restrict__ in, float4 *__restrict__ out, int N, int Ns,
                                         const float4 *__restrict__ tw, int lane, int nl) {
    const int NR = N / R;
    for (int j = lane; j < NR; j += nl) {
        const int jm = j % Ns;
        dfc v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[r] = ld4(in[j + r * NR]);
            if (r > 0 && jm > 0) v[r] = cmul(v[r], ld4(tw[jm * R + r]));
        }
        dft<R>(v);
        const int d = (j / Ns) * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; ++r) out[d + r * Ns] = st4(v[r]);
    }
}

// Forward DFT of the line in a (b is scratch of the same length) by one warp;
// returns the buffer that holds the result.
__device__ float4 *df_fft_line(float4 *a, float4 *b, const DfAxisPlan &p, const float4 *tw, int lane) {
    for (int s = 0; s < p.nst; ++s) {
        const float4 *t = tw + p.twoff[s];
        switch (p.R[s]) {
            case 4: df_stage<4>(a, b, p.N, p.Ns[s], t, lane, 32); break;
            case 3: df_stage<3>(a, b, p.N, p.Ns[s], t, lane, 32); break;
            case 5: df_stage<5>(a, b, p.N, p.Ns[s], t, lane, 32); break;
            default: df_stage<2>(a, b, p.N, p.Ns[s], t, lane, 32); break;
        }
        __syncwarp();
        float4 *x = a;
        a = b;
        b = x;
    }
    return a;
}

// Runs the line FFT and leaves the result in `a`.
__device__ __forceinline__ void df_fft_inplace(float4 *a, float4 *b, const DfAxisPlan &p, const float4 *tw,
                                               int lane) {
    float4 *r = df_fft_line(a, b, p, tw, lane);
    if (r != a) {
        for (int i = lane; i < p.N; i += 32) a[i] = r[i];
        __syncwarp();
    }
}

__device__ __forceinline__ void load_twiddles(float4 *dst, const DfAxisPlan &p) {
    for (int i = threadIdx.x; i < p.ntw; i += blockDim.x) dst[i] = p.tw[i];
}

// ---------------------------------------------------------------------------
// x pass
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_df_x_fwd(const double *__restrict__ grid, float4 *__restrict__ spec,
                                                  int ncomp, GridParams gp, DfAxisPlan px) {
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    float4 *tw = sm;
    float4 *A = sm + px.ntw + warp * 2 * Nx, *B = A + Nx;
    load_twiddles(tw, px);
    __syncthreads();
    const int npairs = (Ny + 1) / 2;
    const int64_t total = (int64_t)ncomp * Nz * npairs;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < total; t += (int64_t)gridDim.x * nw) {
        const int yp = (int)(t % npairs);
        const int64_t cz = t / npairs;
        const int y0 = 2 * yp;
        const bool has1 = y0 + 1 < Ny;
        const double *r0 = grid + (cz * Ny + y0) * (int64_t)Nx;
        const double *r1 = r0 + Nx;
        for (int n = lane; n < Nx; n += 32) {
            dfc z;
            z.re = dfrom(r0[n]);
            z.im = has1 ? dfrom(r1[n]) : dfr{0.f, 0.f};
            A[n] = st4(z);
        }
        __syncwarp();
        const float4 *Z = df_fft_line(A, B, px, tw, lane);
        float4 *o0 = spec + (cz * Ny + y0) * (int64_t)Nxh;
        float4 *o1 = o0 + Nxh;
        for (int k = lane; k < Nxh; k += 32) {
            const dfc zk = ld4(Z[k]);
            const dfc zc = cconj(ld4(Z[(Nx - k) % Nx]));
            o0[k] = st4(chalf(cadd(zk, zc)));
            if (has1) o1[k] = st4(mul_mi(chalf(csub(zk, zc))));
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(128) k_df_x_inv(const float4 *__restrict__ spec, double *__restrict__ grid,
                                                  int ncomp, GridParams gp, DfAxisPlan px) {
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    float4 *tw = sm;
    float4 *A = sm + px.ntw + warp * 2 * Nx, *B = A + Nx;
    load_twiddles(tw, px);
    __syncthreads();
    const int npairs = (Ny + 1) / 2;
    const int64_t total = (int64_t)ncomp * Nz * npairs;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < total; t += (int64_t)gridDim.x * nw) {
        const int yp = (int)(t % npairs);
        const int64_t cz = t / npairs;
        const int y0 = 2 * yp;
        const bool has1 = y0 + 1 < Ny;
        const float4 *i0 = spec + (cz * Ny + y0) * (int64_t)Nxh;
        const float4 *i1 = i0 + Nxh;
        for (int n = lane; n < Nx; n += 32) {
            const bool upper = n > Nx / 2;
            const int k = upper ? Nx - n : n;
            dfc x0 = ld4(i0[k]);
            dfc x1 = has1 ? ld4(i1[k]) : czero();
            if (k == 0 || 2 * k == Nx) {   // real bins of a real line
                x0.im = dfr{0.f, 0.f};
                x1.im = dfr{0.f, 0.f};
            }
            if (upper) {
                x0 = cconj(x0);
                x1 = cconj(x1);
            }
            A[n] = st4(cconj(cadd(x0, mul_i(x1))));
        }
        __syncwarp();
        const float4 *Z = df_fft_line(A, B, px, tw, lane);
        double *r0 = grid + (cz * Ny + y0) * (int64_t)Nx;
        double *r1 = r0 + Nx;
        for (int n = lane; n < Nx; n += 32) {
            const dfc z = ld4(Z[n]);   // conj of the inverse: re as is, im negated
            r0[n] = dto(z.re);
            if (has1) r1[n] = -dto(z.im);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// y pass: tiles of TX consecutive kx columns of one (component, z) plane
// ---------------------------------------------------------------------------
__global__ void k_df_y(float4 *__restrict__ spec, int64_t nplanes, GridParams gp, DfAxisPlan py, int tx,
                       int inverse) {
    extern __shared__ float4 sm[];
    const int Ny = gp.N[1], Nxh = gp.N[0] / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4 *tw = sm;
    float4 *D = sm + py.ntw;
    float4 *S = D + (int64_t)tx * Ny;
    load_twiddles(tw, py);
    const int nblk = (Nxh + tx - 1) / tx;
    for (int64_t tile = blockIdx.x; tile < nplanes * nblk; tile += gridDim.x) {
        const int64_t plane = tile / nblk;
        const int kx0 = (int)(tile % nblk) * tx;
        float4 *base = spec + plane * Ny * (int64_t)Nxh + kx0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < tx * Ny; idx += blockDim.x) {
            const int y = idx / tx, t = idx % tx;
            if (kx0 + t < Nxh) {
                dfc v = ld4(base[(int64_t)y * Nxh + t]);
                D[t * Ny + y] = st4(inverse ? cconj(v) : v);
            }
        }
        __syncthreads();
        if (warp < tx && kx0 + warp < Nxh) df_fft_inplace(D + warp * Ny, S + warp * Ny, py, tw, lane);
        __syncthreads();
        for (int idx = threadIdx.x; idx < tx * Ny; idx += blockDim.x) {
            const int y = idx / tx, t = idx % tx;
            if (kx0 + t < Nxh) {
                const dfc v = ld4(D[t * Ny + y]);
                base[(int64_t)y * Nxh + t] = st4(inverse ? cconj(v) : v);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// z pass + dipole scale + inverse z pass, the 3 components of one vector
// ---------------------------------------------------------------------------
__global__ void k_df_z_scale(float4 *__restrict__ spec, int nrhs, GridParams gp, DfAxisPlan pz,
                             const double *__restrict__ H, int tx) {
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t Gc = (int64_t)Nxh * Ny * Nz;
    const int64_t zstride = (int64_t)Ny * Nxh;
    float4 *tw = sm;
    float4 *D = sm + pz.ntw;                   // [3 tx][Nz]
    float4 *S = D + 3 * (int64_t)tx * Nz;
    load_twiddles(tw, pz);
    const int nblk = (Nxh + tx - 1) / tx;
    const int64_t ntiles = (int64_t)nrhs * Ny * nblk;
    const int col = warp;                      // column of this warp: component col / tx, kx0 + col % tx
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int kb = (int)(tile % nblk);
        const int ky = (int)((tile / nblk) % Ny);
        const int r = (int)(tile / ((int64_t)nblk * Ny));
        const int kx0 = kb * tx;
        float4 *base = spec + (int64_t)(3 * r) * Gc + (int64_t)ky * Nxh + kx0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < 3 * tx * Nz; idx += blockDim.x) {
            const int c = idx / (tx * Nz), rem = idx % (tx * Nz);
            const int z = rem / tx, t = rem % tx;
            if (kx0 + t < Nxh) D[(c * tx + t) * Nz + z] = base[c * Gc + z * zstride + t];
        }
        __syncthreads();
        const bool active = col < 3 * tx && kx0 + col % tx < Nxh;
        if (active) df_fft_inplace(D + col * Nz, S + col * Nz, pz, tw, lane);
        __syncthreads();
        // H k k^T with the Nyquist rule of the float64 path; conj for the inverse
        for (int idx = threadIdx.x; idx < tx * Nz; idx += blockDim.x) {
            const int z = idx / tx, t = idx % tx;
            const int kx = kx0 + t;
            if (kx >= Nxh) continue;
            const double qx = fft_freq(kx, Nx) * gp.kfac[0];
            const double qy = fft_freq(ky, Ny) * gp.kfac[1];
            const double qz = fft_freq(z, Nz) * gp.kfac[2];
            const double k2 = qx * qx + qy * qy + qz * qz;
            const double h = H[kx + (int64_t)Nxh * (ky + (int64_t)Ny * z)];
            double q[3] = {0.0, 0.0, 0.0};
            if (k2 > 0.0) {
                const double inv = 1.0 / sqrt(k2);
                q[0] = qx * inv;
                q[1] = qy * inv;
                q[2] = qz * inv;
            }
            const bool ny3[3] = {(Nx % 2 == 0) && (kx == Nx / 2), (Ny % 2 == 0) && (ky == Ny / 2),
                                 (Nz % 2 == 0) && (z == Nz / 2)};
            dfc f[3], g[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c] = ld4(D[(c * tx + t) * Nz + z]);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                g[i] = czero();
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    if (ny3[i] != ny3[j]) continue;
                    const double tij = h * q[i] * q[j];
                    if (tij == 0.0) continue;
                    g[i] = cadd(g[i], cscale(f[j], dfrom(tij)));
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) D[(c * tx + t) * Nz + z] = st4(cconj(g[c]));
        }
        __syncthreads();
        if (active) df_fft_inplace(D + col * Nz, S + col * Nz, pz, tw, lane);
        __syncthreads();
        for (int idx = threadIdx.x; idx < 3 * tx * Nz; idx += blockDim.x) {
            const int c = idx / (tx * Nz), rem = idx % (tx * Nz);
            const int z = rem / tx, t = rem % tx;
            if (kx0 + t < Nxh) base[c * Gc + z * zstride + t] = st4(cconj(ld4(D[(c * tx + t) * Nz + z])));
        }
    }
}

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
struct DfTable {
    float4 *tw = nullptr;
    DfAxisPlan plan;
};
static std::map<std::pair<int, int>, DfTable> g_df_tables;
static std::mutex g_df_mu;

static bool df_axis(int N, int dev, DfAxisPlan *out) {
    if (N < 2 || N > 1024) return false;
    auto key = std::make_pair(dev, N);
    std::lock_guard<std::mutex> lk(g_df_mu);
    auto it = g_df_tables.find(key);
    if (it != g_df_tables.end()) {
        *out = it->second.plan;
        return true;
    }
    DfAxisPlan p;
    p.N = N;
    int m = N;
    const int radices[4] = {4, 3, 5, 2};
    for (int R : radices)
        while (m % R == 0) {
            if (p.nst >= kDfMaxStages) return false;
            p.R[p.nst++] = R;
            m /= R;
        }
    if (m != 1) return false;
    std::vector<float4> tw;
    int ns = 1;
    for (int s = 0; s < p.nst; ++s) {
        const int R = p.R[s];
        p.Ns[s] = ns;
        p.twoff[s] = (int)tw.size();
        for (int jm = 0; jm < ns; ++jm)
            for (int r = 0; r < R; ++r) {
                const double ang = -2.0 * M_PI * (double)(jm * r) / (double)(ns * R);
                const double c = cos(ang), sn = sin(ang);
                const float ch = (float)c, sh = (float)sn;
                tw.push_back(make_float4(ch, (float)(c - (double)ch), sh, (float)(sn - (double)sh)));
            }
        ns *= R;
    }
    p.ntw = (int)tw.size();
    float4 *d = nullptr;
    if (cudaMalloc((void **)&d, sizeof(float4) * tw.size()) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (cudaMemcpy(d, tw.data(), sizeof(float4) * tw.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return false;
    }
    p.tw = d;
    g_df_tables[key] = DfTable{d, p};
    *out = p;
    return true;
}

int df_plan(const GridParams &gp, DfPlan3 *out) {
    out->ok = false;
    if (gp.N[0] % 2 != 0) return MPS_OK;
    int dev = 0;
    MPS_CUDA_TRY(cudaGetDevice(&dev));
    for (int d = 0; d < 3; ++d)
        if (!df_axis(gp.N[d], dev, &out->ax[d])) return MPS_OK;
    out->ok = true;
    return MPS_OK;
}

static int max_smem_optin() {
    static int v = -1;
    if (v < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) v = 48 * 1024;
    }
    return v;
}

template <typename K>
static int set_smem(K kernel, size_t bytes) {
    if (bytes > (size_t)max_smem_optin()) return MPS_BAD_ARG;
    if (bytes > 48 * 1024)
        MPS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return MPS_OK;
}

static int launch_x(bool fwd, const double *gin, double *gout, float4 *spec, int ncomp, const GridParams &gp,
                    const DfAxisPlan &px, cudaStream_t s) {
    const int nw = 4;
    const size_t smem = sizeof(float4) * ((size_t)px.ntw + (size_t)nw * 2 * gp.N[0]);
    const int64_t total = (int64_t)ncomp * gp.N[2] * ((gp.N[1] + 1) / 2);
    const int blocks = grid_for(total, nw, 152 * 16);
    if (fwd) {
        MPS_TRY_STATUS(set_smem(k_df_x_fwd, smem));
        k_df_x_fwd<<<blocks, nw * 32, smem, s>>>(gin, spec, ncomp, gp, px);
    } else {
        MPS_TRY_STATUS(set_smem(k_df_x_inv, smem));
        k_df_x_inv<<<blocks, nw * 32, smem, s>>>(spec, gout, ncomp, gp, px);
    }
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

static int launch_y(float4 *spec, int ncomp, const GridParams &gp, const DfAxisPlan &py, int inverse,
                    cudaStream_t s) {
    int tx = 8;
    size_t smem = 0;
    for (; tx >= 1; tx /= 2) {
        smem = sizeof(float4) * ((size_t)py.ntw + 2 * (size_t)tx * gp.N[1]);
        if (smem <= (size_t)max_smem_optin()) break;
    }
    if (tx < 1) return MPS_BAD_ARG;
    MPS_TRY_STATUS(set_smem(k_df_y, smem));
    const int64_t nplanes = (int64_t)ncomp * gp.N[2];
    const int nblk = (gp.N[0] / 2 + 1 + tx - 1) / tx;
    const int blocks = grid_for(nplanes * nblk, 1, 152 * 8);
    k_df_y<<<blocks, tx * 32, smem, s>>>(spec, nplanes, gp, py, tx, inverse);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int df_forward_xy(const double *grid, float4 *spec, int ncomp, const GridParams &gp, const DfPlan3 &pl,
                  cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS(launch_x(true, grid, nullptr, spec, ncomp, gp, pl.ax[0], s));
    return launch_y(spec, ncomp, gp, pl.ax[1], 0, s);
}

int df_inverse_yx(float4 *spec, double *grid, int ncomp, const GridParams &gp, const DfPlan3 &pl, cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS(launch_y(spec, ncomp, gp, pl.ax[1], 1, s));
    return launch_x(false, nullptr, grid, spec, ncomp, gp, pl.ax[0], s);
}

int df_z_scale_dipole(float4 *spec, int nrhs, const GridParams &gp, const DfPlan3 &pl, const double *H,
                      cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    const DfAxisPlan &pz = pl.ax[2];
    int tx = 4;
    size_t smem = 0;
    for (; tx >= 1; tx /= 2) {
        smem = sizeof(float4) * ((size_t)pz.ntw + 2 * 3 * (size_t)tx * gp.N[2]);
        if (smem <= (size_t)max_smem_optin()) break;
    }
    if (tx < 1) return MPS_BAD_ARG;
    MPS_TRY_STATUS(set_smem(k_df_z_scale, smem));
    const int nblk = (gp.N[0] / 2 + 1 + tx - 1) / tx;
    const int64_t ntiles = (int64_t)nrhs * gp.N[1] * nblk;
    k_df_z_scale<<<grid_for(ntiles, 1, 152 * 8), 3 * tx * 32, smem, s>>>(spec, nrhs, gp, pz, H, tx);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

}  // namespace mps
