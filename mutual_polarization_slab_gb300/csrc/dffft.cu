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
// Sums and products inside a butterfly leave their result unnormalised: (s, e)
// with s the rounded leading sum (product) and e its exact rounding error plus
// the companion terms, |e| a few ulp of s.  The two-sum and the FMA residual are
// exact for any leading parts, so an unnormalised operand costs at most a couple
// of bits of the ~2^-48 accuracy; values are normalised once when a stage stores
// them (st4, re_s, nim_s), not after every operation.
__device__ __forceinline__ dfr dadd(dfr a, dfr b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return {s, e};
}
__device__ __forceinline__ dfr dneg(dfr a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfr dsub(dfr a, dfr b) { return dadd(a, dneg(b)); }
__device__ __forceinline__ dfr dmul(dfr a, dfr b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
}
__device__ __forceinline__ dfr dnorm(dfr a) { return fts(a.hi, a.lo); }
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
__device__ __forceinline__ float4 st4(dfc a) {
    const dfr r = dnorm(a.re), i = dnorm(a.im);
    return make_float4(r.hi, r.lo, i.hi, i.lo);
}
__device__ __forceinline__ dfc czero() { return {{0.f, 0.f}, {0.f, 0.f}}; }

// Arithmetic policies: the storage type S of a complex value in memory and its
// register form V, with the operations the transforms use.
struct ArithDF {
    using S = float4;
    using V = dfc;
    __device__ static __forceinline__ V ld(S v) { return ld4(v); }
    __device__ static __forceinline__ S st(V v) { return st4(v); }
    __device__ static __forceinline__ V tw(float4 t) { return ld4(t); }
    __device__ static __forceinline__ V add(V a, V b) { return cadd(a, b); }
    __device__ static __forceinline__ V sub(V a, V b) { return csub(a, b); }
    __device__ static __forceinline__ V mul(V a, V b) { return cmul(a, b); }
    __device__ static __forceinline__ V scl(V a, double c) { return cscale(a, dfrom(c)); }
    __device__ static __forceinline__ V half(V a) { return chalf(a); }
    __device__ static __forceinline__ V pi(V a) { return mul_i(a); }
    __device__ static __forceinline__ V mi(V a) { return mul_mi(a); }
    __device__ static __forceinline__ V conj(V a) { return cconj(a); }
    __device__ static __forceinline__ V zero() { return czero(); }
    __device__ static __forceinline__ V make(double re, double im) { return {dfrom(re), dfrom(im)}; }
    // grids stored as (hi, lo) pairs
    __device__ static __forceinline__ V make(float2 re, float2 im) { return {{re.x, re.y}, {im.x, im.y}}; }
    __device__ static __forceinline__ float2 re_s(V a) {
        const dfr r = dnorm(a.re);
        return make_float2(r.hi, r.lo);
    }
    __device__ static __forceinline__ float2 nim_s(V a) {
        const dfr r = dnorm(a.im);
        return make_float2(-r.hi, -r.lo);
    }
    __device__ static __forceinline__ double re(V a) { return dto(a.re); }
    __device__ static __forceinline__ double im(V a) { return dto(a.im); }
    __device__ static __forceinline__ V zero_im(V a) { return {a.re, {0.f, 0.f}}; }
    // real coefficient from a table entry (hi, lo), carried in the re part
    __device__ static __forceinline__ V tm(float2 t) { return {{t.x, t.y}, {0.f, 0.f}}; }
    __device__ static __forceinline__ V mulr(V a, V c) { return cscale(a, c.re); }
};

struct ArithF32 {
    using S = float2;
    using V = float2;
    __device__ static __forceinline__ V ld(S v) { return v; }
    __device__ static __forceinline__ S st(V v) { return v; }
    __device__ static __forceinline__ V tw(float4 t) { return make_float2(t.x, t.z); }
    __device__ static __forceinline__ V add(V a, V b) { return make_float2(a.x + b.x, a.y + b.y); }
    __device__ static __forceinline__ V sub(V a, V b) { return make_float2(a.x - b.x, a.y - b.y); }
    __device__ static __forceinline__ V mul(V a, V b) {
        return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
    __device__ static __forceinline__ V scl(V a, double c) {
        const float f = (float)c;
        return make_float2(a.x * f, a.y * f);
    }
    __device__ static __forceinline__ V half(V a) { return make_float2(0.5f * a.x, 0.5f * a.y); }
    __device__ static __forceinline__ V pi(V a) { return make_float2(-a.y, a.x); }
    __device__ static __forceinline__ V mi(V a) { return make_float2(a.y, -a.x); }
    __device__ static __forceinline__ V conj(V a) { return make_float2(a.x, -a.y); }
    __device__ static __forceinline__ V zero() { return make_float2(0.f, 0.f); }
    __device__ static __forceinline__ V make(float re, float im) { return make_float2(re, im); }
    __device__ static __forceinline__ float re_s(V a) { return a.x; }
    __device__ static __forceinline__ float nim_s(V a) { return -a.y; }
    __device__ static __forceinline__ float re(V a) { return a.x; }
    __device__ static __forceinline__ float im(V a) { return a.y; }
    __device__ static __forceinline__ V zero_im(V a) { return make_float2(a.x, 0.f); }
    __device__ static __forceinline__ V tm(float2 t) { return make_float2(t.x, 0.f); }
    __device__ static __forceinline__ V mulr(V a, V c) { return make_float2(a.x * c.x, a.y * c.x); }
};

// Small DFTs, forward sign (w = exp(-2 pi i / R)).
template <class A, int R>
struct Dft;

template <class A>
struct Dft<A, 2> {
    __device__ static __forceinline__ void run(typename A::V *v) {
        const auto a = v[0], b = v[1];
        v[0] = A::add(a, b);
        v[1] = A::sub(a, b);
    }
};

template <class A>
struct Dft<A, 3> {
    __device__ static __forceinline__ void run(typename A::V *v) {
        const auto a = A::add(v[1], v[2]), b = A::sub(v[1], v[2]);
        const auto m = A::sub(v[0], A::half(a));
        const auto tb = A::scl(b, 0.86602540378443864676372317075294);
        v[0] = A::add(v[0], a);
        v[1] = A::add(m, A::mi(tb));
        v[2] = A::add(m, A::pi(tb));
    }
};

template <class A>
struct Dft<A, 4> {
    __device__ static __forceinline__ void run(typename A::V *v) {
        const auto a = A::add(v[0], v[2]), b = A::sub(v[0], v[2]), c = A::add(v[1], v[3]), d = A::sub(v[1], v[3]);
        v[0] = A::add(a, c);
        v[2] = A::sub(a, c);
        v[1] = A::add(b, A::mi(d));
        v[3] = A::add(b, A::pi(d));
    }
};

template <class A>
struct Dft<A, 5> {
    __device__ static __forceinline__ void run(typename A::V *v) {
        const double c1 = 0.30901699437494742410229341718282, c2 = -0.80901699437494742410229341718282;
        const double s1 = 0.95105651629515357211643933337938, s2 = 0.58778525229247312916870595463907;
        const auto a1 = A::add(v[1], v[4]), b1 = A::sub(v[1], v[4]), a2 = A::add(v[2], v[3]),
                   b2 = A::sub(v[2], v[3]);
        const auto m1 = A::add(v[0], A::add(A::scl(a1, c1), A::scl(a2, c2)));
        const auto m2 = A::add(v[0], A::add(A::scl(a1, c2), A::scl(a2, c1)));
        const auto t1 = A::add(A::scl(b1, s1), A::scl(b2, s2));
        const auto t2 = A::sub(A::scl(b1, s2), A::scl(b2, s1));
        v[0] = A::add(v[0], A::add(a1, a2));
        v[1] = A::add(m1, A::mi(t1));
        v[2] = A::add(m2, A::mi(t2));
        v[3] = A::add(m2, A::pi(t2));
        v[4] = A::add(m1, A::pi(t1));
    }
};

template <class A, int R>
__device__ __forceinline__ void fft_stage(const typename A::S *__restrict__ in, typename A::S *__restrict__ out,
                                          int N, int Ns, const float4 *__restrict__ tw, int lane) {
    const int NR = N / R;
    // j / Ns through a float reciprocal: j < 512 and Ns <= 512, so (j + 1/2) / Ns
    // stays at least 1/(2 Ns) >= 2^-10 from an integer while the float error is
    // below 2^-13 -- the truncation is exact
    const float inv_ns = 1.0f / (float)Ns;
    for (int j = lane; j < NR; j += 32) {
        const int jq = __float2int_rz(((float)j + 0.5f) * inv_ns);
        const int jm = j - jq * Ns;
        typename A::V v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[r] = A::ld(in[j + r * NR]);
            if (r > 0 && jm > 0) v[r] = A::mul(v[r], A::tw(tw[jm * R + r]));
        }
        Dft<A, R>::run(v);
        const int d = jq * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; ++r) out[d + r * Ns] = A::st(v[r]);
    }
}

// Forward DFT of the line in a (b is scratch of the same length) by one warp;
// returns the buffer that holds the result.
template <class A>
__device__ typename A::S *fft_line(typename A::S *a, typename A::S *b, const DfAxisPlan &p, const float4 *tw,
                                   int lane) {
    for (int s = 0; s < p.nst; ++s) {
        const float4 *t = tw + p.twoff[s];
        switch (p.R[s]) {
            case 4: fft_stage<A, 4>(a, b, p.N, p.Ns[s], t, lane); break;
            case 3: fft_stage<A, 3>(a, b, p.N, p.Ns[s], t, lane); break;
            case 5: fft_stage<A, 5>(a, b, p.N, p.Ns[s], t, lane); break;
            default: fft_stage<A, 2>(a, b, p.N, p.Ns[s], t, lane); break;
        }
        __syncwarp();
        typename A::S *x = a;
        a = b;
        b = x;
    }
    return a;
}

// Runs the line FFT and leaves the result in `a`.
template <class A>
__device__ __forceinline__ void fft_inplace(typename A::S *a, typename A::S *b, const DfAxisPlan &p,
                                            const float4 *tw, int lane) {
    typename A::S *r = fft_line<A>(a, b, p, tw, lane);
    if (r != a) {
        for (int i = lane; i < p.N; i += 32) a[i] = r[i];
        __syncwarp();
    }
}

__device__ __forceinline__ void load_twiddles(float4 *dst, const DfAxisPlan &p) {
    for (int i = threadIdx.x; i < p.ntw; i += blockDim.x) dst[i] = p.tw[i];
}

// Dynamic shared memory: the twiddle table (float4) first, the lines after it.
template <class A>
__device__ __forceinline__ typename A::S *lines_after(float4 *sm, int ntw) {
    return reinterpret_cast<typename A::S *>(sm + ntw);
}

// ---------------------------------------------------------------------------
// x pass (Rl = real type of the grids)
// ---------------------------------------------------------------------------
template <class A, typename Rl>
__global__ void __launch_bounds__(128) k_fft_x_fwd(const Rl *__restrict__ grid, typename A::S *__restrict__ spec,
                                                   int ncomp, GridParams gp, DfAxisPlan px) {
    using S = typename A::S;
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    S *Ab = lines_after<A>(sm, px.ntw) + warp * 2 * Nx, *Bb = Ab + Nx;
    load_twiddles(sm, px);
    __syncthreads();
    const int npairs = (Ny + 1) / 2;
    const int64_t total = (int64_t)ncomp * Nz * npairs;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < total; t += (int64_t)gridDim.x * nw) {
        const int yp = (int)(t % npairs);
        const int64_t cz = t / npairs;
        const int y0 = 2 * yp;
        const bool has1 = y0 + 1 < Ny;
        const Rl *r0 = grid + (cz * Ny + y0) * (int64_t)Nx;
        const Rl *r1 = r0 + Nx;
        for (int n = lane; n < Nx; n += 32) Ab[n] = A::st(A::make(r0[n], has1 ? r1[n] : Rl{}));
        __syncwarp();
        const S *Z = fft_line<A>(Ab, Bb, px, sm, lane);
        S *o0 = spec + (cz * Ny + y0) * (int64_t)Nxh;
        S *o1 = o0 + Nxh;
        for (int k = lane; k < Nxh; k += 32) {
            const auto zk = A::ld(Z[k]);
            const auto zc = A::conj(A::ld(Z[(Nx - k) % Nx]));
            o0[k] = A::st(A::half(A::add(zk, zc)));
            if (has1) o1[k] = A::st(A::mi(A::half(A::sub(zk, zc))));
        }
        __syncwarp();
    }
}

template <class A, typename Rl>
__global__ void __launch_bounds__(128) k_fft_x_inv(const typename A::S *__restrict__ spec, Rl *__restrict__ grid,
                                                   int ncomp, GridParams gp, DfAxisPlan px) {
    using S = typename A::S;
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    S *Ab = lines_after<A>(sm, px.ntw) + warp * 2 * Nx, *Bb = Ab + Nx;
    load_twiddles(sm, px);
    __syncthreads();
    const int npairs = (Ny + 1) / 2;
    const int64_t total = (int64_t)ncomp * Nz * npairs;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < total; t += (int64_t)gridDim.x * nw) {
        const int yp = (int)(t % npairs);
        const int64_t cz = t / npairs;
        const int y0 = 2 * yp;
        const bool has1 = y0 + 1 < Ny;
        const S *i0 = spec + (cz * Ny + y0) * (int64_t)Nxh;
        const S *i1 = i0 + Nxh;
        for (int n = lane; n < Nx; n += 32) {
            const bool upper = n > Nx / 2;
            const int k = upper ? Nx - n : n;
            auto x0 = A::ld(i0[k]);
            auto x1 = has1 ? A::ld(i1[k]) : A::zero();
            if (k == 0 || 2 * k == Nx) {   // real bins of a real line
                x0 = A::zero_im(x0);
                x1 = A::zero_im(x1);
            }
            if (upper) {
                x0 = A::conj(x0);
                x1 = A::conj(x1);
            }
            Ab[n] = A::st(A::conj(A::add(x0, A::pi(x1))));
        }
        __syncwarp();
        const S *Z = fft_line<A>(Ab, Bb, px, sm, lane);
        Rl *r0 = grid + (cz * Ny + y0) * (int64_t)Nx;
        Rl *r1 = r0 + Nx;
        for (int n = lane; n < Nx; n += 32) {
            const auto z = A::ld(Z[n]);   // conj of the inverse: re as is, im negated
            r0[n] = A::re_s(z);
            if (has1) r1[n] = A::nim_s(z);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// y pass: tiles of TX consecutive kx columns of one (component, z) plane
// ---------------------------------------------------------------------------
template <class A>
__global__ void k_fft_y(typename A::S *__restrict__ spec, int64_t nplanes, GridParams gp, DfAxisPlan py, int tx,
                        int inverse) {
    using S = typename A::S;
    extern __shared__ float4 sm[];
    const int Ny = gp.N[1], Nxh = gp.N[0] / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Ly = Ny + 1;                     // padded line stride: the transposes hit distinct banks
    S *D = lines_after<A>(sm, py.ntw);
    S *Sc = D + (int64_t)tx * Ly;
    load_twiddles(sm, py);
    const int nblk = (Nxh + tx - 1) / tx;
    for (int64_t tile = blockIdx.x; tile < nplanes * nblk; tile += gridDim.x) {
        const int64_t plane = tile / nblk;
        const int kx0 = (int)(tile % nblk) * tx;
        S *base = spec + plane * Ny * (int64_t)Nxh + kx0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < tx * Ny; idx += blockDim.x) {
            const int y = idx / tx, t = idx % tx;
            if (kx0 + t < Nxh) {
                const auto v = A::ld(base[(int64_t)y * Nxh + t]);
                D[t * Ly + y] = A::st(inverse ? A::conj(v) : v);
            }
        }
        __syncthreads();
        if (warp < tx && kx0 + warp < Nxh) fft_inplace<A>(D + warp * Ly, Sc + warp * Ly, py, sm, lane);
        __syncthreads();
        for (int idx = threadIdx.x; idx < tx * Ny; idx += blockDim.x) {
            const int y = idx / tx, t = idx % tx;
            if (kx0 + t < Nxh) {
                const auto v = A::ld(D[t * Ly + y]);
                base[(int64_t)y * Nxh + t] = A::st(inverse ? A::conj(v) : v);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// z pass + dipole scale + inverse z pass, the 3 components of one vector.
// CT: arithmetic of the scale's coefficient H q_i q_j (float64 for the
// double-float path, float32 for the float32 operator, as its cuFFT form).
// ---------------------------------------------------------------------------
template <class A, typename CT>
__global__ void k_fft_z_scale(typename A::S *__restrict__ spec, int nrhs, GridParams gp, DfAxisPlan pz,
                              const CT *__restrict__ H, const float2 *__restrict__ tm6, int tx) {
    using S = typename A::S;
    extern __shared__ float4 sm[];
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2], Nxh = Nx / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t Gc = (int64_t)Nxh * Ny * Nz;
    const int64_t zstride = (int64_t)Ny * Nxh;
    const int Lz = Nz + 1;                     // padded line stride
    S *D = lines_after<A>(sm, pz.ntw);         // [3 tx][Lz]
    S *Sc = D + 3 * (int64_t)tx * Lz;
    load_twiddles(sm, pz);
    const int nblk = (Nxh + tx - 1) / tx;
    const int64_t ntiles = (int64_t)nrhs * Ny * nblk;
    const int col = warp;                      // column of this warp: component col / tx, kx0 + col % tx
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int kb = (int)(tile % nblk);
        const int ky = (int)((tile / nblk) % Ny);
        const int r = (int)(tile / ((int64_t)nblk * Ny));
        const int kx0 = kb * tx;
        S *base = spec + (int64_t)(3 * r) * Gc + (int64_t)ky * Nxh + kx0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < 3 * tx * Nz; idx += blockDim.x) {
            const int c = idx / (tx * Nz), rem = idx % (tx * Nz);
            const int z = rem / tx, t = rem % tx;
            if (kx0 + t < Nxh) D[(c * tx + t) * Lz + z] = base[c * Gc + z * zstride + t];
        }
        __syncthreads();
        const bool active = col < 3 * tx && kx0 + col % tx < Nxh;
        if (active) fft_inplace<A>(D + col * Lz, Sc + col * Lz, pz, sm, lane);
        __syncthreads();
        // H k k^T with the Nyquist rule of the cuFFT path; conj for the inverse
        for (int idx = threadIdx.x; idx < tx * Nz; idx += blockDim.x) {
            const int z = idx / tx, t = idx % tx;
            const int kx = kx0 + t;
            if (kx >= Nxh) continue;
            typename A::V f[3], g[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c] = A::ld(D[(c * tx + t) * Lz + z]);
            if (tm6) {
                // precomputed symmetric tensor (00, 01, 02, 11, 12, 22), double-float entries
                const float2 *tp = tm6 + 6 * (kx + (int64_t)Nxh * (ky + (int64_t)Ny * z));
                typename A::V T[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) T[q] = A::tm(tp[q]);
                g[0] = A::add(A::mulr(f[0], T[0]), A::add(A::mulr(f[1], T[1]), A::mulr(f[2], T[2])));
                g[1] = A::add(A::mulr(f[0], T[1]), A::add(A::mulr(f[1], T[3]), A::mulr(f[2], T[4])));
                g[2] = A::add(A::mulr(f[0], T[2]), A::add(A::mulr(f[1], T[4]), A::mulr(f[2], T[5])));
#pragma unroll
                for (int c = 0; c < 3; ++c) D[(c * tx + t) * Lz + z] = A::st(A::conj(g[c]));
                continue;
            }
            const CT qx = (CT)(fft_freq(kx, Nx) * gp.kfac[0]);
            const CT qy = (CT)(fft_freq(ky, Ny) * gp.kfac[1]);
            const CT qz = (CT)(fft_freq(z, Nz) * gp.kfac[2]);
            const CT k2 = qx * qx + qy * qy + qz * qz;
            const CT h = H[kx + (int64_t)Nxh * (ky + (int64_t)Ny * z)];
            CT q[3] = {(CT)0, (CT)0, (CT)0};
            if (k2 > (CT)0) {
                const CT inv = (CT)1 / sqrt(k2);
                q[0] = qx * inv;
                q[1] = qy * inv;
                q[2] = qz * inv;
            }
            const bool ny3[3] = {(Nx % 2 == 0) && (kx == Nx / 2), (Ny % 2 == 0) && (ky == Ny / 2),
                                 (Nz % 2 == 0) && (z == Nz / 2)};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                g[i] = A::zero();
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    if (ny3[i] != ny3[j]) continue;
                    const CT tij = h * q[i] * q[j];
                    if (tij == (CT)0) continue;
                    g[i] = A::add(g[i], A::scl(f[j], (double)tij));
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) D[(c * tx + t) * Lz + z] = A::st(A::conj(g[c]));
        }
        __syncthreads();
        if (active) fft_inplace<A>(D + col * Lz, Sc + col * Lz, pz, sm, lane);
        __syncthreads();
        for (int idx = threadIdx.x; idx < 3 * tx * Nz; idx += blockDim.x) {
            const int c = idx / (tx * Nz), rem = idx % (tx * Nz);
            const int z = rem / tx, t = rem % tx;
            if (kx0 + t < Nxh) base[c * Gc + z * zstride + t] = A::st(A::conj(A::ld(D[(c * tx + t) * Lz + z])));
        }
    }
}

// Symmetric scale tensor H q q^T per half-spectrum point, Nyquist rule applied,
// as double-float entries (00, 01, 02, 11, 12, 22): computed once per grid in
// float64 so the double-float z pass only reads it.  One thread per point of the
// spectrum's quarter (iy <= Ny/2, iz <= Nz/2): a mirrored point has H and the
// Nyquist flags of the original and q_y (q_z) negated exactly, so its entries are
// the original's with the signs of q_I q_J.
__global__ void k_df_tm6(GridParams gp, const double *__restrict__ H, float2 *__restrict__ tm6) {
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const HalfQuarter hq(gp.N);
    const int64_t Gq = hq.size();
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gq; t += (int64_t)gridDim.x * blockDim.x) {
        int kx, ky, kz;
        hq.point(t, &kx, &ky, &kz);
        const double qx = fft_freq(kx, Nx) * gp.kfac[0];
        const double qy = fft_freq(ky, Ny) * gp.kfac[1];
        const double qz = fft_freq(kz, Nz) * gp.kfac[2];
        const double k2 = qx * qx + qy * qy + qz * qz;
        double q[3] = {0.0, 0.0, 0.0};
        if (k2 > 0.0) {
            const double inv = 1.0 / sqrt(k2);
            q[0] = qx * inv;
            q[1] = qy * inv;
            q[2] = qz * inv;
        }
        const bool ny3[3] = {(Nx % 2 == 0) && (kx == Nx / 2), (Ny % 2 == 0) && (ky == Ny / 2),
                             (Nz % 2 == 0) && (kz == Nz / 2)};
        const double h = H[((int64_t)kz * Ny + ky) * hq.Nxh + kx];
        const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
        float2 e6[6];
        for (int e = 0; e < 6; ++e) {
            const double v = (ny3[I[e]] == ny3[J[e]]) ? h * q[I[e]] * q[J[e]] : 0.0;
            const dfr d = dfrom(v);
            e6[e] = make_float2(d.hi, d.lo);
        }
        mirror_points(hq, kx, ky, kz, [&](int64_t i, int sy, int sz) {
            const int sg[3] = {1, sy, sz};
            for (int e = 0; e < 6; ++e) {
                const float2 v = e6[e];
                tm6[6 * i + e] = sg[I[e]] * sg[J[e]] > 0 ? v : make_float2(-v.x, -v.y);
            }
        });
    }
}

int df_scale_table(const GridParams &gp, const double *H, float2 *tm6, cudaStream_t s) {
    k_df_tm6<<<grid_for(HalfQuarter(gp.N).size(), 256), 256, 0, s>>>(gp, H, tm6);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
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
    static const int v = [] {   // thread-safe one-time initialisation
        int dev = 0, r = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&r, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) r = 48 * 1024;
        return r;
    }();
    return v;
}

template <typename K>
static int set_smem(K kernel, size_t bytes) {
    if (bytes > (size_t)max_smem_optin()) return MPS_BAD_ARG;
    if (bytes > 48 * 1024)
        MPS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return MPS_OK;
}

template <class A, typename Rl>
static int launch_x(bool fwd, const Rl *gin, Rl *gout, typename A::S *spec, int ncomp, const GridParams &gp,
                    const DfAxisPlan &px, cudaStream_t s) {
    const int nw = 4;
    const size_t smem = sizeof(float4) * (size_t)px.ntw + sizeof(typename A::S) * (size_t)nw * 2 * gp.N[0];
    const int64_t total = (int64_t)ncomp * gp.N[2] * ((gp.N[1] + 1) / 2);
    const int blocks = grid_for(total, nw, 152 * 16);
    if (fwd) {
        MPS_TRY_STATUS(set_smem(k_fft_x_fwd<A, Rl>, smem));
        k_fft_x_fwd<A, Rl><<<blocks, nw * 32, smem, s>>>(gin, spec, ncomp, gp, px);
    } else {
        MPS_TRY_STATUS(set_smem(k_fft_x_inv<A, Rl>, smem));
        k_fft_x_inv<A, Rl><<<blocks, nw * 32, smem, s>>>(spec, gout, ncomp, gp, px);
    }
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <class A>
static int launch_y(typename A::S *spec, int ncomp, const GridParams &gp, const DfAxisPlan &py, int inverse,
                    cudaStream_t s) {
    int tx = 8;
    size_t smem = 0;
    for (; tx >= 1; tx /= 2) {
        smem = sizeof(float4) * (size_t)py.ntw + sizeof(typename A::S) * 2 * (size_t)tx * (gp.N[1] + 1);
        if (smem <= (size_t)max_smem_optin()) break;
    }
    if (tx < 1) return MPS_BAD_ARG;
    MPS_TRY_STATUS(set_smem(k_fft_y<A>, smem));
    const int64_t nplanes = (int64_t)ncomp * gp.N[2];
    const int nblk = (gp.N[0] / 2 + 1 + tx - 1) / tx;
    const int blocks = grid_for(nplanes * nblk, 1, 152 * 8);
    k_fft_y<A><<<blocks, tx * 32, smem, s>>>(spec, nplanes, gp, py, tx, inverse);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <class A, typename CT>
static int launch_z_scale(typename A::S *spec, int nrhs, const GridParams &gp, const DfAxisPlan &pz, const CT *H,
                          const float2 *tm6, cudaStream_t s) {
    int tx = 4;
    size_t smem = 0;
    for (; tx >= 1; tx /= 2) {
        smem = sizeof(float4) * (size_t)pz.ntw + sizeof(typename A::S) * 2 * 3 * (size_t)tx * (gp.N[2] + 1);
        if (smem <= (size_t)max_smem_optin()) break;
    }
    if (tx < 1) return MPS_BAD_ARG;
    MPS_TRY_STATUS(set_smem(k_fft_z_scale<A, CT>, smem));
    const int nblk = (gp.N[0] / 2 + 1 + tx - 1) / tx;
    const int64_t ntiles = (int64_t)nrhs * gp.N[1] * nblk;
    k_fft_z_scale<A, CT><<<grid_for(ntiles, 1, 152 * 8), 3 * tx * 32, smem, s>>>(spec, nrhs, gp, pz, H, tm6, tx);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int df_forward_xy(const float2 *grid, float4 *spec, int ncomp, const GridParams &gp, const DfPlan3 &pl,
                  cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS((launch_x<ArithDF, float2>(true, grid, nullptr, spec, ncomp, gp, pl.ax[0], s)));
    return launch_y<ArithDF>(spec, ncomp, gp, pl.ax[1], 0, s);
}

int df_inverse_yx(float4 *spec, float2 *grid, int ncomp, const GridParams &gp, const DfPlan3 &pl, cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS(launch_y<ArithDF>(spec, ncomp, gp, pl.ax[1], 1, s));
    return launch_x<ArithDF, float2>(false, nullptr, grid, spec, ncomp, gp, pl.ax[0], s);
}

int df_z_scale_dipole(float4 *spec, int nrhs, const GridParams &gp, const DfPlan3 &pl, const double *H,
                      const float2 *tm6, cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    return launch_z_scale<ArithDF, double>(spec, nrhs, gp, pl.ax[2], H, tm6, s);
}

int f32_forward_xy(const float *grid, float2 *spec, int ncomp, const GridParams &gp, const DfPlan3 &pl,
                   cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS((launch_x<ArithF32, float>(true, grid, nullptr, spec, ncomp, gp, pl.ax[0], s)));
    return launch_y<ArithF32>(spec, ncomp, gp, pl.ax[1], 0, s);
}

int f32_inverse_yx(float2 *spec, float *grid, int ncomp, const GridParams &gp, const DfPlan3 &pl, cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    MPS_TRY_STATUS(launch_y<ArithF32>(spec, ncomp, gp, pl.ax[1], 1, s));
    return launch_x<ArithF32, float>(false, nullptr, grid, spec, ncomp, gp, pl.ax[0], s);
}

int f32_z_scale_dipole(float2 *spec, int nrhs, const GridParams &gp, const DfPlan3 &pl, const float *H,
                       cudaStream_t s) {
    if (!pl.ok) return MPS_BAD_ARG;
    return launch_z_scale<ArithF32, float>(spec, nrhs, gp, pl.ax[2], H, nullptr, s);
}

}  // namespace mps
