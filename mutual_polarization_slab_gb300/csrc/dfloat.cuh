// Double-float scalar (value = hi + lo, two floats, ~48-bit significand) with the
// operators the tiled spread / contract templates use.  Sums use the two-sum
// error-free transformation, products the FMA two-product; every step is an
// explicitly rounded intrinsic so the compiler cannot contract or reorder it.
#pragma once

#include <cuda_runtime.h>

namespace mps {

struct __align__(8) dfv {
    float hi, lo;
    dfv() = default;
    __device__ __forceinline__ dfv(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit dfv(double v) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(v - (double)hi);
    }
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfv dfv_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dfv(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dfv operator+(dfv a, dfv b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return dfv_fast_two_sum(s, e);
}

__device__ __forceinline__ dfv operator*(dfv a, dfv b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return dfv_fast_two_sum(p, e);
}

__device__ __forceinline__ dfv operator-(dfv a) { return dfv(-a.hi, -a.lo); }
__device__ __forceinline__ dfv operator-(dfv a, dfv b) { return a + (-b); }

// Exact difference of two floats as a double-float (two-sum).
__device__ __forceinline__ dfv dfv_two_diff(float a, float b) {
    const float s = __fsub_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-b, bb));
    return dfv(s, e);
}

__device__ __forceinline__ dfv &operator+=(dfv &a, dfv b) {
    a = a + b;
    return a;
}

__device__ __forceinline__ dfv warp_sum(dfv v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const dfv w(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
        v = v + w;
    }
    return v;
}

// Accumulator of a sum of products.  Plain for float and double; for dfv an
// unnormalised (sum, error) float pair: exact leading products (FMA residual),
// a two-sum of the leading parts, the error terms summed in the companion float,
// one normalisation when the value is read.  About 2/3 of the work of dfv
// operator+= (a * b), to the same ~2^-48 relative accuracy for sums of a few
// dozen terms.
template <typename T>
struct ProdAcc {
    T v;
    __device__ __forceinline__ void zero() { v = (T)0; }
    __device__ __forceinline__ void add(T a, T b) { v += a * b; }
    __device__ __forceinline__ T get() const { return v; }
};
template <>
struct ProdAcc<dfv> {
    float s, e;
    __device__ __forceinline__ void zero() { s = e = 0.f; }
    __device__ __forceinline__ void add(dfv a, dfv b) {
        const float p = __fmul_rn(a.hi, b.hi);
        float q = __fmaf_rn(a.hi, b.hi, -p);
        q = __fmaf_rn(a.hi, b.lo, q);
        q = __fmaf_rn(a.lo, b.hi, q);
        const float t = __fadd_rn(s, p);
        const float bp = __fsub_rn(t, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
        e = __fadd_rn(e, __fadd_rn(err, q));
        s = t;
    }
    __device__ __forceinline__ dfv get() const { return dfv_fast_two_sum(s, e); }
};

}  // namespace mps
