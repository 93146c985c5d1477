// Dot-product accumulators of the cluster kernels.
//
// A kernel's accumulation type A is float (native FP32 systems), double
// (FP64 systems, or FP32 systems with FP64 accumulation), or f2acc:
// float-float, the unevaluated sum hi + lo of two floats.  On GB300 the FP64
// pipe issues at a small fraction of the FP32 rate, and a cluster-wide
// reduction in double (per-thread products, warp butterflies, slot sums, the
// alpha / beta divisions in every thread) costs several times the rest of a
// PCG iteration.  f2acc keeps that work on the FP32 pipe with a 48-bit
// significand:
//   * a product of two floats is exact as a pair (Dekker's product with one
//     fused multiply-add: p = a*b, e = fma(a, b, -p));
//   * sums are cascaded (Ogita, Rump and Oishi, "Accurate sum and dot
//     product", SIAM J. Sci. Comput. 26, 2005, algorithms Sum2 / Dot2): the
//     high words are added with Knuth's TwoSum (the exact rounding error of a
//     float addition, six additions, no branch) and every error term, like
//     every low word, is added into the low word.  The result is as accurate
//     as if summed in twice the working precision and rounded:
//     |s - sum x| <= u |sum x| + gamma_d^2 sum |x|, u = 2^-24, d the depth of
//     the summation tree, gamma_d = d u / (1 - d u).  The critical path of a
//     sum chain is one float addition per term, as for plain float sums;
//   * a finished reduction is renormalised once (TwoSum of its two words), so
//     that comparisons and the quotients see hi + lo with |lo| <= ulp(hi)/2;
//   * the quotients alpha = eta / p.Sp and beta = eta' / eta are needed in
//     FP32 only; they come from one float division and one correction step of
//     the double-word remainder.
// Every addition uses the round-to-nearest intrinsics so that the compiler
// neither contracts nor reassociates them.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace gbdpcg {

struct __align__(8) f2acc {
    float hi, lo;
    f2acc() = default;
    __host__ __device__ constexpr f2acc(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ constexpr f2acc(float h) : hi(h), lo(0.f) {}
    __host__ __device__ constexpr f2acc(float h, float l) : hi(h), lo(l) {}
    // nearest pair to a double (threshold set-up, once per system)
    __device__ explicit f2acc(double d) {
        hi = __double2float_rn(d);
        lo = __double2float_rn(d - (double)hi);
    }
    __device__ explicit operator double() const { return (double)hi + (double)lo; }
    __device__ explicit operator float() const { return hi; }
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Cascaded addition: the pair is not renormalised (see acc_normalize).
__device__ __forceinline__ f2acc operator+(const f2acc &a, const f2acc &b) {
    float s, t;
    two_sum(a.hi, b.hi, s, t);
    return f2acc(s, __fadd_rn(__fadd_rn(a.lo, b.lo), t));
}

// hi + lo with |lo| <= ulp(hi)/2, the same value to within the rounding of lo
__device__ __forceinline__ f2acc renormalize(const f2acc &a) {
    float s, e;
    two_sum(a.hi, a.lo, s, e);
    return f2acc(s, e);
}
__device__ __forceinline__ f2acc &operator+=(f2acc &a, const f2acc &b) { return a = a + b; }
__device__ __forceinline__ f2acc operator-(const f2acc &a) { return f2acc(-a.hi, -a.lo); }
__device__ __forceinline__ bool operator==(const f2acc &a, const f2acc &b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator<(const f2acc &a, const f2acc &b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator<=(const f2acc &a, const f2acc &b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}

// ---- uniform helpers over float, double and f2acc

// v += a * b (float / double: the expression the kernels always used)
template <typename A, typename T>
__device__ __forceinline__ void acc_madd(A &v, T a, T b) {
    if constexpr (std::is_same<A, f2acc>::value) {
        static_assert(std::is_same<T, float>::value, "float-float accumulates float products");
        const float p = __fmul_rn(a, b);
        v += f2acc(p, __fmaf_rn(a, b, -p));
    } else {
        v += A(a) * A(b);
    }
}

// T(a / b)
template <typename T, typename A>
__device__ __forceinline__ T acc_ratio(const A &a, const A &b) {
    if constexpr (std::is_same<A, f2acc>::value) {
        const float q = __fdiv_rn(a.hi, b.hi);
        float r = __fmaf_rn(-q, b.hi, a.hi);  // a.hi - q b.hi, exact
        r = __fadd_rn(r, a.lo);
        r = __fmaf_rn(-q, b.lo, r);
        return T(__fadd_rn(q, __fdiv_rn(r, b.hi)));
    } else {
        return T(a / b);
    }
}

// A finished reduction, ready for comparisons and quotients.
template <typename A>
__device__ __forceinline__ A acc_normalize(const A &a) {
    if constexpr (std::is_same<A, f2acc>::value) return renormalize(a);
    else return a;
}

template <typename A>
__device__ __forceinline__ bool acc_finite(const A &a) {
    if constexpr (std::is_same<A, f2acc>::value) return isfinite(a.hi) && isfinite(a.lo);
    else return isfinite(a);
}

template <typename A>
__device__ __forceinline__ A acc_abs(const A &a) {
    if constexpr (std::is_same<A, f2acc>::value) return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? -a : a;
    else return fabs(a);
}

template <typename A>
__device__ __forceinline__ A acc_shfl_xor(const A &v, int off) {
    if constexpr (std::is_same<A, f2acc>::value)
        return f2acc(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
    else return __shfl_xor_sync(0xffffffffu, v, off);
}

// Accumulator code of a (T, A) pair as the variant registry records it:
// 0 native (A = T = float), 1 double, 2 float-float.
template <typename T, typename A>
constexpr int acc_code() {
    return std::is_same<A, f2acc>::value ? 2 : (sizeof(A) == 8 ? 1 : 0);
}

}  // namespace gbdpcg
