// Double-word arithmetic: a value as an unevaluated sum hi + lo of two FP32
// numbers (|lo| <= ulp(hi) / 2), about 48 bits of precision from FP32
// instructions.  GB300 executes FP64 at 1/72 of its FP32 rate, so work that
// needs more than FP32 but not all of FP64 is cheaper this way.
//
// The building blocks are the published error-free transformations (Knuth's
// TwoSum, Dekker's Fast2Sum, the FMA-based TwoProd) and the double-word
// algorithms analysed by Joldes, Muller and Popescu, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic" (ACM TOMS
// 44, 2017): AccurateDWPlusDW (relative error <= 3 u^2), DWTimesDW3
// (<= 4 u^2) and DWTimesFP3 (<= 2 u^2), u = 2^-24.  All operations use the
// round-to-nearest intrinsics so the compiler cannot contract them.
#pragma once
#include <cuda_runtime.h>

namespace dfcsr {

struct dw {
    float hi, lo;
};

__device__ __forceinline__ dw dw_make(float hi, float lo) { return dw{hi, lo}; }

// exact split of a double into hi + lo (lo rounds the remainder)
__device__ __forceinline__ dw dw_from(double v) {
    const float hi = __double2float_rn(v);
    return dw{hi, __double2float_rn(v - (double)hi)};
}

__device__ __forceinline__ double dw_to_double(dw a) { return (double)a.hi + (double)a.lo; }

// nearest FP32 value of hi + lo
__device__ __forceinline__ float dw_float(dw a) { return __fadd_rn(a.hi, a.lo); }

__device__ __forceinline__ dw two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dw{s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dw fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dw{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dw two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return dw{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dw dw_neg(dw a) { return dw{-a.hi, -a.lo}; }

__device__ __forceinline__ dw dw_add(dw x, dw y) {
    const dw s = two_sum(x.hi, y.hi);
    const dw t = two_sum(x.lo, y.lo);
    const dw v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

__device__ __forceinline__ dw dw_sub(dw x, dw y) { return dw_add(x, dw_neg(y)); }

// double-word + FP32
__device__ __forceinline__ dw dw_add_f(dw x, float y) {
    const dw s = two_sum(x.hi, y);
    return fast_two_sum(s.hi, __fadd_rn(x.lo, s.lo));
}

__device__ __forceinline__ dw dw_mul(dw x, dw y) {
    const dw c = two_prod(x.hi, y.hi);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    return fast_two_sum(c.hi, __fadd_rn(c.lo, cl2));
}

// double-word x FP32
__device__ __forceinline__ dw dw_mul_f(dw x, float y) {
    const dw c = two_prod(x.hi, y);
    return fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}

// x + a * b (double-word)
__device__ __forceinline__ dw dw_fma(dw a, dw b, dw x) { return dw_add(dw_mul(a, b), x); }

// square root of a non-negative double-word: the FP32 root corrected by one
// Newton step on the double-word residual x - s^2.
__device__ __forceinline__ dw dw_sqrt(dw x) {
    if (!(x.hi > 0.f)) return dw{__fsqrt_rn(x.hi), 0.f};
    const float s = __fsqrt_rn(x.hi);
    const dw p = two_prod(s, s);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p.hi), p.lo), x.lo);
    return fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.f, s)));
}

// x + y when only the absolute error matters, or when x and y have the same
// sign (Dekker's add: one TwoSum on the high parts, the low parts added in
// FP32): |error| <= about 2^-47 * (|x| + |y|), i.e. it may lose relative
// accuracy under cancellation but never absolute accuracy.
__device__ __forceinline__ dw dw_add_abs(dw x, dw y) {
    const dw s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ dw dw_sub_abs(dw x, dw y) { return dw_add_abs(x, dw_neg(y)); }

// quotient of double-words: the FP32 quotient corrected by one step on the
// double-word remainder x - q y.
__device__ __forceinline__ dw dw_div(dw x, dw y) {
    const float q = __fdiv_rn(x.hi, y.hi);
    const dw p = dw_mul_f(y, q);
    const dw r = dw_sub(x, p);
    return fast_two_sum(q, __fdiv_rn(r.hi, y.hi));
}

// Square root and reciprocal square root of a positive double-word x from
// one hardware reciprocal square root y ~ 1/sqrt(x.hi) (a few ulp): the root
// is s + (x - s^2) y / 2 with s = x.hi y (one Newton step on the exact
// double-word residual, ~2^-46 relative); *inv_root gets y (FP32 accuracy).
__device__ __forceinline__ dw dw_sqrt_rsq(dw x, float *inv_root) {
    const float y = rsqrtf(x.hi);
    const float s = __fmul_rn(x.hi, y);
    const dw p = two_prod(s, s);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p.hi), p.lo), x.lo);
    *inv_root = y;
    return fast_two_sum(s, __fmul_rn(__fmul_rn(0.5f, res), y));
}

// reciprocal of a positive double-word x given y ~ 1/x.hi (a few ulp): one
// Newton step y + y (1 - x y), the residual 1 - x y formed with FMAs.
__device__ __forceinline__ dw dw_recip_from(dw x, float y) {
    const float e = __fsub_rn(__fmaf_rn(-x.hi, y, 1.f), __fmul_rn(x.lo, y));
    return fast_two_sum(y, __fmul_rn(y, e));
}

// floor of the double-word value as a double-word integer (hi + lo is the
// exact value; floor(hi) can be off by one when hi is an integer and lo < 0,
// or when hi is so large that lo carries the fraction)
__device__ __forceinline__ float dw_floor(dw a) {
    float f = floorf(a.hi);
    if (f == a.hi) {                    // hi integral: the fraction is in lo
        f = __fadd_rn(f, floorf(a.lo));
    }
    return f;
}

}  // namespace dfcsr
