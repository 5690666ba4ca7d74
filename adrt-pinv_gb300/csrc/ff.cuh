// Float-float arithmetic shared by the kernels that need FP64-class accuracy on the FP32 pipe.
#pragma once
#include <cuda_runtime.h>

namespace adrt {

// Float-float ("double-float") numbers: an unevaluated sum hi + lo of two FP32 values with |lo| <= ulp(hi)/2, about
// 48 significant bits, on the FP32 pipe (GB300's FP64 rate is a small fraction of its FP32 rate). Error-free
// transformations: TwoSum (Knuth, 6 operations, any magnitudes), Fast2Sum (Dekker, |a| >= |b|) and TwoProd through
// one fused multiply-add; double-word sum and product as in Joldes, Muller and Popescu, "Tight and rigorous error
// bounds for basic building blocks of double-word arithmetic", ACM TOMS 44 (2017): DWPlusDW (Algorithm 6, relative
// error below 3u^2) and DWTimesDW (Algorithm 12, below 4u^2), u = 2^-24. Every operation is an explicitly rounded
// intrinsic, so the compiler neither contracts nor reassociates them.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float ap = __fsub_rn(s, b);
    const float bp = __fsub_rn(s, ap);
    return {s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
    const ff s = two_sum(x.hi, y.hi);
    const ff t = two_sum(x.lo, y.lo);
    const ff v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}
__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_mul(ff x, ff y) {
    const float ch = __fmul_rn(x.hi, y.hi);
    const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
    const float tl1 = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.lo));
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}

__device__ __forceinline__ ff ff_from_d(double d) {
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double ff_to_d(ff v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }

// complex float-float values and the operations of the butterflies and the Chebyshev recurrence
struct ffc {
    ff re, im;
};
__device__ __forceinline__ ffc ffc_add(ffc a, ffc b) { return {ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ ffc ffc_sub(ffc a, ffc b) { return {ff_sub(a.re, b.re), ff_sub(a.im, b.im)}; }
// w * b
__device__ __forceinline__ ffc ffc_mul(ffc w, ffc b) {
    return {ff_sub(ff_mul(w.re, b.re), ff_mul(w.im, b.im)), ff_add(ff_mul(w.re, b.im), ff_mul(w.im, b.re))};
}
// conj(w) * b
__device__ __forceinline__ ffc ffc_mulc(ffc w, ffc b) {
    return {ff_add(ff_mul(w.re, b.re), ff_mul(w.im, b.im)), ff_sub(ff_mul(w.re, b.im), ff_mul(w.im, b.re))};
}
__device__ __forceinline__ ffc ffc_scale(ff s, ffc b) { return {ff_mul(s, b.re), ff_mul(s, b.im)}; }
__device__ __forceinline__ ffc ffc_from_d2(double2 v) { return {ff_from_d(v.x), ff_from_d(v.y)}; }
__device__ __forceinline__ ffc ffc_from_f2(float2 v) { return {{v.x, 0.f}, {v.y, 0.f}}; }
__device__ __forceinline__ float2 ffc_to_f2(ffc v) {
    return make_float2(__fadd_rn(v.re.hi, v.re.lo), __fadd_rn(v.im.hi, v.im.lo));
}

}  // namespace adrt
