// Float-float arithmetic: a value as the unevaluated sum of two FP32 numbers hi + lo (|lo| <= ulp(hi)/2), ~48
// significant bits from FP32 operations only. GB300's FP64 rate is 1/64 of its FP32 rate, so the mixed path's points
// that FP32 alone cannot take (near a source's edges, corners or plane, where the offsets and cross products cancel)
// are evaluated in float-float instead of FP64: their cancelling quantities keep ~48 bits, and the functions applied to
// them are the FP32 functions, as KMathHyb does with FP64 arguments.
//
// The error-free transformations are the published ones: Knuth's TwoSum, Dekker's Fast2Sum, and the product's error
// by a fused multiply-add; the sum is the accurate (IEEE-style) float-float addition, the quotient and the square root
// one Newton correction of the FP32 result (Dekker 1971; the double-word algorithms of Joldes, Muller and Popescu,
// ACM TOMS 44(2), 2017).
#pragma once
#include "vp_math.cuh"

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr ff(float h) : hi(h), lo(0.f) {}
    __host__ __device__ constexpr ff(int h) : hi(float(h)), lo(0.f) {}
    // constants: the split of a double (at compile time for literals)
    __host__ __device__ constexpr ff(double d) : hi(float(d)), lo(float(d - double(float(d)))) {}
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return ff(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
    const float s = a + b;
    return ff(s, b - (s - a));
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    const ff t = ff_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = ff_fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ff operator/(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    const ff r = a - b * ff(q1);
    const float q2 = r.hi / b.hi;
    return ff_fast_two_sum(q1, q2);
}
__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { return a = a - b; }
__device__ __forceinline__ bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(ff a, ff b) { return b < a; }
__device__ __forceinline__ bool operator<=(ff a, ff b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(ff a, ff b) { return !(a < b); }
__device__ __forceinline__ ff fabs(ff a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ float ff_f(ff a) { return a.hi + a.lo; }
__device__ __forceinline__ ff vsqrt(ff a) {
    const float x = sqrtf(a.hi);
    if (!(x > 0.f)) return ff(x);
    const float p = x * x;
    const float e = fmaf(x, x, -p);  // x^2 = p + e exactly
    const float r = ((a.hi - p) - e + a.lo) / (2.f * x);
    return ff_fast_two_sum(x, r);
}
__device__ __forceinline__ ff vacos(ff a) { return ff(acosf(ff_f(a))); }
template <> __host__ __device__ __forceinline__ ff vp_pi<ff>() { return ff(3.141592653589793238462643383279502884); }

// the scalar functions of the exact kernel for float-float arguments: the square root and the quotient in
// float-float; log, log1p and atan2 the FP32 functions of the rounded argument (relative error ~1e-7, as for the
// FP32 points). A value outside FP32's comfortable range makes the evaluation give up (ok = false), and the caller
// takes the point in FP64.
struct KMathFF {
    static constexpr bool hybrid = true;
    static __device__ __forceinline__ ff sqrt(ff x) { return vsqrt(x); }
    static __device__ __forceinline__ ff div(ff a, ff b) { return a / b; }
    static __device__ __forceinline__ ff log(ff x) { return ff(logf(ff_f(x))); }
    static __device__ __forceinline__ ff log1p(ff x) { return ff(log1pf(ff_f(x))); }
    static __device__ __forceinline__ ff atan2(ff y, ff x) { return ff(atan2f(ff_f(y), ff_f(x))); }
};

__device__ __forceinline__ v3<float> f3(v3<ff> v) { return mk3(ff_f(v.x), ff_f(v.y), ff_f(v.z)); }
__device__ __forceinline__ bool ff_ok(ff v) { return fabsf(v.hi) < 1e30f; }
