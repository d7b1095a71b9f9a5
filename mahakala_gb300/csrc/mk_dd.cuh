// mk_dd.cuh -- double-float arithmetic: a value is an unevaluated sum
// hi + lo of two floats (|lo| <= ulp(hi)/2), about 44-48 significant bits.
//
// Used by the mixed form's "df" variant for the near-horizon region, where
// the FP64 pipe (1/64 of FP32 on GB300) makes a few hundred serial FP64
// steps the critical path.  Published methods, written from their
// definitions:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and FastTwoSum (Dekker 1971) for
//   error-free addition; TwoProd by one fused multiply-add (the error of a
//   float product is exactly fma(a, b, -a*b)); division by one residual
//   correction of the float quotient; reciprocal square root by one Newton
//   step y <- y + y (1 - x y^2) / 2 on the float estimate.
// None of these steps may be reassociated or contracted; nvcc does neither
// without fast-math, and every product that must fuse is an explicit fmaf.
// This is not IEEE binary64: results carry ~1e-13 relative error.
#pragma once

#include <math.h>

namespace mk {

struct dd {
    float hi, lo;
    dd() = default;
    __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit constexpr dd(float h) : hi(h), lo(0.0f) {}
    __host__ __device__ explicit constexpr dd(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
};

__host__ __device__ __forceinline__ dd dd_two_sum(float a, float b) {
    const float s = a + b;
    const float v = s - a;
    return dd(s, (a - (s - v)) + (b - v));
}

__host__ __device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
    const float s = a + b;
    return dd(s, b - (s - a));
}

__host__ __device__ __forceinline__ dd operator+(dd x, dd y) {
    dd s = dd_two_sum(x.hi, y.hi);
    const dd t = dd_two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = dd_fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return dd_fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ dd operator-(dd x) { return dd(-x.hi, -x.lo); }
__host__ __device__ __forceinline__ dd operator-(dd x, dd y) { return x + (-y); }

__host__ __device__ __forceinline__ dd operator*(dd x, dd y) {
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return dd_fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ dd operator/(dd x, dd y) {
    const float q1 = x.hi / y.hi;
    const dd r = x - y * dd(q1, 0.0f);
    const float q2 = r.hi / y.hi;
    return dd_fast_two_sum(q1, q2);
}

__host__ __device__ __forceinline__ dd inv_sqrt(dd x) {
#ifdef __CUDA_ARCH__
    const float y = rsqrtf(x.hi);
#else
    const float y = 1.0f / sqrtf(x.hi);
#endif
    const dd yy(y, 0.0f);
    const dd e = dd(1.0f, 0.0f) - x * yy * yy;
    return yy + yy * e * dd(0.5f, 0.0f);
}

// 1/sqrt for each arithmetic the geodesic code is instantiated with
__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt(double x) { return ::rsqrt(x); }

__host__ __device__ __forceinline__ double to_double(dd x) { return x.to_double(); }
__host__ __device__ __forceinline__ double to_double(double x) { return x; }
__host__ __device__ __forceinline__ float to_float(dd x) { return x.hi; }
__host__ __device__ __forceinline__ float to_float(double x) { return (float)x; }
__host__ __device__ __forceinline__ float to_float(float x) { return x; }

}  // namespace mk
