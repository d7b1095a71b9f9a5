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

// Float unit approximations (PTX rsqrt.approx.ftz / rcp.approx.ftz, ~2 ulp)
// with subnormal inputs and results flushed to zero: the float geodesic's
// arguments (r^2, Q ~ r^4, (r^4 + a^2 z^2)(r^2 + a^2), the step rule's
// divisor) and the emission's are normal numbers, or give a zero emission
// either way, so the flush changes nothing and saves the subnormal handling.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ------------------------------------------------------------------------
// Binary64 reciprocal square root and reciprocal for the FP64 path, whose
// time is its FP64-pipe instruction count (1/64 of the FP32 rate on this
// part).  The seed is the float unit's approximation (rsqrt_ftz, rcp_ftz)
// of the argument moved to float and back by bit operations on the integer
// pipe -- exponent rebased between the two formats, significand truncated
// to 23 bits -- so only the correction runs on the FP64 pipe.  One
// third-order correction (Householder's method of order 3: the binomial
// series (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 + O(e^3) and (1 - e)^(-1) =
// 1 + e + e^2 + O(e^3), e the seed's residual, |e| < 2^-20) leaves a
// truncation below 2^-58; with the correction's own roundings the result
// is within 2 ulp of the exact value (tests/test_gpu_math.py checks it
// against the correctly rounded library forms).  Arguments whose binary
// exponent lies outside [-120, 119] -- zero, subnormals, negative values,
// infinities and NaN included -- take the library forms.

// |x| with biased exponent in [903, 1142] -> float with the same value,
// significand truncated (positive x only)
__device__ __forceinline__ float f32_bits_of(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    return __uint_as_float(((hi - (896u << 20)) << 3) | (lo >> 29));
}

// positive normal float -> the same value as a double, with the sign bit
// `sign` (0 or 0x80000000)
__device__ __forceinline__ double f64_bits_of(float y, unsigned sign = 0u) {
    const unsigned u = __float_as_uint(y);
    return __hiloint2double((int)(((u >> 3) + (896u << 20)) | sign), (int)(u << 29));
}

// biased exponent of the high word hi (sign included) in [903, 1142]
__device__ __forceinline__ bool f64_seed_range(unsigned hi) { return (hi >> 20) - 903u <= 239u; }

__device__ __forceinline__ double rsqrt64(double x) {
    if (f64_seed_range((unsigned)((unsigned long long)__double_as_longlong(x) >> 32))) {
        const double y = f64_bits_of(rsqrt_ftz(f32_bits_of(x)));
        const double e = fma(-(x * y), y, 1.0);          // 1 - x y^2
        return fma(y * e, fma(0.375, e, 0.5), y);        // y (1 + e/2 + 3e^2/8)
    }
    return 1.0 / sqrt(x);
}

// sqrt(x) = x / sqrt(x), from rsqrt64 where its seed applies (exact
// library form elsewhere: zero, subnormals, infinities, NaN)
__device__ __forceinline__ double sqrt64(double x) {
    if (f64_seed_range((unsigned)((unsigned long long)__double_as_longlong(x) >> 32))) return x * rsqrt64(x);
    return sqrt(x);
}

__device__ __forceinline__ double rcp64(double d) {
    const unsigned hi = (unsigned)((unsigned long long)__double_as_longlong(d) >> 32);
    if (f64_seed_range(hi & 0x7fffffffu)) {
        const double a = __hiloint2double((int)(hi & 0x7fffffffu), __double2loint(d));  // |d|
        const double y = f64_bits_of(rcp_ftz(f32_bits_of(a)), hi & 0x80000000u);
        const double e = fma(-d, y, 1.0);                  // 1 - d y
        return fma(y, fma(e, e, e), y);                    // y (1 + e + e^2)
    }
    return 1.0 / d;
}

// 1/sqrt for each arithmetic the geodesic code is instantiated with
__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt(double x) { return rsqrt64(x); }

__host__ __device__ __forceinline__ double to_double(dd x) { return x.to_double(); }
__host__ __device__ __forceinline__ double to_double(double x) { return x; }
__host__ __device__ __forceinline__ float to_float(dd x) { return x.hi; }
__host__ __device__ __forceinline__ float to_float(double x) { return (float)x; }
__host__ __device__ __forceinline__ float to_float(float x) { return x; }

}  // namespace mk
