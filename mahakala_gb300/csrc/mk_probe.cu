// mk_probe.cu -- FMA throughput probes: the FP64 and FP32 ALU peaks the
// integrator's roofline is reported against (the measured-peak file holds
// HBM and tensor figures only).  Each thread runs 8 independent FMA chains
// over an int32 loop counter unrolled 16 times, so the loop's own compare
// and increment take a negligible share of the issue slots; the grid fills
// every SM.  A third probe runs the chains on Blackwell's paired FP32 FMA
// (two FMAs per instruction), which shows whether the FP32 figure was
// bound by issue or by the pipe.
#include "mk_common.cuh"
#include "mk_dd.cuh"

namespace mk {

template <typename T>
__global__ void fma_probe_kernel(int iters, T seed, T *out) {
    T a0 = seed + threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T m = T(0.999999), c = T(1e-7);
#pragma unroll 16
    for (int i = 0; i < iters; i++) {
        a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
        a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
    }
    const T s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == T(-12345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

// 8 independent chains of paired FP32 FMAs (16 FMAs per iteration)
__global__ void ffma2_probe_kernel(int iters, float seed, float *out) {
    float2 a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = make_float2(seed + threadIdx.x + 2 * k, seed + threadIdx.x + 2 * k + 1);
    const float2 m = make_float2(0.999999f, 0.999999f), c = make_float2(1e-7f, 1e-7f);
#pragma unroll 16
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = __ffma2_rn(a[k], m, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k].x + a[k].y;
    if (s == -12345.0f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// the FP64 path's reciprocal square root, reciprocal and square root beside
// the library's correctly rounded forms, element by element
__global__ void math_probe_kernel(int fn, const double *__restrict__ x, long long n, double *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = x[i];
        double r;
        switch (fn) {
            case MK_MATH_RSQRT: r = rsqrt64(v); break;
            case MK_MATH_RCP: r = rcp64(v); break;
            case MK_MATH_SQRT: r = sqrt64(v); break;
            case MK_MATH_LIB_RSQRT: r = 1.0 / __dsqrt_rn(v); break;
            case MK_MATH_LIB_RCP: r = __drcp_rn(v); break;
            default: r = __dsqrt_rn(v); break;
        }
        out[i] = r;
    }
}

}  // namespace mk

using namespace mk;

extern "C" int mk_probe_math(int32_t fn, const double *x_dev, int64_t n, double *out_dev, void *stream) {
    MK_REQUIRE(fn >= MK_MATH_RSQRT && fn <= MK_MATH_LIB_SQRT, MK_ERR_ARG, "mk_probe_math: unknown function %d",
               (int)fn);
    MK_REQUIRE(n >= 0 && (n == 0 || (x_dev && out_dev)), MK_ERR_ARG, "mk_probe_math: bad arguments");
    if (n == 0) return MK_OK;
    math_probe_kernel<<<grid_for(n < 65536 ? n : 65536, 256), 256, 0, as_stream(stream)>>>(fn, x_dev, (long long)n,
                                                                                           out_dev);
    MK_LAUNCHED("math_probe_kernel");
    return MK_OK;
}

// Launches the probe: blocks x threads threads, iters x 8 FMAs each (x 16
// for MK_PROBE_FFMA2).  kind: MK_FP64, MK_MIXED (= FP32) or MK_PROBE_FFMA2.
// out_dev: blocks*threads elements of the chosen type (written only in a
// case that never occurs).
extern "C" int mk_probe_fma(int32_t precision, int32_t blocks, int32_t threads, int64_t iters, void *out_dev,
                            void *stream) {
    MK_REQUIRE(out_dev && blocks > 0 && threads > 0 && threads <= 1024 && iters > 0 && iters <= (1ll << 30),
               MK_ERR_ARG, "mk_probe_fma: bad arguments");
    const cudaStream_t st = as_stream(stream);
    if (precision == MK_FP64)
        fma_probe_kernel<double><<<blocks, threads, 0, st>>>((int)iters, 1.0, (double *)out_dev);
    else if (precision == MK_MIXED)
        fma_probe_kernel<float><<<blocks, threads, 0, st>>>((int)iters, 1.0f, (float *)out_dev);
    else if (precision == MK_PROBE_FFMA2)
        ffma2_probe_kernel<<<blocks, threads, 0, st>>>((int)iters, 1.0f, (float *)out_dev);
    else
        MK_REQUIRE(false, MK_ERR_ARG, "mk_probe_fma: unknown kind %d", (int)precision);
    MK_LAUNCHED("fma_probe_kernel");
    return MK_OK;
}
