// mk_probe.cu -- FMA throughput probes: the FP64 and FP32 ALU peaks the
// integrator's roofline is reported against (the measured-peak file holds
// HBM and tensor figures only).  Each thread runs 8 independent FMA chains;
// the grid fills every SM.
#include "mk_common.cuh"

namespace mk {

template <typename T>
__global__ void fma_probe_kernel(int64_t iters, T seed, T *out) {
    T a0 = seed + threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T m = T(0.999999), c = T(1e-7);
    for (int64_t i = 0; i < iters; i++) {
        a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
        a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
    }
    const T s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == T(-12345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace mk

using namespace mk;

// Launches the probe: blocks x threads threads, iters x 8 FMAs each.
// precision: MK_FP64 or MK_MIXED (= FP32).  out_dev: blocks*threads
// elements of the chosen type (written only in a case that never occurs).
extern "C" int mk_probe_fma(int32_t precision, int32_t blocks, int32_t threads, int64_t iters, void *out_dev,
                            void *stream) {
    MK_REQUIRE(out_dev && blocks > 0 && threads > 0 && threads <= 1024 && iters > 0, MK_ERR_ARG,
               "mk_probe_fma: bad arguments");
    if (precision == MK_FP64)
        fma_probe_kernel<double><<<blocks, threads, 0, as_stream(stream)>>>(iters, 1.0, (double *)out_dev);
    else
        fma_probe_kernel<float><<<blocks, threads, 0, as_stream(stream)>>>(iters, 1.0f, (float *)out_dev);
    MK_LAUNCHED("fma_probe_kernel");
    return MK_OK;
}
