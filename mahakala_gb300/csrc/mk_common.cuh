// mk_common.cuh -- host-side helpers shared by the C-ABI translation units:
// per-thread last-error message, argument checks, launch checks.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "mahakala_gb300.h"

namespace mk {

void set_error(const char *fmt, ...);
int device_sm_count();
// scratch bytes mk_render cannot do without: the counter header and, in the
// mixed forms, the two ray queues (mk_render_workspace_bytes may add an
// optional camera-state region on top)
size_t render_ws_base(int64_t rays, int32_t precision);

#define MK_REQUIRE(cond, code, ...)        \
    do {                                   \
        if (!(cond)) {                     \
            ::mk::set_error(__VA_ARGS__);  \
            return (code);                 \
        }                                  \
    } while (0)

#define MK_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            ::mk::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                            __FILE__, __LINE__);                                        \
            return MK_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)

#define MK_LAUNCHED(name)                                                               \
    do {                                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess) {                                                        \
            ::mk::set_error("launch of %s failed: %s", name, cudaGetErrorString(e_));   \
            return MK_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace mk
