// mk_noalloc.cu -- mk_render without a caller-provided workspace.
//
// Some hosts cannot hand this library scratch memory: a plugin living
// inside another framework's fixed device-memory pool, a caller that must
// not trigger cudaMalloc (it can synchronise the device or fail outright
// under that host's allocation policy), or C code that only holds the
// request, snapshot and image buffers it was given.  For them the render's
// scratch -- the launch counters and, in the mixed forms, the two ray
// queues -- lives in one static device array of this file, sized once at
// compile time (MK_NOALLOC_WORKSPACE_BYTES).  Every GPU that loads the
// library holds that array until the process exits.
//
// Its device address is looked up once per device, with that device
// current, by the first call on that device; make that first call before
// any stream capture begins.  All calls share the one array: the header
// the launches count with is cleared on every call, and calls that
// overlap on the GPU (two streams, or two threads) race on it.
#include <mutex>

#include "mk_common.cuh"

namespace mk {

static __device__ __align__(256) unsigned char g_noalloc_ws[MK_NOALLOC_WORKSPACE_BYTES];

static std::mutex g_noalloc_mutex;
static void *g_noalloc_addr[64] = {nullptr};

static int noalloc_address(void **out) {
    int dev = 0;
    MK_CUDA(cudaGetDevice(&dev));
    MK_REQUIRE(dev >= 0 && dev < 64, MK_ERR_LIMIT, "mk_render_noalloc: device ordinal %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        MK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_ws));
        MK_REQUIRE(p != nullptr, MK_ERR_CUDA, "mk_render_noalloc: no device address for the scratch array");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return MK_OK;
}

}  // namespace mk

extern "C" int mk_render_noalloc(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
                                 const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision,
                                 void *stream) {
    MK_REQUIRE(total_rays >= 0, MK_ERR_ARG, "mk_render_noalloc: negative ray count");
    const size_t need = mk_render_workspace_bytes(total_rays, precision);
    MK_REQUIRE(need <= (size_t)MK_NOALLOC_WORKSPACE_BYTES, MK_ERR_LIMIT,
               "mk_render_noalloc: %lld rays need %zu bytes of scratch at precision %d, above the %zu-byte "
               "static workspace (at most %lld rays in the mixed forms); use mk_render with a caller workspace",
               (long long)total_rays, need, (int)precision, (size_t)MK_NOALLOC_WORKSPACE_BYTES,
               (long long)MK_NOALLOC_MAX_MIXED_RAYS);
    void *ws = nullptr;
    const int rc = mk::noalloc_address(&ws);
    if (rc != MK_OK) return rc;
    // mk_render clears the counter header at the start of every launch
    return mk_render(reqs_dev, nreq, total_rays, snaps_dev, nsnap, precision, ws, MK_NOALLOC_WORKSPACE_BYTES,
                     stream);
}
