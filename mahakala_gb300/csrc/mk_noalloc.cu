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
// Its device address is looked up by the first call on a device, with that
// device current, and cached per device together with the id of the CUDA
// context it was looked up in; a call that finds another context current
// (the primary context was reset and re-created) looks the address up
// again.  Make the first call on a device before any stream capture begins.
// All calls share the one array: the header the launches count with is
// cleared on every call, and calls that overlap on the GPU (two streams, or
// two threads) race on it.
#include <cuda.h>

#include <mutex>

#include "mk_common.cuh"

namespace mk {

static __device__ __align__(256) unsigned char g_noalloc_ws[MK_NOALLOC_WORKSPACE_BYTES];

static std::mutex g_noalloc_mutex;
struct NoallocSlot {
    void *addr = nullptr;
    unsigned long long ctx_id = 0;
};
static NoallocSlot g_noalloc_slot[64];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// id of the calling thread's current CUDA context (0 when none is current),
// through the driver entry points the runtime hands out
static int current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        MK_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
        MK_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
        MK_REQUIRE(q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess && f1 && f2, MK_ERR_CUDA,
                   "mk_render_noalloc: the driver does not provide cuCtxGetCurrent / cuCtxGetId");
        get_current = (CtxGetCurrentFn)f1;
        get_id = (CtxGetIdFn)f2;
    }
    CUcontext ctx = nullptr;
    MK_REQUIRE(get_current(&ctx) == CUDA_SUCCESS, MK_ERR_CUDA, "mk_render_noalloc: cuCtxGetCurrent failed");
    *id = 0;
    if (ctx) MK_REQUIRE(get_id(ctx, id) == CUDA_SUCCESS, MK_ERR_CUDA, "mk_render_noalloc: cuCtxGetId failed");
    return MK_OK;
}

static int noalloc_address(void **out) {
    int dev = 0;
    MK_CUDA(cudaGetDevice(&dev));
    MK_REQUIRE(dev >= 0 && dev < 64, MK_ERR_LIMIT, "mk_render_noalloc: device ordinal %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocSlot &slot = g_noalloc_slot[dev];
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc != MK_OK) return rc;
    if (!slot.addr || id == 0 || id != slot.ctx_id) {
        // set-up: the device's address of the array, looked up with the
        // device current (this also makes the runtime's context current)
        void *p = nullptr;
        MK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_ws));
        MK_REQUIRE(p != nullptr, MK_ERR_CUDA, "mk_render_noalloc: no device address for the scratch array");
        if ((rc = current_context_id(&id)) != MK_OK) return rc;
        slot.addr = p;
        slot.ctx_id = id;
    }
    *out = slot.addr;
    return MK_OK;
}

}  // namespace mk

extern "C" int mk_render_noalloc(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
                                 const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision,
                                 void *stream) {
    MK_REQUIRE(total_rays >= 0, MK_ERR_ARG, "mk_render_noalloc: negative ray count");
    // the render needs the counter header and the ray queues; the optional
    // camera-state region of mk_render_workspace_bytes is used only when it
    // fits in what is left
    const size_t need = mk::render_ws_base(total_rays, precision);
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
