// mk_capi.cu -- library-wide C-ABI entry points: version, last error,
// device properties.
#include <string.h>

#include "mk_common.cuh"

namespace mk {

static thread_local char g_last_error[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int device_sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev < 64 && cached[dev]) return cached[dev];
    int sms = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    if (dev < 64) cached[dev] = sms;
    return sms;
}

}  // namespace mk

extern "C" const char *mk_version(void) { return "mahakala_gb300 0.1 (sm_103a)"; }
extern "C" int32_t mk_abi_version(void) { return MK_ABI_VERSION; }
extern "C" const char *mk_last_error(void) { return mk::g_last_error; }
extern "C" int32_t mk_device_sm_count(void) { return mk::device_sm_count(); }

extern "C" size_t mk_sizeof(const char *name) {
    if (!name) return 0;
    if (!strcmp(name, "mk_step_policy")) return sizeof(mk_step_policy);
    if (!strcmp(name, "mk_camera")) return sizeof(mk_camera);
    if (!strcmp(name, "mk_snapshot_view")) return sizeof(mk_snapshot_view);
    if (!strcmp(name, "mk_mesh_desc")) return sizeof(mk_mesh_desc);
    if (!strcmp(name, "mk_request")) return sizeof(mk_request);
    return 0;
}
