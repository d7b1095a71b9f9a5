/* A C host of the library: includes the public header as C11, links
   libmahakala_gb300.so and calls the entry points that need no GPU -- the
   version queries, the workspace size, the struct layouts as this C
   compiler lays them out against the library's own, and argument
   validation, which runs before any CUDA call.  Prints "ok" or the first
   mismatch. */
#include <stdio.h>
#include <string.h>

#include "mahakala_gb300.h"

#define CHECK(cond, what)                          \
    do {                                           \
        if (!(cond)) {                             \
            printf("mismatch: %s\n", what);        \
            return 1;                              \
        }                                          \
    } while (0)

int main(void) {
    CHECK(mk_abi_version() == 1, "abi version");
    CHECK(strstr(mk_version(), "sm_103a") != NULL, "version string names sm_103a");
    CHECK(mk_sizeof("mk_request") == sizeof(mk_request), "sizeof mk_request");
    CHECK(mk_sizeof("mk_camera") == sizeof(mk_camera), "sizeof mk_camera");
    CHECK(mk_sizeof("mk_step_policy") == sizeof(mk_step_policy), "sizeof mk_step_policy");
    CHECK(mk_sizeof("mk_snapshot_view") == sizeof(mk_snapshot_view), "sizeof mk_snapshot_view");
    CHECK(mk_sizeof("mk_mesh_desc") == sizeof(mk_mesh_desc), "sizeof mk_mesh_desc");
    CHECK(mk_sizeof("no_such_struct") == 0, "unknown struct name");
    CHECK(mk_render_workspace_bytes(100, MK_FP64) == 256, "FP64 workspace is the counter header");
    CHECK(mk_render(NULL, 1, 10, NULL, 1, MK_FP64, NULL, 256, NULL) == MK_ERR_ARG, "null arguments refused");
    CHECK(strstr(mk_last_error(), "null") != NULL, "last error names the null argument");
    CHECK(mk_set_tuning("no_such_switch", 1) == MK_ERR_ARG, "unknown tuning switch refused");
    printf("ok\n");
    return 0;
}
