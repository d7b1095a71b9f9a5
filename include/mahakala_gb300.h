/*
 * mahakala_gb300.h -- C ABI of the GB300 (sm_103a) per-ray imaging path.
 *
 * Every entry point takes plain pointers and sizes.  Pointers named *_dev
 * are CUDA device pointers owned by the caller; host structs are read
 * during the call only.  `stream` is a cudaStream_t passed as void* (NULL =
 * the legacy default stream).  Work is enqueued on that stream and the call
 * returns without synchronising; results are valid once the stream reaches
 * that point.  Every function returns MK_OK (0) or an mk_status code, and
 * mk_last_error() returns a message for the calling thread's last failure.
 * No function allocates device memory except where its comment says so;
 * scratch space is passed in by the caller (see mk_render_workspace_bytes).
 *
 * The reference is Mahakala (Python + JAX).  Each entry point names the
 * reference function it replaces (file:line within that project).
 */
#ifndef MAHAKALA_GB300_H
#define MAHAKALA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MK_ABI_VERSION 1
#define MK_MAX_NU 4

typedef enum {
    MK_OK = 0,
    MK_ERR_ARG = 1,          /* invalid argument (null pointer, bad size)   */
    MK_ERR_CUDA = 2,         /* a CUDA runtime call or launch failed        */
    MK_ERR_LIMIT = 3,        /* a size exceeds a documented maximum         */
    MK_ERR_UNSUPPORTED = 4,  /* valid request this build does not implement */
    MK_ERR_TIMEOUT = 5       /* a bounded wait inside a kernel ran out: the
                                launch's outputs are invalid (reported in the
                                workspace header word MK_WS_ERROR)          */
} mk_status;

/* per-ray stop reasons (status arrays) */
typedef enum {
    MK_RAY_ACTIVE = 0,
    MK_RAY_CAPTURED = 1,     /* reference rule: r - r_EH < tol; fixed rule: r < capture*r_h */
    MK_RAY_ESCAPED = 2,      /* reference rule: r - r_EH > 1500; fixed rule: outbound r > r_escape */
    MK_RAY_MAXSTEPS = 3,
    MK_RAY_NAN = 4
} mk_ray_status;

/* MK_FP64: every operation in binary64.
   MK_MIXED: FP32 arithmetic (ray state as float pairs, Kahan-compensated
   intensity); near the hole (r < 3 M, or inbound inside 6 M where
   photon-ring rays turn) the wavevector is renormalised to null on entry
   (binary64) and at every radial turning point (double-float pairs, ~1e-13
   relative); accelerations and emission stay FP32.
   MK_MIXED_STRICT: as MK_MIXED, but near the hole the whole geodesic step
   (accelerations included) is binary64.
   MK_MIXED_DF: as MK_MIXED_STRICT with that step in double-float (pairs of
   FP32, ~1e-13 relative) instead of binary64 -- not IEEE FP64.
   The mixed forms end a ray that moves outward beyond the snapshot's
   bounding radius with MK_RAY_ESCAPED: outside the photon region it has no
   radial turning point left, takes no further sample and its intensity is
   final, so the image equals running it on to the reference's stop; its
   nsteps is the steps taken (mk_set_tuning "escape_cut" 0 runs every ray
   to the reference's stop).  MK_FP64 always follows the reference's rule. */
typedef enum { MK_FP64 = 0, MK_MIXED = 1, MK_MIXED_DF = 2, MK_MIXED_STRICT = 3 } mk_precision;

typedef enum {
    /* dt = -(r - r_EH)/div, stop (and reject the step) when the next dt
       would be NaN, |dt|*div < tol or |dt|*div > 1500
       (geodesic_integrator, geodesics.py:246-269) */
    MK_POLICY_REFERENCE = 0,
    /* h = -clamp(hfrac*r, hmin, hmax); captured at r < capture*r_h;
       escaped at r > r_escape once r increases (no reference counterpart) */
    MK_POLICY_FIXED = 1
} mk_policy_kind;

typedef enum { MK_CAMERA_GRID = 0, MK_CAMERA_EQUATOR = 1 } mk_camera_kind;

typedef struct {
    int32_t kind;            /* mk_policy_kind */
    int32_t nmax;            /* N, the maximum number of steps */
    double div, tol;         /* MK_POLICY_REFERENCE */
    double hfrac, hmin, hmax, capture, r_escape; /* MK_POLICY_FIXED */
} mk_step_policy;

/* camera of initialize_geodesics_at_camera (geodesics.py:29-55, 137-216).
   cos_inc/sin_inc: cos and sin of inclination*pi/180, as the host's libm
   evaluates them (geodesics.py:205). */
typedef struct {
    int32_t kind;            /* mk_camera_kind */
    int32_t pixels;          /* pixels per side (grid) or along the line (equator) */
    double bhspin, cos_inc, sin_inc, distance, fov_lower, fov_upper;
} mk_camera;

/* Device view of one resident snapshot (meshblocks with one ghost layer,
   AoS float32 [mb][k][j][i][prim], prim order dens, velx, vely, velz, eint,
   bcc1, bcc2, bcc3), single- or multi-level.  Filled by mk_snapshot_build;
   plain data, copyable. */
typedef struct {
    const float *blocks;     /* (nmb, n+2, n+2, n+2, 8) */
    const double *geom;      /* (nmb, 6): x1v[0], x2v[0], x3v[0], dx1, dx2, dx3 per block */
    const float *geom_f32;   /* (nmb, 8): x1v[0], x2v[0], x3v[0], 1/dx1, 1/dx2, 1/dx3, 0, 0 (mixed form) */
    const double *faces;     /* (nmb, 6): x1f[0], x1f[n], x2f[0], x2f[n], x3f[0], x3f[n] per block */
    const int32_t *table;    /* (nb[2], nb[1], nb[0]) block covering each cell of the finest-level
                                block grid, -1 where no block is */
    const double *blocks64;  /* (n64, n+2, n+2, n+2, 8) binary64 copies of the blocks whose ghost
                                cells average finer cells (their means are not float32 values), or
                                NULL when no block has such ghosts */
    const int32_t *block64;  /* (nmb) row of blocks64 for each block or -1; NULL with blocks64 */
    int32_t nmb, n;
    int32_t nb[3], pad0;
    double lo[3], width[3];  /* first face and finest block width per axis */
} mk_snapshot_view;

/* Key of a block in a mesh's sorted key list: level and logical location
   (i, j, k), each location < 2^18, level < 2^9. */
#define MK_MESH_KEY(level, i, j, k)                                                                   \
    (((int64_t)(level) << 54) | ((int64_t)(i) << 36) | ((int64_t)(j) << 18) | (int64_t)(k))

/* A mesh for mk_snapshot_build (device pointers, kept by reference except
   uov/B/locs/levels/keys, which are read only during the build). */
typedef struct {
    const float *uov;        /* (5, nmb, n, n, n) float32: dens, velx, vely, velz, eint */
    const float *B;          /* (3, nmb, n, n, n) float32: bcc1..3 */
    const int32_t *locs;     /* (nmb, 3) logical locations (i, j, k) at each block's level */
    const int32_t *levels;   /* (nmb) refinement levels */
    const int64_t *keys;     /* (nmb) MK_MESH_KEY of every block, ascending */
    const int32_t *key_block;/* (nmb) block of each sorted key */
    const double *geom;      /* as mk_snapshot_view.geom */
    const double *faces;     /* as mk_snapshot_view.faces */
    const int32_t *table;    /* as mk_snapshot_view.table */
    double *blocks64;        /* storage for n64 binary64 blocks, or NULL (n64 = 0) */
    const int32_t *block64;  /* (nmb) row of blocks64 or -1, or NULL */
    int32_t nmb, n, n64, pad0;
    int32_t nb[3], pad1;
    double lo[3], width[3];
} mk_mesh_desc;

/* One render request: the arguments of make_image (images.py:30-35) after
   the host-side scalar prologue (units, grmhd/grmhd.py:40-55). */
typedef struct {
    mk_camera camera;
    mk_step_policy policy;
    double fluid_gamma, r_low, r_high;
    double electron_gamma_m1, ion_gamma_m1;  /* electron_gamma - 1., ion_gamma - 1. */
    double Ne_unit, B_unit, L_unit;
    double cos_fallback_pitch;               /* cos(fallback pitch angle) */
    double sigma_cut;                        /* images.py:116 */
    int32_t nnu, snapshot;                   /* frequencies; index into the snapshot array */
    double nu[MK_MAX_NU];                    /* observing frequencies (Hz) */
    double *image;                           /* (nnu, npx) device output, specific intensity */
    int32_t *nsteps;                         /* (npx) device output or NULL */
    int32_t *status;                         /* (npx) device output or NULL */
    int64_t ray_offset;                      /* first global ray of this request */
    /* Per-step diagnostics, MK_FP64 only (NULL to skip): for trajectory row
       i (1 <= i < rows) of each ray, rows_em/rows_ab (nnu, rows, npx)
       receive the invariant emissivity and absorptivity of the sample
       there (after the sigma cut; 0 outside the snapshot) and rows_dt
       (rows, npx) the step size dt of row i-1 -> i at index i-1: the
       arrays solve_specific_intensity (dIs) and solve_attenuated_emissivity
       (transfer.py:89-144) take.  Rows after a ray stops are not written:
       zero them first (the reference's frozen rows carry dt = 0). */
    double *rows_em, *rows_ab, *rows_dt;
    int64_t rows;
} mk_request;

/* ---------------------------------------------------------------- misc */
const char *mk_version(void);
int32_t mk_abi_version(void);
const char *mk_last_error(void);
/* number of SMs of the current device (for callers sizing their own grids) */
int32_t mk_device_sm_count(void);
/* sizeof of a public struct by name ("mk_request", ...), 0 if unknown; lets
   a binding check its struct layout against the library's */
size_t mk_sizeof(const char *name);

/* ------------------------------------------------------------- camera */
/* initialize_geodesics_at_camera (geodesics.py:29-55) incl. get_initial_grid
   (:137-216) and initial_condition/_Nullify (:58-85, 219-230).
   s0_dev: (npx, 8) with npx = pixels^2 (grid) or pixels (equator); pixel
   index ix*pixels + iy as meshgrid(indexing='ij') orders it. */
int mk_camera_init(const mk_camera *camera, double *s0_dev, void *stream);

/* get_camera_pixel (geodesics.py:107-134) + initial_condition: image-plane
   points (x_dev[i], y_dev[i]) -> s0_dev (n, 8). */
int mk_camera_points(const double *x_dev, const double *y_dev, int64_t n, double bhspin,
                     double cos_inc, double sin_inc, double distance, double *s0_dev,
                     void *stream);

/* ---------------------------------------------------------- geodesics */
/* geodesic_integrator (geodesics.py:233-281) with RK4_gen (:317-336) and
   the closed-form Kerr-Schild Christoffel contraction in place of
   rhs/jacfwd/inv (:294-347).
   MK_POLICY_REFERENCE: rows_dev (nmax, npx, 8) and dt_dev (nmax, npx), if
   not NULL, receive the reference's trajectory rows (row i = state before
   step i; rows after a ray stops repeat its frozen state with dt 0).
   K_dev (npx) gets the first stopped step (nmax if none), why_dev the
   mk_ray_status reason, state_dev (npx, 8) the state after K steps.
   MK_POLICY_FIXED: rows/dt must be NULL; K_dev gets the steps taken and
   state_dev the final state. */
int mk_integrate(const double *s0_dev, int64_t npx, double bhspin, const mk_step_policy *policy,
                 double *rows_dev, double *dt_dev, int32_t *K_dev, int32_t *why_dev,
                 double *state_dev, void *stream);

/* radius_cal (geodesics.py:284-291) on npts points of stride `stride` doubles */
int mk_radius_cal(const double *x_dev, int64_t npts, int64_t stride, double bhspin,
                  double *r_dev, void *stream);

/* One bisection pass of find_shadow_bisection_angles (geodesics.py:405-435):
   integrates the polar-camera rays at radii mid_dev (n) with the reference
   rule (div 40, tol 1e-2, max_steps) and writes per ray what
   select_photons_integrator (:354-378) needs: K (first stopped step),
   best (argmax of dt over the accepted steps, -1 if none), best_dt, and
   radius_cal at rows K-1, best-1 and at the last row. */
int mk_shadow_pass(const double *cos_dev, const double *sin_dev, const double *mid_dev, int64_t n,
                   double bhspin, double cos_inc, double sin_inc, double distance, int32_t max_steps,
                   int32_t *K_dev, int32_t *best_dev, double *best_dt_dev, double *r_km1_dev,
                   double *r_best_dev, double *r_last_dev, void *stream);

/* --------------------------------------------------------- snapshots */
/* Bytes of device storage mk_snapshot_build needs for nmb blocks of n^3. */
size_t mk_snapshot_bytes(int32_t nmb, int32_t n);

/* Builds the ghost-filled AoS meshblocks on the device from AthenaK arrays
   (load_athenak_meshblocks, grmhd/athenak.py:67-158 with the multi-level
   ghost fill of :160-525): a ghost region takes the same-level neighbour's
   cells, else the coarser neighbour's (each coarse cell copied to the fine
   ghosts it covers), else the mean of the finer neighbours' 2x2x2 cells
   summed in binary64 in the reference's term order (including its first
   edge term, which reads one cell), else zero.  Means are stored rounded to
   float32 in `blocks` and exactly in `blocks64` for the FP64 path.  storage
   >= mk_snapshot_bytes(nmb, n), 16-byte aligned. */
int mk_snapshot_build(const mk_mesh_desc *mesh, void *storage_dev, size_t storage_bytes,
                      mk_snapshot_view *view_out, void *stream);

/* ------------------------------------------------------ stage kernels */
/* get_fluid_scalars_from_geodesics (grmhd/athenak.py:639-812): for npts
   points S_dev (npts, 8) -> out_dev (npts, 5) = dens, u, pitch_angle,
   kdotu, b.  cos_fallback = cos(fallback_pitch_angle). */
int mk_fluid_scalars(const mk_snapshot_view *view, double bhspin, const double *S_dev,
                     int64_t npts, double cos_fallback, double *out_dev, void *stream);

/* get_prims_from_geodesics (grmhd/athenak.py:527-637): out_dev (npts, 8) in
   the order dens, velx, vely, velz, eint, bcc1..3; block_dev (npts) the
   meshblock of each point (-1 outside) or NULL. */
int mk_fluid_prims(const mk_snapshot_view *view, const double *S_dev, int64_t npts,
                   double *out_dev, int32_t *block_dev, void *stream);

/* rlow_rhigh_model (electrons.py:32-50) */
int mk_rlow_rhigh(const double *dens_dev, const double *u_dev, const double *beta_dev, int64_t n,
                  double r_low, double r_high, double electron_gamma_m1, double ion_gamma_m1,
                  double *theta_dev, void *stream);

/* synchrotron_coefficients (transfer.py:30-86) */
int mk_synchrotron(const double *Ne_dev, const double *theta_dev, const double *B_dev,
                   const double *pitch_dev, const double *nu_dev, int64_t n, int32_t invariant,
                   double rescale_nu, double *em_dev, double *ab_dev, void *stream);

/* solve_specific_intensity (transfer.py:89-119) on (nsteps, npx) arrays;
   dIs_dev (nsteps-1, npx) or NULL (row r is step nsteps-1-r) */
int mk_solve_intensity(const double *em_dev, const double *ab_dev, const double *dt_dev,
                       int64_t nsteps, int64_t npx, double L_unit, double *I_dev, double *dIs_dev,
                       void *stream);

/* solve_attenuated_emissivity (transfer.py:122-144); out_dev (nsteps-1, npx) */
int mk_attenuated_emissivity(const double *em_dev, const double *ab_dev, const double *dt_dev,
                             int64_t nsteps, int64_t npx, double L_unit, double *out_dev,
                             void *stream);

/* ------------------------------------------------------- fused render */
/* Scratch bytes mk_render needs in workspace_dev for total_rays rays at
   the given precision: a 256-byte header of counters (MK_FP64), plus two
   ray queues of total_rays 160-byte records each for the hand-offs between
   the phases (mixed forms), plus -- when total_rays is more than one wave
   of the FP32 phase on the current device (4 blocks of 128 threads per SM)
   -- 64 bytes a ray for camera states computed ahead of it.  A workspace of
   at least the size without that last part also renders (the FP32 phase
   then computes the camera states itself, more slowly).  The caller
   allocates it (16-byte aligned) and may reuse it for calls that do not
   overlap on the device.
   After a launch the header holds, as uint64 at these word offsets, the
   launch's totals: MK_WS_STEPS accepted RK4 steps, MK_WS_SAMPLES
   in-snapshot samples, MK_WS_MAX_TAU the bits of a double, the largest
   per-step optical depth w*alpha of the transfer solve (the reference's
   explicit Euler update is stable below 1), MK_WS_TO_FP64 rays handed to
   the near-hole phase, MK_WS_TO_FP32 rays that left it outward,
   MK_WS_FP32_QUEUE rays in the FP32 continuation queue (MK_MIXED: rays
   parked leaving the photon-ring region outward; the other mixed forms:
   the near-hole phase's exits), MK_WS_STEPS_FP64 steps and
   MK_WS_SAMPLES_FP64 in-snapshot samples taken near the hole (mixed
   forms), MK_WS_ZONE_RUN_MAX the most steps one ray took in one visit to
   the near-hole phase (MK_MIXED; its serial chain), MK_WS_STEPS_B /
   MK_WS_SAMPLES_B the steps and samples MK_MIXED's near-hole kernel took
   (near the hole and after), MK_WS_STEPS_C / MK_WS_SAMPLES_C those the
   FP32 continuation kernel took (mixed forms), MK_WS_ERROR the waits of
   MK_MIXED's near-hole pipeline that ran out (each bounded by the
   "zone_wait_ns" tuning): nonzero means the launch's images are invalid,
   and a host reads it as status MK_ERR_TIMEOUT once the stream has passed
   the launch. */
#define MK_WS_STEPS 1
#define MK_WS_SAMPLES 2
#define MK_WS_MAX_TAU 3
#define MK_WS_TO_FP64 4
#define MK_WS_FP32_QUEUE 6
#define MK_WS_TO_FP32 14
#define MK_WS_STEPS_FP64 8
#define MK_WS_SAMPLES_FP64 10
#define MK_WS_ZONE_RUN_MAX 11
/* Requests one mixed-form launch takes (mk_render refuses more with
   MK_ERR_LIMIT; rays of requests beyond it in an mk_render_job header end
   with MK_RAY_NAN). */
#define MK_MAX_REQUESTS_MIXED 128
#define MK_WS_STEPS_B 12
#define MK_WS_SAMPLES_B 13
#define MK_WS_STEPS_C 15
#define MK_WS_SAMPLES_C 16
#define MK_WS_ERROR 17
size_t mk_render_workspace_bytes(int64_t total_rays, int32_t precision);

/* make_image (images.py:30-144) for nreq requests in ONE persistent launch
   (three in the mixed forms: FP32 from the camera, then the near-hole
   phase and the FP32 continuation -- MK_MIXED runs these two at the same
   time, the second on a per-thread side stream forked from and joined back
   to `stream` with events, so a graph capture of `stream` takes both):
   camera -> geodesics -> sampling -> electrons -> synchrotron -> sigma cut ->
   transfer, fused per ray; no trajectory is stored.  reqs_dev (nreq)
   device array with ray_offset the exclusive prefix sum of the requests'
   pixel counts; total_rays the sum (ray indices that fall outside their
   request's pixels -- a total_rays above the sum -- are skipped, nothing
   written).  snaps_dev (nsnap) device array of
   views.  precision: mk_precision.  Request images receive the specific
   intensity the reference's solve_specific_intensity returns. */
int mk_render(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
              const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision,
              void *workspace_dev, size_t workspace_bytes, void *stream);

/* A render job whose size lives in device memory, so one launch sequence
   can be captured once (a CUDA graph per size bucket) and replayed with
   new requests: the replay copies the header and the request table in,
   then runs the render.  total_rays <= the max_rays the sequence was
   built for. */
typedef struct {
    int32_t nreq, nsnap;
    int64_t total_rays;
} mk_job;

/* mk_render with nreq and total_rays read from job_dev on the device;
   grids and workspace (mk_render_workspace_bytes(max_rays, precision)) are
   sized for max_rays. */
int mk_render_job(const mk_job *job_dev, const mk_request *reqs_dev, const mk_snapshot_view *snaps_dev,
                  int32_t precision, int64_t max_rays, void *workspace_dev, size_t workspace_bytes,
                  void *stream);

/* Allocation-free render.  No counterpart in the reference (Mahakala is
   Python and never manages device scratch).  For callers that cannot give
   this library device memory -- a plugin confined to its host framework's
   fixed memory pool, code that must not call cudaMalloc mid-render -- this
   is mk_render with its scratch in a static device array of
   MK_NOALLOC_WORKSPACE_BYTES that every GPU loading the library holds until
   exit.  The caller still passes requests, snapshots and images.  Limit:
   any ray count in MK_FP64; at most MK_NOALLOC_MAX_MIXED_RAYS rays per call
   in the mixed forms (larger jobs return MK_ERR_LIMIT), on every GPU.  The
   first call on a device looks the array up (cudaGetSymbolAddress) and
   should come before any stream capture; a later call that finds another
   CUDA context current on that device (after a reset) looks it up again.
   All calls share the array: calls that overlap on the GPU race.  The
   workspace header, MK_WS_ERROR included, stays inside the library: a
   near-hole wait that ran out (never expected) is not reported here. */
#define MK_NOALLOC_WORKSPACE_BYTES (16u << 20)
#define MK_NOALLOC_MAX_MIXED_RAYS ((MK_NOALLOC_WORKSPACE_BYTES - 256u) / 320u)
int mk_render_noalloc(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
                      const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision, void *stream);

/* Process-wide tuning knobs (no reference counterpart).
   "fp64_rays_per_warp" (1, 2, 4, 8, 16 or 32; default 32): rays each warp
   of the mixed form's FP64 phase carries.
   "fp64_zone" (0 or 1; default 1): 0 keeps every ray of the mixed forms in
   FP32 to its end, with no FP64 phase (measures what that phase buys).
   "f32_blocks_per_sm" (0, 3, 4 or 5; default 0): the FP32 phases' kernels
   compiled for 3 resident blocks per SM (no register spills), 4 (128
   registers) or 5 (96 registers); 0 takes 4 when the launch's rays fit one
   wave of 4-block slots and 5 otherwise, and 3 for MK_MIXED's FP32
   continuation, which runs beside the near-hole phase.
   "escape_cut" (0 or 1; default 1): the mixed forms end outbound rays
   beyond the snapshot's bounding radius (see mk_precision).
   "phase_events" (0 or 1; default 0): renders record CUDA events on their
   stream around each kernel for mk_render_phase_ms; not for renders that
   are captured into a CUDA graph.
   "zone_wait_ns" (1 .. 6e10; default 1e9): the limit of each wait between
   the warps of MK_MIXED's near-hole pipeline; a wait that runs out ends
   its block and counts in the workspace word MK_WS_ERROR.
   "zone_wait_test" (0 or 1; default 0): test switch -- the near-hole
   pipeline's integrating warps withhold their first message, so the
   launch ends through its wait limit and reports MK_WS_ERROR. */
int mk_set_tuning(const char *name, int64_t value);

/* Durations (ms) of the kernels of the last render launched with the
   "phase_events" tuning set, on the current device: one for MK_FP64,
   three (A, B, C) for the mixed forms -- in MK_MIXED, B and C both start
   when A ends and run at the same time; *nphases receives the count.
   Waits for that render to finish.  No reference counterpart. */
int mk_render_phase_ms(float *ms_out, int32_t *nphases);

/* ------------------------------------------------------------ probes */
/* FMA throughput probe (no reference counterpart): blocks x threads
   threads each run iters x 8 independent-chain FMAs in FP64 (precision
   MK_FP64), FP32 (MK_MIXED), or iters x 8 paired FP32 FMAs, 16 FMAs
   (MK_PROBE_FFMA2); time it with events to get the ALU peak a roofline is
   reported against.  out_dev: blocks*threads elements of that type
   (float for MK_PROBE_FFMA2).  iters <= 2^30. */
#define MK_PROBE_FFMA2 100
int mk_probe_fma(int32_t precision, int32_t blocks, int32_t threads, int64_t iters, void *out_dev,
                 void *stream);

/* The FP64 path's own reciprocal square root, reciprocal and square root
   (float-unit seed refined by one third-order correction in binary64;
   no reference counterpart) and, for comparison, the library's correctly
   rounded forms, applied to x_dev (n) -> out_dev (n). */
typedef enum {
    MK_MATH_RSQRT = 0, MK_MATH_RCP = 1, MK_MATH_SQRT = 2,
    MK_MATH_LIB_RSQRT = 3, MK_MATH_LIB_RCP = 4, MK_MATH_LIB_SQRT = 5
} mk_math_fn;
int mk_probe_math(int32_t fn, const double *x_dev, int64_t n, double *out_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MAHAKALA_GB300_H */
