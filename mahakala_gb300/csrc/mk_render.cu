// mk_render.cu -- fused persistent render kernel (make_image, images.py:30-144).
//
// One CUDA thread owns one ray at a time.  Per accepted RK4 step it samples
// the snapshot at the new point, evaluates the electron temperature and the
// synchrotron coefficients for every requested frequency, and folds the
// sample into the transfer solution.  Nothing per-step is written to HBM.
//
// Transfer: the reference integrates the ray camera->source, then solves
// I <- I + w_i (j_i - alpha_i I) backwards from the far end, w_i = -dt_{i-1} L
// (transfer.py:106-119).  Unrolled, the camera intensity is the affine sum
//   I_cam = sum_i (w_i j_i) prod_{k<i} (1 - w_k alpha_k),
// which a forward pass accumulates with a running product P, so the solve
// happens in the same pass as the geodesic push.
//
// Work distribution: rays are handed out by a global atomic counter; when a
// lane's ray finishes it takes the next ray (warp-aggregated atomics), so
// warps stay full while rays of very different lengths finish.  Requests of
// any size can share one launch: a ray index maps to its request by a binary
// search over the requests' ray offsets.
#include "mk_common.cuh"
#include "mk_fluid.cuh"

namespace mk {

constexpr int RENDER_THREADS = 128;

// scratch of one launch: the ray counter and the work totals the launch
// accumulates (accepted steps, in-snapshot samples) for throughput and
// roofline accounting
struct RenderWorkspace {
    unsigned long long counter;
    unsigned long long steps;
    unsigned long long samples;
    unsigned long long max_tau_bits;  // max per-step optical depth w*alpha (bits of a double >= 0)
    int error;
    int pad;
};

__device__ __forceinline__ int find_request(const mk_request *__restrict__ reqs, int nreq, long long ray) {
    int lo = 0, hi = nreq - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (reqs[mid].ray_offset <= ray) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int64_t request_pixels(const mk_camera &c) {
    return c.kind == MK_CAMERA_EQUATOR ? (int64_t)c.pixels : (int64_t)c.pixels * c.pixels;
}

// One sample of the emission at state s after a step of size dt_used,
// folded into (I, P) for each frequency.  Returns without touching I, P
// outside the snapshot, where the reference's zeroed primitives give
// j = alpha = 0 exactly.
__device__ __forceinline__ void sample_fp64(const mk_request &R, const mk_snapshot_view &sv, const double s[8],
                                            double dt_used, double I[MK_MAX_NU], double P[MK_MAX_NU],
                                            int &nsamples, double &max_tau) {
    CellPos c;
    if (!locate(sv, s[1], s[2], s[3], c)) return;
    ++nsamples;
    double prim[8];
    trilinear8(sv, c, prim);
    const double a = R.camera.bhspin;
    const FluidScalars fs = fluid_frame(prim, s[1], s[2], s[3], s + 4, a, R.cos_fallback_pitch);
    // derived quantities (images.py:87-102)
    const double bsq = fs.b * fs.b;
    const double beta = fs.u * (R.fluid_gamma - 1.) / bsq / 0.5;
    const double sigma = bsq / fs.dens;
    const double Th = rlow_rhigh(fs.dens, fs.u, beta, R.r_low, R.r_high, R.electron_gamma_m1, R.ion_gamma_m1);
    const SynchroPre sp = synchro_pre(R.Ne_unit * fs.dens, Th, R.B_unit * fs.b, fs.pitch);
    const double w = -dt_used * R.L_unit;
    const bool cut = sigma > R.sigma_cut;  // images.py:116-118
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) {
        if (ch < R.nnu) {
            const double nu_obs = R.nu[ch];
            double em, ab;
            synchro_eval(sp, -fs.kdotu * nu_obs, true, 1. / nu_obs, em, ab);
            if (cut) { em = 0.0; ab = 0.0; }
            const double tau = w * ab;
            I[ch] += (w * em) * P[ch];
            P[ch] *= (1.0 - tau);
            max_tau = fmax(max_tau, tau);
        }
    }
}

__device__ __forceinline__ void finish_ray(const mk_request &R, int64_t pix, const double I[MK_MAX_NU], int steps,
                                           int why, int nsamples, double max_tau, RenderWorkspace *ws) {
    const int64_t npx = request_pixels(R.camera);
    // explicit Euler transfer is stable while every step has w*alpha < 1;
    // the launch records its largest value (non-negative doubles order like
    // their bit patterns)
    if (max_tau > 0.0) atomicMax(&ws->max_tau_bits, (unsigned long long)__double_as_longlong(max_tau));
    if (steps) atomicAdd(&ws->steps, (unsigned long long)steps);
    if (nsamples) atomicAdd(&ws->samples, (unsigned long long)nsamples);
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++)
        if (ch < R.nnu) R.image[ch * npx + pix] = I[ch];
    if (R.nsteps) R.nsteps[pix] = steps;
    if (R.status) R.status[pix] = why;
}

__global__ void __launch_bounds__(RENDER_THREADS)
render_fp64_kernel(const mk_request *__restrict__ reqs, int nreq, long long total,
                   const mk_snapshot_view *__restrict__ snaps, RenderWorkspace *ws) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int rq = 0, steps = 0, nsamples = 0, why = MK_RAY_ACTIVE;
    double max_tau = 0.0;
    int64_t pix = 0;
    double s[8], dt = 0.0, I[MK_MAX_NU], P[MK_MAX_NU];

    for (;;) {
        const unsigned need = __ballot_sync(FULL, !active && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&ws->counter, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (!active && !exhausted) {
                const long long idx = (long long)base + __popc(need & lt_mask);
                if (idx < total) {
                    rq = find_request(reqs, nreq, idx);
                    const mk_request &R = reqs[rq];
                    pix = idx - R.ray_offset;
                    camera_ray(R.camera, pix, s);
                    steps = 0;
                    nsamples = 0;
                    max_tau = 0.0;
#pragma unroll
                    for (int ch = 0; ch < MK_MAX_NU; ch++) { I[ch] = 0.0; P[ch] = 1.0; }
                    const double a = R.camera.bhspin;
                    dt = reference_dt(radius_cal(s[1], s[2], s[3], a), radius_eh(a), R.policy.div,
                                      R.policy.tol, why);
                    if (dt == 0.0 || R.policy.nmax < 2) {
                        // stopped before its first step (reference K = 0), or
                        // N < 2 leaves no row pair for the transfer solve
                        if (why == MK_RAY_ACTIVE) why = MK_RAY_MAXSTEPS;
                        finish_ray(R, pix, I, 0, why, 0, 0.0, ws);
                    } else {
                        active = true;
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;
        if (active) {
            const mk_request &R = reqs[rq];
            const double a = R.camera.bhspin;
            double nw[8];
            rk4_step(s, dt, a, nw);
            int w1;
            const double dtn = reference_dt(radius_cal(nw[1], nw[2], nw[3], a), radius_eh(a), R.policy.div,
                                            R.policy.tol, w1);
            if (dtn == 0.0) {
                // the step is rejected and the ray stays frozen (geodesics.py:263-267)
                finish_ray(R, pix, I, steps, w1, nsamples, max_tau, ws);
                active = false;
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) s[i] = nw[i];
                const double dt_used = dt;
                dt = dtn;
                ++steps;
                sample_fp64(R, snaps[R.snapshot], s, dt_used, I, P, nsamples, max_tau);
                // trajectory rows stop at N-1: step N-1 never reaches the solve
                if (steps >= R.policy.nmax - 1) {
                    finish_ray(R, pix, I, steps, MK_RAY_MAXSTEPS, nsamples, max_tau, ws);
                    active = false;
                }
            }
        }
    }
}

static int blocks_per_sm_fp64() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && cached[dev]) return cached[dev];
    int nb = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, render_fp64_kernel, RENDER_THREADS, 0);
    if (nb < 1) nb = 1;
    if (dev < 64) cached[dev] = nb;
    return nb;
}

}  // namespace mk

using namespace mk;

extern "C" size_t mk_render_workspace_bytes(void) { return 256; }

extern "C" int mk_render(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
                         const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision,
                         void *workspace_dev, size_t workspace_bytes, void *stream) {
    MK_REQUIRE(reqs_dev && snaps_dev && workspace_dev, MK_ERR_ARG, "mk_render: null pointer");
    MK_REQUIRE(nreq > 0 && nsnap > 0 && total_rays >= 0, MK_ERR_ARG, "mk_render: bad sizes");
    MK_REQUIRE(workspace_bytes >= mk_render_workspace_bytes(), MK_ERR_ARG,
               "mk_render: workspace of %zu bytes, need %zu", workspace_bytes, mk_render_workspace_bytes());
    MK_REQUIRE(((uintptr_t)workspace_dev & 7) == 0, MK_ERR_ARG, "mk_render: workspace not 8-byte aligned");
    MK_REQUIRE(precision == MK_FP64, MK_ERR_UNSUPPORTED, "mk_render: precision %d not built", (int)precision);
    cudaStream_t st = as_stream(stream);
    MK_CUDA(cudaMemsetAsync(workspace_dev, 0, sizeof(RenderWorkspace), st));
    if (total_rays == 0) return MK_OK;
    const int64_t warps = (total_rays + 31) / 32;
    int64_t grid = (int64_t)device_sm_count() * blocks_per_sm_fp64();
    const int64_t need = (warps * 32 + RENDER_THREADS - 1) / RENDER_THREADS;
    if (grid > need) grid = need;
    render_fp64_kernel<<<(unsigned)grid, RENDER_THREADS, 0, st>>>(reqs_dev, nreq, (long long)total_rays, snaps_dev,
                                                                  (RenderWorkspace *)workspace_dev);
    MK_LAUNCHED("render_fp64_kernel");
    return MK_OK;
}
