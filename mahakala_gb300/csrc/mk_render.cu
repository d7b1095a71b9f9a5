// mk_render.cu -- fused persistent render kernels (make_image, images.py:30-144).
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
// any size share one launch: a ray index maps to its request by a binary
// search over the requests' ray offsets.
//
// Precision forms:
//   MK_FP64  one launch, every operation in FP64 (the reference's x64).
//   MK_MIXED three launches, A on the caller's stream, then B on it and C
//   on a side stream forked after A and joined back after C:
//     A  FP32 from the camera (camera rays in double-float).  A ray whose
//        radius drops below R_FP64 (3 M), or that moves inward inside
//        R_TURN (6 M, where photon-ring rays reach their turning points), is
//        handed to the near-hole queue; a ray moving outward past R_TURN is
//        parked in the FP32 queue (records in binary64);
//     B  the near-hole queue (render_zone_kernel): the float-pair state is
//        renormalised to null on entry (binary64) and at each radial
//        turning point inside R_TURN (double-float); the kernel carries the
//        ray on to its end;
//     C  the FP32 queue (render_f32_kernel over the queue), beside B: the
//        two share no ray and no counter.
//   MK_MIXED_STRICT: phase B integrates the near-hole geodesic entirely in
//   binary64 (render_fp64_kernel over the queue) and parks rays leaving it
//   for phase C, after it; MK_MIXED_DF: the same in double-float pairs.
//   Splitting by precision keeps each warp uniform: on a part whose FP64
//   rate is 1/64 of FP32, one FP64 lane would stall the other 31.  The
//   intensity accumulates with a compensated (Kahan) FP32 sum and the
//   transmission product in FP32, in MK_MIXED's phase B too; the strict
//   and DF forms move both to FP64 with the ray.
#include <string.h>

#include <algorithm>

#include "mk_common.cuh"
#include "mk_dd.cuh"
#include "mk_fluid.cuh"

namespace mk {

constexpr int RENDER_THREADS = 128;
constexpr double R_FP64 = 3.0;
constexpr double R_TURN = 6.0;
// F32_RENULL (the FP32 queue): renormalise each resumed ray to null in
// binary64 -- for rays leaving the binary64 near-hole phase of
// MK_MIXED_STRICT / MK_MIXED_DF; MK_MIXED's parked rays come from phase A's
// float-pair state, null to well under half a float ulp of k^t (the images
// were bit-identical with and without), and skip it
// F32_ESCAPE (mixed forms): a ray moving outward beyond the snapshot's
// bounding radius r_out ends there as escaped (see g_escape_cut).
enum : int { F32_HANDOFF = 1, F32_PARK = 2, F32_RENULL = 4, F32_ESCAPE = 8 };

// rays per warp in the mixed form's FP64 phase (mk_set_tuning
// "fp64_rays_per_warp"): 32 fills every lane; fewer rays per warp shorten
// each warp's FP64 chain when the FP64 unit processes only active lanes
static int g_fp64_rays_per_warp = 32;
// 1: the mixed forms hand rays near the hole to FP64 (phase B); 0: phase A
// keeps every ray in FP32 to its end (a measurement switch: it shows what
// the FP64 region buys in accuracy)
static int g_fp64_zone = 1;
// resident blocks per SM the FP32 phases are compiled for: 3 (no register
// spills), 4 (registers capped at 128, a few spills), 5 (96 registers, more
// spills); 0 picks 4 when the launch's rays fit the GPU's 4-block slots in
// one wave and 5 when they do not (more resident warps pay only then)
static int g_f32_blocks = 0;
// 1: the mixed forms end a ray moving outward beyond the snapshot's
// bounding radius (SnapF32::r_out) with MK_RAY_ESCAPED.  Outside the photon
// region a null geodesic has no radial turning point, so such a ray never
// reaches the snapshot again: it takes no further sample and its intensity
// is final -- the image is bit-identical to integrating on to the
// reference's stop (r - r_EH > 1500), only its step count and the radius
// it stops at differ.  The FP64 form always keeps the reference's rule.
// 0: the mixed forms run every ray to the reference's stop as well.
static int g_escape_cut = 1;
// limit of each wait in the near-hole phase's pipeline, in ns
// (mk_set_tuning "zone_wait_ns"); a wait that runs out aborts the block and
// counts in the workspace header's MK_WS_ERROR word
static unsigned long long g_zone_wait_ns = 1000000000ull;
// test switch (mk_set_tuning "zone_wait_test"): the integrating warps
// withhold their first message, so the first wait of every block's first
// sampler can only run out -- the path by which a stalled pipeline ends
static int g_zone_wait_test = 0;
// measurement switch: when set, each render records a CUDA event on its
// stream before its first kernel and after each kernel, so the phases can
// be timed apart (mk_render_phase_ms).  Process-wide, off by default; not
// for renders captured into a graph.
static int g_phase_events = 0;
static cudaEvent_t g_phase_ev[64][4];
static bool g_phase_ev_made[64] = {false};
static int g_phase_dev = -1, g_phase_n = 0;
static int g_phase_from[4] = {0, 1, 2, 3};  // phase i runs from event g_phase_from[i] to event i + 1

// event i ends phase i - 1, which started at event `from`
static int phase_mark(cudaStream_t st, int i, int from = -1) {
    if (!g_phase_events) return MK_OK;
    int dev = 0;
    MK_CUDA(cudaGetDevice(&dev));
    MK_REQUIRE(dev >= 0 && dev < 64, MK_ERR_LIMIT, "phase events: device ordinal %d not supported", dev);
    if (!g_phase_ev_made[dev]) {
        for (int k = 0; k < 4; k++) MK_CUDA(cudaEventCreate(&g_phase_ev[dev][k]));
        g_phase_ev_made[dev] = true;
    }
    MK_CUDA(cudaEventRecord(g_phase_ev[dev][i], st));
    g_phase_dev = dev;
    g_phase_n = i;
    if (i > 0) g_phase_from[i - 1] = from < 0 ? i - 1 : from;
    return MK_OK;
}

// A second stream per host thread and device, with the two events that fork
// it from and join it back to the caller's stream within one render.  Reused
// across calls: a wait takes the event's latest record at the time it is
// enqueued.  Created on a thread's first mixed-form render; a render
// captured into a graph records its fork and join as graph edges.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

static int side_stream(SideStream **out) {
    static thread_local SideStream t_side[64];
    int dev = 0;
    MK_CUDA(cudaGetDevice(&dev));
    MK_REQUIRE(dev >= 0 && dev < 64, MK_ERR_LIMIT, "side stream: device ordinal %d not supported", dev);
    SideStream &x = t_side[dev];
    if (!x.s) {
        // the first call may come inside a stream capture: create the stream
        // and events under the relaxed capture mode, then restore the caller's
        cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
        MK_CUDA(cudaThreadExchangeStreamCaptureMode(&mode));
        const cudaError_t e1 = cudaStreamCreateWithFlags(&x.s, cudaStreamNonBlocking);
        const cudaError_t e2 = e1 == cudaSuccess ? cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) : e1;
        const cudaError_t e3 = e2 == cudaSuccess ? cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming) : e2;
        MK_CUDA(cudaThreadExchangeStreamCaptureMode(&mode));
        if (e3 != cudaSuccess) x.s = nullptr;
        MK_CUDA(e3);
    }
    *out = &x;
    return MK_OK;
}

// launch scratch: counters and work totals, then (mixed form) two queues
struct RenderWorkspace {
    unsigned long long counter;       // next camera ray (phase A / FP64 form)
    unsigned long long steps;         // accepted RK4 steps
    unsigned long long samples;       // in-snapshot samples
    unsigned long long max_tau_bits;  // max per-step optical depth w*alpha (bits of a double >= 0)
    unsigned long long q64_count;     // rays handed to FP64
    unsigned long long q64_next;
    unsigned long long q32_count;     // rays in the FP32 continuation queue
    unsigned long long q32_next;
    unsigned long long steps_fp64;    // accepted steps taken in FP64 (mixed form)
    unsigned long long overflow;      // queue overflow (cannot happen: capacity = rays)
    unsigned long long samples_fp64;  // in-snapshot samples taken in the FP64 phase (mixed form)
    unsigned long long zone_run_max;  // most steps one ray took in one visit to the near-hole phase
    unsigned long long steps_b;       // all steps render_zone_kernel took (near the hole and after)
    unsigned long long samples_b;     // all samples render_zone_kernel took
    unsigned long long zone_exits;    // rays that left the near-hole phase outward (back to FP32)
    unsigned long long steps_c;       // steps the FP32 continuation over the FP32 queue took
    unsigned long long samples_c;     // samples it took
    unsigned long long zone_error;    // bounded waits of the near-hole phase that ran out (images invalid)
};
constexpr size_t WS_HEADER = 256;
static_assert(sizeof(RenderWorkspace) <= WS_HEADER, "workspace header");

// a ray in flight between the precision phases
struct RayRecord {
    double s[8];
    double I[MK_MAX_NU];
    double P[MK_MAX_NU];
    double max_tau;
    long long ray;
    int steps, nsamples;
    int rq, pad;
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

// false for a ray index outside its request's pixels, which happens only
// when total_rays exceeds the sum of the requests' pixel counts (a caller
// error the host cannot see: the table is on the device); such a ray is
// skipped, so no image is written out of bounds
__device__ __forceinline__ bool ray_in_request(const mk_request *__restrict__ reqs, int nreq, long long ray) {
    const int rq = find_request(reqs, nreq, ray);
    const long long pix = ray - reqs[rq].ray_offset;
    return pix >= 0 && pix < request_pixels(reqs[rq].camera);
}

// integer square root (floor) of 0 <= i < 2^31
__device__ __forceinline__ int isqrt_floor(int i) {
    int q = (int)sqrtf((float)i);
    while (q > 0 && q * q > i) --q;
    while ((q + 1) * (q + 1) <= i) ++q;
    return q;
}

// The j-th pixel of an n x n grid in centre-out order: square rings around
// the image centre, innermost first (rays near the centre reach the
// photon-ring region and the horizon and take the most steps, so fetching
// them first starts the longest chains when the launch starts); returns the
// pixel index ix * n + iy.  A bijection of [0, n^2).
__device__ __forceinline__ int64_t center_out_pixel(int64_t j64, int n) {
    const int j = (int)j64;
    int k, lo, side, e;
    if (n & 1) {
        const int c = (n - 1) >> 1;
        if (j == 0) return (int64_t)c * n + c;
        k = (isqrt_floor(j) + 1) >> 1;
        e = j - (2 * k - 1) * (2 * k - 1);
        lo = c - k;
        side = 2 * k + 1;
    } else {
        k = isqrt_floor(j) >> 1;
        e = j - 4 * k * k;
        lo = (n >> 1) - 1 - k;
        side = 2 * k + 2;
    }
    const int hi = lo + side - 1, edge = side - 1;
    int ix, iy;
    if (e < edge) { ix = lo + e; iy = lo; }
    else if (e < 2 * edge) { ix = hi; iy = lo + (e - edge); }
    else if (e < 3 * edge) { ix = hi - (e - 2 * edge); iy = hi; }
    else { ix = lo; iy = hi - (e - 3 * edge); }
    return (int64_t)ix * n + iy;
}

// pixel of a request for its local fetch index: centre-out on grid cameras
// (the FP64 form: 1-3 % faster at 256x256; the mixed form's camera phase
// keeps pixel order, in which its parked rays' queue coheres better --
// centre-out there made the 1024x1024 stress render 20.6 -> 21.4 ms)
__device__ __forceinline__ int64_t fetch_pixel(const mk_camera &c, int64_t local) {
    return c.kind == MK_CAMERA_GRID ? center_out_pixel(local, c.pixels) : local;
}

// warp-aggregated work fetch: returns this lane's item index, -1 when the
// lane asked and the work is exhausted, -2 when the lane did not ask
__device__ __forceinline__ long long fetch(bool want, unsigned long long *counter, long long total) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned need = __ballot_sync(FULL, want);
    if (!need) return -2;
    const int leader = __ffs(need) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
    base = __shfl_sync(FULL, base, leader);
    if (!want) return -2;
    const long long idx = (long long)base + __popc(need & ((1u << lane) - 1u));
    return idx < total ? idx : -1;
}

__device__ __forceinline__ void record_tau(RenderWorkspace *ws, double max_tau) {
    // explicit Euler transfer is stable while every step has w*alpha < 1;
    // non-negative doubles order like their bit patterns
    if (max_tau > 0.0) atomicMax(&ws->max_tau_bits, (unsigned long long)__double_as_longlong(max_tau));
}

template <typename T>
__device__ __forceinline__ void finish_ray(const mk_request &R, int64_t pix, const T I[MK_MAX_NU], int steps,
                                           int why, int nsamples, double max_tau, RenderWorkspace *ws) {
    const int64_t npx = request_pixels(R.camera);
    if (steps) atomicAdd(&ws->steps, (unsigned long long)steps);
    if (nsamples) atomicAdd(&ws->samples, (unsigned long long)nsamples);
    record_tau(ws, max_tau);
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++)
        if (ch < R.nnu) R.image[ch * npx + pix] = (double)I[ch];
    if (R.nsteps) R.nsteps[pix] = steps;
    if (R.status) R.status[pix] = why;
}

// ------------------------------------------------------------------ FP64
// One sample of the emission at state s after a step of size dt_used,
// folded into (I, P) for each frequency.  Returns without touching I, P
// outside the snapshot, where the reference's zeroed primitives give
// j = alpha = 0 exactly.
// row >= 0: also store em and ab at that trajectory row of the request's
// per-step diagnostic arrays (row < R.rows).
__device__ __forceinline__ void sample_fp64(const mk_request &R, const mk_snapshot_view &sv, const double s[8],
                                            const KerrPoint<double> &m, double dt_used, double I[MK_MAX_NU],
                                            double P[MK_MAX_NU], int &nsamples, double &max_tau, int64_t pix,
                                            int64_t row) {
    CellPos c;
    if (!locate_fast(sv, s[1], s[2], s[3], c)) return;
    ++nsamples;
    double prim[8];
    trilinear8_fast(sv, c, prim);
    const FluidFrame fs = fluid_frame_m(prim, m, s + 4, R.cos_fallback_pitch);
    // derived quantities (images.py:87-102)
    // quotients as products with rcp64 reciprocals (within a few ulp of the
    // reference's divisions; the FP64 pipe is this kernel's bound)
    const double bsq = fs.b * fs.b;
    const double beta = fs.u * (R.fluid_gamma - 1.) * 2.0 * rcp64(bsq);
    const double sigma = bsq * rcp64(fs.dens);
    const double Th = rlow_rhigh_fast(fs.dens, fs.u, beta, R.r_low, R.r_high, R.electron_gamma_m1, R.ion_gamma_m1);
    const SynchroPre sp = synchro_pre_sin(R.Ne_unit * fs.dens, Th, R.B_unit * fs.b, sin_from_cos(fs.cos_pitch));
    const double w = -dt_used * R.L_unit;
    const bool cut = sigma > R.sigma_cut;  // images.py:116-118
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) {
        if (ch < R.nnu) {
            const double nu_obs = R.nu[ch];
            double em, ab;
            synchro_eval(sp, -fs.kdotu * nu_obs, true, rcp64(nu_obs), em, ab);
            if (cut) { em = 0.0; ab = 0.0; }
            if (row >= 0) {
                const int64_t at = (ch * R.rows + row) * request_pixels(R.camera) + pix;
                R.rows_em[at] = em;
                R.rows_ab[at] = ab;
            }
            const double tau = w * ab;
            I[ch] += (w * em) * P[ch];
            P[ch] *= (1.0 - tau);
            max_tau = fmax(max_tau, tau);
        }
    }
}

// Rescale k^t so that g(k, k) = 0 at x, keeping the spatial wavevector:
// g00 k0^2 + 2 g0i k^i k0 + gij k^i k^j = 0, the root nearest the current k0.
// Binary64 throughout, with the reciprocal and roots of the FP64 render
// (rcp64, rsqrt64, sqrt64: within 2 ulp of the correctly rounded forms)
// in place of the division and square-root subroutines: those made one
// renormalisation ~200 FP64-pipe instructions, ~9 k cycles of the
// near-hole phase's serial chain each time a lane of its warp reached a
// radial turning point.
__device__ __forceinline__ void renull_fp64(double s[8], double a) {
    const double x = s[1], y = s[2], z = s[3];
    const double aa = a * a, zz = z * z;
    const double kk = 0.5 * (x * x + y * y + zz - aa);
    const double Q = kk * kk + aa * zz;
    const double rr = sqrt64(Q) + kk;
    const double ir = rsqrt64(rr);
    const double r = rr * ir;
    const double den = rr * rr + aa * zz, rra = rr + aa;
    const double inv2 = rcp64(den * rra);          // 1 / (den (r^2 + a^2))
    const double f = 2.0 * (rr * r * (rra * inv2));
    const double ira = den * inv2;
    const double l1 = (r * x + a * y) * ira, l2 = (r * y - a * x) * ira, l3 = z * ir;
    const double lk = l1 * s[5] + l2 * s[6] + l3 * s[7];
    const double A = -1.0 + f;                      // g00
    const double B = 2.0 * f * lk;                  // 2 g0i k^i
    const double C = s[5] * s[5] + s[6] * s[6] + s[7] * s[7] + f * lk * lk;
    const double disc = B * B - 4.0 * A * C;
    if (!(disc >= 0.0) || A == 0.0) return;
    const double sq = sqrt64(disc);
    const double i2A = rcp64(2.0 * A);
    const double r1 = (sq - B) * i2A, r2 = -(B + sq) * i2A;
    s[4] = fabs(r1 - s[4]) < fabs(r2 - s[4]) ? r1 : r2;
}

// ------------------------------------------------------------------ FP32
// A request's scalars in float, loaded once per ray: converting them from
// the request's doubles at every sample would put ~12 instructions per step
// on the FP64 pipe (1/64 rate), which the one-warp phases wait on.
struct RayF32 {
    float cos_fb, gam1, r_high, r_low, gem1, gim1, Ne_unit, B_unit, sigma_cut, L_unit, div, tol;
    int nnu;
};

__device__ __forceinline__ RayF32 ray_f32(const mk_request &R) {
    RayF32 c;
    c.cos_fb = (float)R.cos_fallback_pitch;
    c.gam1 = (float)(R.fluid_gamma - 1.);
    c.r_high = (float)R.r_high;
    c.r_low = (float)R.r_low;
    c.gem1 = (float)R.electron_gamma_m1;
    c.gim1 = (float)R.ion_gamma_m1;
    c.Ne_unit = (float)R.Ne_unit;
    c.B_unit = (float)R.B_unit;
    c.sigma_cut = (float)R.sigma_cut;
    c.L_unit = (float)R.L_unit;
    c.div = (float)R.policy.div;
    c.tol = (float)R.policy.tol;
    c.nnu = R.nnu;
    return c;
}

// emission coefficients of one sample in float (mixed forms) at the located
// cell c: em, ab per frequency (invariant, rescaled as in the FP64 path)
__device__ __forceinline__ void emission_f32_at(const mk_snapshot_view &sv, const CellPosF &c, const RayF32 &rc,
                                                const float s[8], const KerrPoint<float> &m,
                                                const SynchroF32 sc[MK_MAX_NU], float em_out[MK_MAX_NU],
                                                float ab_out[MK_MAX_NU]) {
    float prim[8];
    trilinear8_f32(sv, c, prim);
    const FluidF32 fs = fluid_frame_f32(prim, m, s + 4, rc.cos_fb);
    const float bsq = fs.b * fs.b;
    // float quotients by the hardware reciprocal (fdiv: ~2 ulp)
    const float beta = fdiv(fs.u * rc.gam1, bsq) * 2.0f;
    const float sigma = fdiv(bsq, fs.dens);
    const float b2 = beta * beta;
    const float T_ratio = fdiv(rc.r_high * b2 + rc.r_low, 1.0f + b2);
    // Theta_e = (MP/ME) u gem1 gim1 / (dens (gim1 + gem1 T_ratio))
    const float Th = fdiv((float)(MP / ME) * fs.u * rc.gem1 * rc.gim1, fs.dens * (rc.gim1 + rc.gem1 * T_ratio));
    const float Ne = rc.Ne_unit * fs.dens;
    const float Bg = rc.B_unit * fs.b;
    const float sin_p = sqrt_approx((1.0f - fs.cos_pitch) * (1.0f + fs.cos_pitch));
    const float th2 = Th * Th;
    // nus in Hz; nu' = -k.u (observed frequency rescaled to 1)
    const float nus = (float)(TWO_NINTHS * EE / TWO_PI_ME_CL) * Bg * th2 * sin_p;
    const float nup = -fs.kdotu;
    const bool cut = sigma > rc.sigma_cut || Th < 0.3f;
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) {
        if (ch < rc.nnu) {
            const float nusp = nus * sc[ch].inv_nu;  // nus / nu_obs
            const float X = fdiv(nup, nusp);
            const float x3 = cbrt_approx(X);
            const float term = sqrt_approx(X) + (float)C2_11_12 * sqrt_approx(x3);
            // emissivity / nu'^2 (invariant, rescaled): k_em folds
            // sqrt2 pi EE^2 / (3 CL) and nu_obs
            float em = fdiv(Ne * sc[ch].k_em * nusp * term * term, 2.0f * th2 * nup * nup) * __expf(-x3);
            if (X > 1.e12f || cut) em = 0.0f;
            const float bx = fdiv(sc[ch].k_bx * nup, Th);
            // expm1(bx) (series below 2e-3; at radio frequencies bx ~ 1e-9);
            // a branch, so the library expm1f is not evaluated beside it
            float bden;
            if (bx < 2.e-3f)
                bden = bx * (1.0f / 24.0f) * (24.f + bx * (12.f + bx * (4.f + bx)));
            else
                bden = expm1f(bx);
            // alpha nu' = (em nu'^2) / B_nu * nu' with B_nu = k_bnu nu'^3 / bden
            float ab = fdiv(em * bden, sc[ch].k_bnu);
            em_out[ch] = isnan(em) ? 0.0f : em;
            ab_out[ch] = isnan(ab) ? 0.0f : ab;
        }
    }
}

// one FP32 sample at the located cell folded into a compensated (Kahan)
// float intensity sum; w = -dt L
__device__ __forceinline__ void sample_f32(const mk_snapshot_view &sv, const CellPosF &c, const RayF32 &rc,
                                           const float s[8], const KerrPoint<float> &m, float dt_used,
                                           float I[MK_MAX_NU], float Ic[MK_MAX_NU], float P[MK_MAX_NU],
                                           const SynchroF32 sc[MK_MAX_NU], int &nsamples, float &max_tau) {
    float em[MK_MAX_NU], ab[MK_MAX_NU];
    emission_f32_at(sv, c, rc, s, m, sc, em, ab);
    ++nsamples;
    const float w = -dt_used * rc.L_unit;
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) {
        if (ch < rc.nnu) {
            const float tau = w * ab[ch];
            const float y = (w * em[ch]) * P[ch] - Ic[ch];
            const float t = I[ch] + y;
            Ic[ch] = (t - I[ch]) - y;
            I[ch] = t;
            P[ch] *= (1.0f - tau);
            max_tau = fmaxf(max_tau, tau);
        }
    }
}

// FP32 emission at the located cell, accumulated in FP64 (near-hole phase)
__device__ __forceinline__ void sample_f32_sum64(const mk_snapshot_view &sv, const CellPosF &c, const RayF32 &rc,
                                                 const float s[8], const KerrPoint<float> &m, double w,
                                                 double I[MK_MAX_NU], double P[MK_MAX_NU],
                                                 const SynchroF32 sc[MK_MAX_NU], int &nsamples, double &max_tau) {
    float em[MK_MAX_NU], ab[MK_MAX_NU];
    emission_f32_at(sv, c, rc, s, m, sc, em, ab);
    ++nsamples;
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) {
        if (ch < rc.nnu) {
            const double tau = w * (double)ab[ch];
            I[ch] += (w * (double)em[ch]) * P[ch];
            P[ch] *= (1.0 - tau);
            max_tau = fmax(max_tau, tau);
        }
    }
}

// FP32 emission at an FP64 or double-float state (strict and DF phase B),
// accumulated in FP64
template <typename T>
__device__ __forceinline__ void sample_f32_at(const mk_request &R, const mk_snapshot_view &sv, const SnapF32 &sf,
                                              const T s[8], const KerrPoint<T> &m64, double dt_used,
                                              double I[MK_MAX_NU], double P[MK_MAX_NU],
                                              const SynchroF32 sc[MK_MAX_NU], int &nsamples, double &max_tau) {
    float sf8[8];
#pragma unroll
    for (int i = 0; i < 8; i++) sf8[i] = to_float(s[i]);
    KerrPoint<float> m;
    m.r = to_float(m64.r);
    m.f = to_float(m64.f);
    m.l1 = to_float(m64.l1);
    m.l2 = to_float(m64.l2);
    m.l3 = to_float(m64.l3);
    CellPosF c;
    if (!locate_f32(sv, sf, sf8[1], sf8[2], sf8[3], c)) return;
    const RayF32 rc = ray_f32(R);
    sample_f32_sum64(sv, c, rc, sf8, m, -dt_used * R.L_unit, I, P, sc, nsamples, max_tau);
}

enum { SRC_CAMERA = 0, SRC_QUEUE = 1 };

// A request's float constants, one shared-memory entry per request of the
// launch: read where used instead of held in ~37 registers per ray, which
// lets the FP32 phases keep more warps resident.
struct ReqF32 {
    RayF32 rc;
    SynchroF32 sc[MK_MAX_NU];
    SnapF32 sf;
    float a, reh;
    CameraDD cam;           // grid camera constants for camera_ray_pair
    int cam_pixels, cam_grid;
};

__device__ __forceinline__ void fill_req_f32(const mk_request &R, const mk_snapshot_view *snaps, ReqF32 &o) {
    o.rc = ray_f32(R);
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++)
        if (ch < R.nnu) o.sc[ch] = synchro_consts(R.nu[ch]);
    o.sf = snap_f32(snaps[R.snapshot]);
    o.a = (float)R.camera.bhspin;
    o.reh = (float)radius_eh(R.camera.bhspin);
    o.cam = camera_dd(R.camera);
    o.cam_pixels = R.camera.pixels;
    o.cam_grid = R.camera.kind == MK_CAMERA_GRID;
}



// FP64 render.  SRC_CAMERA: every ray of the job, start to end (MK_FP64).
// SRC_QUEUE: mixed-form phase B over the FP64 queue; rays leaving R_TURN
// outward go to the FP32 queue.  T is the geodesic arithmetic: double, or
// dd (double-float pairs) for the MK_MIXED_DF variant of phase B.
template <int SRC, typename T = double>
__global__ void __launch_bounds__(RENDER_THREADS)
render_fp64_kernel(const mk_request *__restrict__ reqs, int nreq, long long total_camera,
                   const mk_snapshot_view *__restrict__ snaps, RenderWorkspace *ws, RayRecord *q64,
                   RayRecord *q32, long long capacity, int lane_stride, const mk_job *job) {
    if (job) {  // request count and ray total from the device (graph replays)
        nreq = job->nreq;
        total_camera = job->total_rays;
    }
    unsigned long long *counter = SRC == SRC_CAMERA ? &ws->counter : &ws->q64_next;
    // lanes not on the stride never take work and stay masked off
    const bool lane_works = ((threadIdx.x & 31) % lane_stride) == 0;
    const long long total =
        SRC == SRC_CAMERA ? total_camera
                          : min((long long)*(volatile unsigned long long *)&ws->q64_count, capacity);
    bool active = false, exhausted = false;
    int rq = 0, steps = 0, nsamples = 0, why = MK_RAY_ACTIVE, fp64_steps = 0, fp64_samples = 0;
    long long ray = 0;
    int64_t pix = 0;
    T s[8], d1[4], dt = T(0.0);
    double r_cur = 0.0, reh = 0.0, I[MK_MAX_NU], P[MK_MAX_NU], max_tau = 0.0;
    SynchroF32 sc[MK_MAX_NU];
    SnapF32 sf;

    for (;;) {
        const long long idx = fetch(lane_works && !active && !exhausted, counter, total);
        if (idx == -1) exhausted = true;
        if (!lane_works) exhausted = true;
        if (idx >= 0 && (SRC != SRC_CAMERA || ray_in_request(reqs, nreq, idx))) {
            if (SRC == SRC_CAMERA) {
                rq = find_request(reqs, nreq, idx);
                pix = fetch_pixel(reqs[rq].camera, idx - reqs[rq].ray_offset);
                ray = reqs[rq].ray_offset + pix;
                double s64[8];
                camera_ray(reqs[rq].camera, pix, s64);
#pragma unroll
                for (int i = 0; i < 8; i++) s[i] = T(s64[i]);
                steps = nsamples = 0;
                max_tau = 0.0;
#pragma unroll
                for (int ch = 0; ch < MK_MAX_NU; ch++) { I[ch] = 0.0; P[ch] = 1.0; }
            } else {
                const RayRecord &q = q64[idx];
                double s64[8];
#pragma unroll
                for (int i = 0; i < 8; i++) s64[i] = q.s[i];
#pragma unroll
                for (int ch = 0; ch < MK_MAX_NU; ch++) { I[ch] = q.I[ch]; P[ch] = q.P[ch]; }
                max_tau = q.max_tau;
                ray = q.ray;
                steps = q.steps;
                nsamples = q.nsamples;
                rq = q.rq;
                pix = ray - reqs[rq].ray_offset;
                renull_fp64(s64, reqs[rq].camera.bhspin);
#pragma unroll
                for (int i = 0; i < 8; i++) s[i] = T(s64[i]);
                const mk_request &Rq = reqs[rq];
#pragma unroll
                for (int ch = 0; ch < MK_MAX_NU; ch++)
                    if (ch < Rq.nnu) sc[ch] = synchro_consts(Rq.nu[ch]);
                sf = snap_f32(snaps[Rq.snapshot]);
            }
            const mk_request &R = reqs[rq];
            const T a = T(R.camera.bhspin);
            // the first RK4 stage at s also yields r for the step rule (the
            // metric's r equals radius_cal, geodesics.py:284-291, analytically)
            KerrPoint<T> m;
            kerr_accel(s[1], s[2], s[3], s[4], s[5], s[6], s[7], a, d1[0], d1[1], d1[2], d1[3], m);
            r_cur = to_double(m.r);
            reh = radius_eh(R.camera.bhspin);
            const double dt0 = reference_dt(r_cur, reh, R.policy.div, R.policy.tol, why);
            dt = T(dt0);
            if (dt0 == 0.0 || R.policy.nmax < 2) {
                // stopped before its next step (reference K = steps), or N < 2
                // leaves no row pair for the transfer solve
                if (why == MK_RAY_ACTIVE) why = MK_RAY_MAXSTEPS;
                finish_ray(R, pix, I, steps, why, nsamples, max_tau, ws);
            } else {
                active = true;
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            const mk_request &R = reqs[rq];
            const T a = T(R.camera.bhspin);
            T nw[8], dn[4];
            rk4_step_k1(s, d1, dt, a, nw);
            // next step's first stage, evaluated now: gives r and the metric
            // at the new point for the rule and the sample
            KerrPoint<T> m;
            kerr_accel(nw[1], nw[2], nw[3], nw[4], nw[5], nw[6], nw[7], a, dn[0], dn[1], dn[2], dn[3], m);
            int w1;
            const double r_new = to_double(m.r);
            const double dtn = reference_dt(r_new, reh, R.policy.div, R.policy.tol, w1);
            if (dtn == 0.0) {
                // the step is rejected and the ray stays frozen (geodesics.py:263-267)
                finish_ray(R, pix, I, steps, w1, nsamples, max_tau, ws);
                active = false;
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) s[i] = nw[i];
#pragma unroll
                for (int i = 0; i < 4; i++) d1[i] = dn[i];
                const double dt_used = to_double(dt);
                dt = T(dtn);
                ++steps;
                ++fp64_steps;
                if constexpr (SRC == SRC_CAMERA) {
                    int64_t row = -1;
                    if (R.rows_dt && steps < R.rows) {  // per-step diagnostics: row `steps` = this state
                        row = steps;
                        R.rows_dt[(int64_t)(steps - 1) * request_pixels(R.camera) + pix] = dt_used;
                    }
                    sample_fp64(R, snaps[R.snapshot], s, m, dt_used, I, P, nsamples, max_tau, pix,
                                R.rows_em ? row : -1);
                }
                else {  // mixed form: FP64 (or pair) geodesic, FP32 emission, FP64 sums
                    const int ns0 = nsamples;
                    sample_f32_at(R, snaps[R.snapshot], sf, s, m, dt_used, I, P, sc, nsamples, max_tau);
                    fp64_samples += nsamples - ns0;
                }
                // trajectory rows stop at N-1: step N-1 never reaches the solve
                if (steps >= R.policy.nmax - 1) {
                    finish_ray(R, pix, I, steps, MK_RAY_MAXSTEPS, nsamples, max_tau, ws);
                    active = false;
                } else if (SRC == SRC_QUEUE && r_new >= R_TURN && r_new > r_cur) {
                    // outbound past the photon-ring region: back to FP32
                    const unsigned long long slot = atomicAdd(&ws->q32_count, 1ull);
                    atomicAdd(&ws->zone_exits, 1ull);
                    if ((long long)slot < capacity) {
                        RayRecord &q = q32[slot];
#pragma unroll
                        for (int i = 0; i < 8; i++) q.s[i] = to_double(s[i]);
#pragma unroll
                        for (int ch = 0; ch < MK_MAX_NU; ch++) { q.I[ch] = I[ch]; q.P[ch] = P[ch]; }
                        q.max_tau = max_tau;
                        q.ray = ray;
                        q.steps = steps;
                        q.nsamples = nsamples;
                        q.rq = rq;
                        active = false;
                    } else {
                        atomicAdd(&ws->overflow, 1ull);  // keep integrating in FP64
                    }
                }
                r_cur = r_new;
            }
        }
    }
    if (SRC == SRC_QUEUE && fp64_steps) atomicAdd(&ws->steps_fp64, (unsigned long long)fp64_steps);
    if (SRC == SRC_QUEUE && fp64_samples) atomicAdd(&ws->samples_fp64, (unsigned long long)fp64_samples);
}

__device__ __forceinline__ void finish_ray_f32(const mk_request &R, int64_t pix, const float I[MK_MAX_NU],
                                               const float Ic[MK_MAX_NU], int steps, int why, int nsamples,
                                               float max_tau, RenderWorkspace *ws) {
    double Iout[MK_MAX_NU];
#pragma unroll
    for (int ch = 0; ch < MK_MAX_NU; ch++) Iout[ch] = (double)I[ch] - (double)Ic[ch];
    finish_ray(R, pix, Iout, steps, why, nsamples, (double)max_tau, ws);
}

// Mixed-form phase B (MK_MIXED): the rays near the hole.  The state is a
// float pair per component (~48-bit significand), advanced by RK4
// increments formed in float (rk4_increment_f32); the wavevector is
// renormalised to null on entry (binary64, from the record) and at every
// radial turning point inside R_TURN (double-float, renull_k0_dd); the
// intensity and transmission sums are
// compensated floats.  The accelerations and the emission are float, as in
// phase A: on this part a binary64 acceleration costs ~33x a float one per
// step, and over the measured images it changed the error against the FP64
// form by less than the float emission already contributes.  A ray leaving
// R_TURN outward is counted as back in FP32 and continues here.
//
// Few rays reach this phase and its time is the serial chain of the
// longest one, so each block is a pipeline of four warps on the SM's four
// sub-partitions.  Warp 0 integrates 32 rays and posts one message per step
// (per lane: the state after the step, the metric there, the step size,
// flags).  Warps 1-3 take the messages in turn -- message j goes to warp
// 1 + j % 3 -- and each locates the sample's cell, interpolates the
// primitives and evaluates the emission, then folds the sample into the
// lane's transfer sums in message order.  One warp takes ~2.4 k cycles for
// a sample and ~1.3 k for an integration step (GB300, one block alone), so
// with three samplers the integrating warp no longer waits on the samples,
// and the cell lookup is off its chain too.
//
// Messages pass through ZONE_SLOTS slots in shared memory, each with two
// mbarriers: `full` (the integrator's 32 lanes arrive after writing the
// slot) and `empty` (its sampler's 32 lanes arrive after reading it).  The
// fold order is a counter in shared memory: the sampler of message j folds
// when it reads j and then sets it to j + 1.  Every wait is bounded
// (mk_set_tuning "zone_wait_ns", 1 s by default): a wait that runs out sets
// the block's abort flag and counts in the workspace header's MK_WS_ERROR
// word, every warp of the block then leaves, and the launch's images are
// invalid (the Python layer raises).  No wait depends on another block.
enum : unsigned { ZM_START = 1u, ZM_SAMPLE = 2u, ZM_END = 4u, ZM_DONE = 16u, ZM_ZONE = 32u };
constexpr int ZONE_THREADS = 128;
constexpr int ZONE_SAMPLERS = 3;
constexpr int ZONE_SLOTS = 6;  // a multiple of ZONE_SAMPLERS: each sampler alternates between two slots
static_assert(ZONE_SLOTS % ZONE_SAMPLERS == 0 && ZONE_THREADS == 32 * (1 + ZONE_SAMPLERS), "zone pipeline");

struct ZoneSlot {
    unsigned flags[32];
    int idx[32];     // the lane's ray: its index in the near-hole queue
    int steps[32];   // ZM_END: steps taken and stop reason
    int why[32];
    float s[7][32];  // ZM_SAMPLE: x^1..x^3, k^0..k^3 after the step
    float m[5][32];  // r, f, l1, l2, l3 there
    float dt[32];    // the step's size
};

struct ZoneShared {
    ZoneSlot slot[ZONE_SLOTS];
    // each lane's transfer sums, touched only by the sampler folding the
    // lane's current message
    float I[MK_MAX_NU][32], Ic[MK_MAX_NU][32], P[MK_MAX_NU][32];
    float max_tau[32];
    int nsamples[32];
    unsigned long long full[ZONE_SLOTS], empty[ZONE_SLOTS];
    int folded;  // messages folded so far
    int abort;   // a wait of this block ran out
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

// release: this thread's earlier shared-memory writes are visible to a
// thread whose wait on the phase succeeds
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b))
                 : "memory");
}

// acquire: true once the phase of parity `parity` has completed
__device__ __forceinline__ bool mbar_test(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait of a whole warp (every lane calls it and gets the same
// answer) for the phase of parity `parity` of mbarrier b: false when
// limit_ns ran out or the block aborted.
__device__ __forceinline__ bool zone_wait(unsigned long long *b, unsigned parity, const ZoneShared &zs,
                                          unsigned long long limit_ns) {
    const unsigned FULL = 0xffffffffu;
    // the common case, a phase already complete, reads no timer
    if (__all_sync(FULL, mbar_test(b, parity))) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned i = 1;; ++i) {
        if (__all_sync(FULL, mbar_test(b, parity))) return true;
        if ((i & 31u) == 0u) {
            const bool stop = *(const volatile int *)&zs.abort != 0 || global_ns() - t0 > limit_ns;
            if (__any_sync(FULL, stop)) return false;
        }
    }
}

// Bounded wait of a whole warp until `folded` reads j.
__device__ __forceinline__ bool zone_wait_fold(const ZoneShared &zs, int j, unsigned long long limit_ns) {
    const unsigned FULL = 0xffffffffu;
    if (__all_sync(FULL, *(const volatile int *)&zs.folded == j)) {
        __threadfence_block();  // the sums written before `folded` was set
        return true;
    }
    const unsigned long long t0 = global_ns();
    for (unsigned i = 1;; ++i) {
        if (__all_sync(FULL, *(const volatile int *)&zs.folded == j)) {
            __threadfence_block();  // the sums written before `folded` was set
            return true;
        }
        if ((i & 31u) == 0u) {
            const bool stop = *(const volatile int *)&zs.abort != 0 || global_ns() - t0 > limit_ns;
            if (__any_sync(FULL, stop)) return false;
        }
    }
}

// a wait ran out: stop the block's other warps and count it once per warp
__device__ __forceinline__ void zone_fail(ZoneShared &zs, RenderWorkspace *ws) {
    *(volatile int *)&zs.abort = 1;
    if ((threadIdx.x & 31) == 0) atomicAdd(&ws->zone_error, 1ull);
}

__device__ __forceinline__ void zone_integrate(const mk_request *__restrict__ reqs,
                                               const mk_snapshot_view *__restrict__ snaps, RenderWorkspace *ws,
                                               const RayRecord *q64, long long capacity, int escape,
                                               ZoneShared &zs, unsigned long long limit_ns, int withhold) {
    const int lane = threadIdx.x & 31;
    unsigned long long *counter = &ws->q64_next;
    const long long total = min((long long)*(volatile unsigned long long *)&ws->q64_count, capacity);
    bool active = false, exhausted = false;
    int steps = 0, nmax = 0, zone_steps = 0, run = 0, run_max = 0, b_steps = 0, ray = -1;
    // float-pair state (X, K) throughout, as in the FP32 phases; near the
    // hole the wavevector is renormalised to null on entry (binary64) and
    // at every radial turning point (double-float).  After the ray leaves
    // outward the integration continues here to the ray's end (its
    // remaining ~250 steps would otherwise wait for a third launch).
    bool inzone = true;
    double bhspin = 0.0;
    dd ad(0.0f);  // the spin as a float pair
    f2 X[4], K[4];
    float xf[8];  // the state rounded to float
    float d1[4], dt = 0.0f, r_cur = 0.0f, dr_prev = 0.0f, reh = 0.0f, a = 0.0f, div = 0.0f, tol = 0.0f;
    float r_out = 0.0f;

    for (int it = 0;; ++it) {
        const int sl = it % ZONE_SLOTS;
        ZoneSlot &msg = zs.slot[sl];
        if (it >= ZONE_SLOTS && !zone_wait(&zs.empty[sl], (unsigned)((it / ZONE_SLOTS) - 1) & 1u, zs, limit_ns)) {
            zone_fail(zs, ws);
            return;
        }
        unsigned flags = 0;
        const long long idx = fetch(!active && !exhausted, counter, total);
        if (idx == -1) exhausted = true;
        if (idx >= 0) {
            const RayRecord &q = q64[idx];
            double s[8];
#pragma unroll
            for (int i = 0; i < 8; i++) s[i] = q.s[i];
            steps = q.steps;
            ray = (int)idx;
            const mk_request &R = reqs[q.rq];
            bhspin = R.camera.bhspin;
            nmax = R.policy.nmax;
            div = (float)R.policy.div;
            tol = (float)R.policy.tol;
            renull_fp64(s, bhspin);
            a = (float)bhspin;
            ad = dd(bhspin);
            reh = (float)radius_eh(bhspin);
            r_out = snap_f32(snaps[R.snapshot]).r_out;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                X[i] = f2_from(s[i]);
                K[i] = f2_from(s[4 + i]);
                xf[i] = X[i].hi;
                xf[4 + i] = K[i].hi;
            }
            KerrPoint<float> m;
            kerr_accel(xf[1], xf[2], xf[3], xf[4], xf[5], xf[6], xf[7], a, d1[0], d1[1], d1[2], d1[3], m);
            r_cur = m.r;
            dr_prev = 0.0f;
            run = 0;
            inzone = true;
            flags |= ZM_START;
            int why = MK_RAY_ACTIVE;
            dt = reference_dt(r_cur, reh, div, tol, why);
            if (dt == 0.0f || nmax < 2) {
                flags |= ZM_END;
                msg.why[lane] = why == MK_RAY_ACTIVE ? MK_RAY_MAXSTEPS : why;
                msg.steps[lane] = steps;
            } else {
                active = true;
            }
        }
        const bool any = __any_sync(0xffffffffu, active);
        if (active) {
            float xa[4], dK[4];
            rk4_increment_f32(xf, xf + 4, d1, dt, a, xa, dK);
            // pair-precision state update (a binary64 state cost the
            // integrating warp 16 FP64-pipe instructions per step, ~1 k
            // cycles of its chain, for no accuracy the float increments keep)
            f2 Xn[4], Kn[4];
            float xn[8];
            pair_state_update(X, K, dt, xa, dK, Xn, Kn);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                xn[i] = Xn[i].hi;
                xn[4 + i] = Kn[i].hi;
            }
            KerrPoint<float> m;
            float dn[4];
            kerr_accel(xn[1], xn[2], xn[3], xn[4], xn[5], xn[6], xn[7], a, dn[0], dn[1], dn[2], dn[3], m);
            int w1;
            const float r_new = m.r;
            const float dtn = reference_dt(r_new, reh, div, tol, w1);
            if (dtn == 0.0f) {
                // the step is rejected and the ray stays frozen (geodesics.py:263-267)
                flags |= ZM_END;
                msg.why[lane] = w1;
                msg.steps[lane] = steps;
                active = false;
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) { X[i] = Xn[i]; K[i] = Kn[i]; }
#pragma unroll
                for (int i = 0; i < 8; i++) xf[i] = xn[i];
#pragma unroll
                for (int i = 0; i < 4; i++) d1[i] = dn[i];
                flags |= ZM_SAMPLE | (inzone ? ZM_ZONE : 0u);
#pragma unroll
                for (int i = 0; i < 7; i++) msg.s[i][lane] = xn[1 + i];
                msg.m[0][lane] = m.r;
                msg.m[1][lane] = m.f;
                msg.m[2][lane] = m.l1;
                msg.m[3][lane] = m.l2;
                msg.m[4][lane] = m.l3;
                msg.dt[lane] = dt;
                dt = dtn;
                ++steps;
                ++b_steps;
                if (inzone) {
                    ++zone_steps;
                    run_max = max(run_max, ++run);
                }
                const float dr = r_new - r_cur;
                if (steps >= nmax - 1) {
                    // trajectory rows stop at N-1: step N-1 never reaches the solve
                    flags |= ZM_END;
                    msg.why[lane] = MK_RAY_MAXSTEPS;
                    msg.steps[lane] = steps;
                    active = false;
                } else if (escape && !inzone && r_new > r_out && dr > 0.0f) {
                    // outbound beyond every snapshot cell: no sample follows
                    flags |= ZM_END;
                    msg.why[lane] = MK_RAY_ESCAPED;
                    msg.steps[lane] = steps;
                    active = false;
                } else if (inzone && r_new >= (float)R_TURN && dr > 0.0f) {
                    // outbound past the photon-ring region: on to the ray's end
                    // in float pairs, as phase C continues its parked rays,
                    // with no renormalisation (one here changed no pixel by
                    // more than 1.5e-9 of its value at 256x256 and cost the
                    // chain ~6 k cycles per ray)
                    inzone = false;
                    atomicAdd(&ws->zone_exits, 1ull);
                } else if (inzone && ((dr_prev < 0.0f && dr > 0.0f) || (dr_prev > 0.0f && dr < 0.0f))) {
                    // a radial turning point: renormalise to null in
                    // double-float arithmetic and re-evaluate the first stage
                    // of the next step there (in binary64 its ~100 FP64-pipe
                    // instructions held the whole warp ~6.5 k cycles each
                    // time, whichever of its lanes turned)
                    const dd k0 = renull_k0_dd(dd(X[1].hi, X[1].lo), dd(X[2].hi, X[2].lo), dd(X[3].hi, X[3].lo),
                                               dd(K[0].hi, K[0].lo), dd(K[1].hi, K[1].lo), dd(K[2].hi, K[2].lo),
                                               dd(K[3].hi, K[3].lo), ad);
                    K[0] = {k0.hi, k0.lo};
                    xf[4] = K[0].hi;
                    kerr_accel(xf[1], xf[2], xf[3], xf[4], xf[5], xf[6], xf[7], a, d1[0], d1[1], d1[2], d1[3]);
                }
                r_cur = r_new;
                dr_prev = dr;
            }
        }
        msg.idx[lane] = ray;
        msg.flags[lane] = flags | (any ? 0u : ZM_DONE);
        __syncwarp();
        if (!(withhold && it == 0)) mbar_arrive(&zs.full[sl]);
        if (!any) {
            // one ZM_DONE message for each of the other samplers
            for (int e = 1; e < ZONE_SAMPLERS; ++e) {
                const int jt = it + e, se = jt % ZONE_SLOTS;
                if (jt >= ZONE_SLOTS &&
                    !zone_wait(&zs.empty[se], (unsigned)((jt / ZONE_SLOTS) - 1) & 1u, zs, limit_ns)) {
                    zone_fail(zs, ws);
                    return;
                }
                zs.slot[se].flags[lane] = ZM_DONE;
                zs.slot[se].idx[lane] = -1;
                __syncwarp();
                mbar_arrive(&zs.full[se]);
            }
            break;
        }
    }
    if (zone_steps) atomicAdd(&ws->steps_fp64, (unsigned long long)zone_steps);
    if (b_steps) atomicAdd(&ws->steps_b, (unsigned long long)b_steps);
    if (run_max) atomicMax(&ws->zone_run_max, (unsigned long long)run_max);
}

// Sampler k (warp 1 + k) of the pipeline: messages k, k + 3, k + 6, ...
__device__ __forceinline__ void zone_sample(int k, const mk_request *__restrict__ reqs,
                                            const mk_snapshot_view *__restrict__ snaps, RenderWorkspace *ws,
                                            const RayRecord *q64, ZoneShared &zs, unsigned long long limit_ns) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int zone_samples = 0, b_samples = 0;
    // constants of the ray this lane's last message belonged to
    int cur = -1, rq = 0;
    int64_t pix = 0;
    SynchroF32 sc[MK_MAX_NU];
    RayF32 rc;
    mk_snapshot_view sv;
    SnapF32 sf;
    BlockCacheF bc;
    bc.key = -1;
    bc.mb = -1;
    for (int j = k;; j += ZONE_SAMPLERS) {
        const int sl = j % ZONE_SLOTS;
        const ZoneSlot &msg = zs.slot[sl];
        if (!zone_wait(&zs.full[sl], (unsigned)(j / ZONE_SLOTS) & 1u, zs, limit_ns)) {
            zone_fail(zs, ws);
            return;
        }
        const unsigned flags = msg.flags[lane];
        const int idx = msg.idx[lane];
        float x[8], dt = 0.0f;
        KerrPoint<float> m;
        int steps = 0, why = 0;
        if (flags & ZM_SAMPLE) {
            x[0] = 0.0f;  // x^0 is not read
#pragma unroll
            for (int i = 0; i < 7; i++) x[1 + i] = msg.s[i][lane];
            m.r = msg.m[0][lane];
            m.f = msg.m[1][lane];
            m.l1 = msg.m[2][lane];
            m.l2 = msg.m[3][lane];
            m.l3 = msg.m[4][lane];
            dt = msg.dt[lane];
        }
        if (flags & ZM_END) {
            steps = msg.steps[lane];
            why = msg.why[lane];
        }
        __syncwarp();
        mbar_arrive(&zs.empty[sl]);  // the slot is free for message j + ZONE_SLOTS
        if ((flags & (ZM_START | ZM_SAMPLE | ZM_END)) && idx != cur) {
            cur = idx;
            const RayRecord &q = q64[idx];
            rq = q.rq;
            const mk_request &R = reqs[rq];
            pix = q.ray - R.ray_offset;
            rc = ray_f32(R);
            sv = snaps[R.snapshot];
            sf = snap_f32(sv);
            bc.key = -1;
#pragma unroll
            for (int ch = 0; ch < MK_MAX_NU; ch++)
                if (ch < R.nnu) sc[ch] = synchro_consts(R.nu[ch]);
        }
        // the sample itself depends on no other message
        float em[MK_MAX_NU], ab[MK_MAX_NU];
        bool sampled = false;
        if (flags & ZM_SAMPLE) {
            CellPosF c;
            if (locate_f32_cached(sv, sf, x[1], x[2], x[3], c, bc)) {
                emission_f32_at(sv, c, rc, x, m, sc, em, ab);
                sampled = true;
            }
        }
        float I0[MK_MAX_NU], Ic0[MK_MAX_NU], P0[MK_MAX_NU], tau0 = 0.0f;
        int n0 = 0;
        if (flags & ZM_START) {
            // the sums the ray arrived with (read before waiting for the fold)
            const RayRecord &q = q64[idx];
#pragma unroll
            for (int ch = 0; ch < MK_MAX_NU; ch++) {
                I0[ch] = (float)q.I[ch];
                Ic0[ch] = (float)((double)I0[ch] - q.I[ch]);
                P0[ch] = (float)q.P[ch];
            }
            tau0 = (float)q.max_tau;
            n0 = q.nsamples;
        }
        // fold in message order
        if (!zone_wait_fold(zs, j, limit_ns)) {
            zone_fail(zs, ws);
            return;
        }
        if (flags & ZM_START) {
#pragma unroll
            for (int ch = 0; ch < MK_MAX_NU; ch++) {
                zs.I[ch][lane] = I0[ch];
                zs.Ic[ch][lane] = Ic0[ch];
                zs.P[ch][lane] = P0[ch];
            }
            zs.max_tau[lane] = tau0;
            zs.nsamples[lane] = n0;
        }
        if (sampled) {
            // sample_f32's fold, term for term
            const float w = -dt * rc.L_unit;
            float max_tau = zs.max_tau[lane];
#pragma unroll
            for (int ch = 0; ch < MK_MAX_NU; ch++) {
                if (ch < rc.nnu) {
                    const float I = zs.I[ch][lane], Ic = zs.Ic[ch][lane];
                    const float tau = w * ab[ch];
                    const float y = (w * em[ch]) * zs.P[ch][lane] - Ic;
                    const float t = I + y;
                    zs.Ic[ch][lane] = (t - I) - y;
                    zs.I[ch][lane] = t;
                    zs.P[ch][lane] *= (1.0f - tau);
                    max_tau = fmaxf(max_tau, tau);
                }
            }
            zs.max_tau[lane] = max_tau;
            ++zs.nsamples[lane];
            if (flags & ZM_ZONE) ++zone_samples;
            ++b_samples;
        }
        if (flags & ZM_END) {
            float I[MK_MAX_NU], Ic[MK_MAX_NU];
#pragma unroll
            for (int ch = 0; ch < MK_MAX_NU; ch++) { I[ch] = zs.I[ch][lane]; Ic[ch] = zs.Ic[ch][lane]; }
            finish_ray_f32(reqs[rq], pix, I, Ic, steps, why, zs.nsamples[lane], zs.max_tau[lane], ws);
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();  // this warp's sums before the counter
            *(volatile int *)&zs.folded = j + 1;
        }
        if (__any_sync(FULL, (flags & ZM_DONE) != 0u)) break;
    }
    if (zone_samples) atomicAdd(&ws->samples_fp64, (unsigned long long)zone_samples);
    if (b_samples) atomicAdd(&ws->samples_b, (unsigned long long)b_samples);
}

__global__ void __launch_bounds__(ZONE_THREADS)
render_zone_kernel(const mk_request *__restrict__ reqs, const mk_snapshot_view *__restrict__ snaps,
                   RenderWorkspace *ws, const RayRecord *q64, long long capacity, int escape,
                   unsigned long long wait_ns, int withhold) {
    __shared__ ZoneShared zs;
    if (threadIdx.x == 0) {
        for (int s = 0; s < ZONE_SLOTS; s++) {
            mbar_init(&zs.full[s], 32);
            mbar_init(&zs.empty[s], 32);
        }
        zs.folded = 0;
        zs.abort = 0;
    }
    __syncthreads();
    const int w = threadIdx.x >> 5;
    if (w == 0)
        zone_integrate(reqs, snaps, ws, q64, capacity, escape, zs, wait_ns, withhold);
    else
        zone_sample(w - 1, reqs, snaps, ws, q64, zs, wait_ns);
}

// Initial states of every camera ray of a launch as float pairs (x^mu
// then k^mu, hi and lo words: 64 B a ray), for mixed-form launches larger
// than one wave of phase A: there each thread of phase A takes a new ray
// many times, and the camera setup, run for whichever lanes refill in a
// given step, held the whole warp each time.  Here it runs once per ray,
// fully parallel, and phase A loads four 16-byte words instead.  Grid
// cameras in double-float (camera_ray_pair), equator cameras in binary64
// (camera_ray).
__global__ void __launch_bounds__(RENDER_THREADS)
camera_states_kernel(const mk_request *__restrict__ reqs, int nreq, long long total, const mk_job *job,
                     float4 *__restrict__ out) {
    if (job) {
        nreq = job->nreq;
        total = job->total_rays;
    }
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const int rq = find_request(reqs, nreq, p);
        if (!ray_in_request(reqs, nreq, p)) continue;
        f2 X[4], K[4];
        camera_pair(reqs[rq].camera, p - reqs[rq].ray_offset, X, K);
        out[4 * p + 0] = make_float4(X[0].hi, X[0].lo, X[1].hi, X[1].lo);
        out[4 * p + 1] = make_float4(X[2].hi, X[2].lo, X[3].hi, X[3].lo);
        out[4 * p + 2] = make_float4(K[0].hi, K[0].lo, K[1].hi, K[1].lo);
        out[4 * p + 3] = make_float4(K[2].hi, K[2].lo, K[3].hi, K[3].lo);
    }
}

// FP32 render phase.  SRC_CAMERA: mixed-form phase A from the camera; mode
// F32_HANDOFF hands rays near the hole to the near-hole queue, F32_PARK
// parks rays leaving the photon-ring region outward in the FP32 queue.
// SRC_QUEUE: the FP32 continuation over that queue (mode 0).
// The ray state is a float pair per component (rk4_step_pair); the
// accelerations, the sampling and the emission are plain float.
template <int SRC, int MINB>
__global__ void __launch_bounds__(RENDER_THREADS, MINB)
render_f32_kernel(const mk_request *__restrict__ reqs, int nreq, long long total_camera,
                  const mk_snapshot_view *__restrict__ snaps, RenderWorkspace *ws, RayRecord *q64, RayRecord *q32,
                  long long capacity, const mk_job *job, int mode, const float4 *__restrict__ cam) {
    if (job) {
        nreq = job->nreq;
        total_camera = job->total_rays;
    }
    // the requests' float constants, sized at launch by the request count
    // (MK_MAX_REQUESTS_MIXED for a job read from the device): shared memory
    // the table does not take stays L1 for the gathers
    extern __shared__ __align__(16) unsigned char s_req_raw[];
    ReqF32 *s_req = reinterpret_cast<ReqF32 *>(s_req_raw);
    for (int q = threadIdx.x; q < min(nreq, MK_MAX_REQUESTS_MIXED); q += blockDim.x) fill_req_f32(reqs[q], snaps, s_req[q]);
    __syncthreads();
    unsigned long long *counter = SRC == SRC_CAMERA ? &ws->counter : &ws->q32_next;
    const long long total =
        SRC == SRC_CAMERA ? total_camera
                          : min((long long)*(volatile unsigned long long *)&ws->q32_count, capacity);
    bool active = false, exhausted = false;
    int rq = 0, steps = 0, nsamples = 0, why = MK_RAY_ACTIVE;
    long long ray = 0;
    int64_t pix = 0;
    f2 X[4], K[4];
    float d1[4], dt = 0.0f, r_cur = 0.0f, max_tau = 0.0f;
    float I[MK_MAX_NU], Ic[MK_MAX_NU], P[MK_MAX_NU];
    int queue_steps = 0, queue_samples = 0;  // SRC_QUEUE: this thread's share of the launch's work

    for (;;) {
        const long long idx = fetch(!active && !exhausted, counter, total);
        if (idx == -1) exhausted = true;
        if (idx >= 0 && (SRC != SRC_CAMERA || ray_in_request(reqs, nreq, idx))) {
            double s64[8];  // a queue record's state
            if (SRC == SRC_CAMERA) {
                ray = idx;
                rq = find_request(reqs, nreq, ray);
                pix = ray - reqs[rq].ray_offset;
                steps = nsamples = 0;
                max_tau = 0.0f;
#pragma unroll
                for (int ch = 0; ch < MK_MAX_NU; ch++) { I[ch] = 0.0f; Ic[ch] = 0.0f; P[ch] = 1.0f; }
            } else {
                const RayRecord &q = q32[idx];
#pragma unroll
                for (int i = 0; i < 8; i++) s64[i] = q.s[i];
#pragma unroll
                for (int ch = 0; ch < MK_MAX_NU; ch++) {
                    I[ch] = (float)q.I[ch];
                    Ic[ch] = (float)((double)I[ch] - q.I[ch]);
                    P[ch] = (float)q.P[ch];
                }
                max_tau = (float)q.max_tau;
                ray = q.ray;
                steps = q.steps;
                nsamples = q.nsamples;
                rq = q.rq;
                pix = ray - reqs[rq].ray_offset;
                if (mode & F32_RENULL) renull_fp64(s64, reqs[rq].camera.bhspin);
            }
            const mk_request &R = reqs[rq];
            if (rq >= MK_MAX_REQUESTS_MIXED) {  // beyond the launch's request table
                atomicAdd(&ws->overflow, 1ull);
                finish_ray_f32(R, pix, I, Ic, steps, MK_RAY_NAN, nsamples, max_tau, ws);
            } else {
                const ReqF32 &Q = s_req[rq];
                if (SRC == SRC_CAMERA) {
                    if (cam) {  // precomputed by camera_states_kernel
                        const float4 c0 = cam[4 * ray], c1 = cam[4 * ray + 1], c2 = cam[4 * ray + 2],
                                     c3 = cam[4 * ray + 3];
                        X[0] = {c0.x, c0.y};
                        X[1] = {c0.z, c0.w};
                        X[2] = {c1.x, c1.y};
                        X[3] = {c1.z, c1.w};
                        K[0] = {c2.x, c2.y};
                        K[1] = {c2.z, c2.w};
                        K[2] = {c3.x, c3.y};
                        K[3] = {c3.z, c3.w};
                    } else if (Q.cam_grid) {
                        camera_ray_pair(Q.cam, Q.cam_pixels, pix, X, K);
                    } else {
                        camera_pair(R.camera, pix, X, K);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 4; i++) { X[i] = f2_from(s64[i]); K[i] = f2_from(s64[4 + i]); }
                }
                KerrPoint<float> m;
                kerr_accel(X[1].hi, X[2].hi, X[3].hi, K[0].hi, K[1].hi, K[2].hi, K[3].hi, Q.a, d1[0], d1[1], d1[2],
                           d1[3], m);
                r_cur = m.r;
                dt = reference_dt(r_cur, Q.reh, Q.rc.div, Q.rc.tol, why);
                if (dt == 0.0f || R.policy.nmax < 2) {
                    if (why == MK_RAY_ACTIVE) why = MK_RAY_MAXSTEPS;
                    finish_ray_f32(R, pix, I, Ic, steps, why, nsamples, max_tau, ws);
                } else {
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (SRC == SRC_QUEUE && queue_steps) {
                atomicAdd(&ws->steps_c, (unsigned long long)queue_steps);
                atomicAdd(&ws->samples_c, (unsigned long long)queue_samples);
            }
            break;
        }
        if (active) {
            const mk_request &R = reqs[rq];
            const ReqF32 &Q = s_req[rq];  // the request's constants, from shared memory
            f2 Xn[4], Kn[4];
            float dn[4];
            rk4_step_pair(X, K, d1, dt, Q.a, Xn, Kn);
            const mk_snapshot_view &sv = snaps[R.snapshot];
            CellPosF cell;
            const bool inside = locate_f32(sv, Q.sf, Xn[1].hi, Xn[2].hi, Xn[3].hi, cell);
            if (inside) prefetch_cells_f32(sv, cell);
            KerrPoint<float> m;
            kerr_accel(Xn[1].hi, Xn[2].hi, Xn[3].hi, Kn[0].hi, Kn[1].hi, Kn[2].hi, Kn[3].hi, Q.a, dn[0], dn[1],
                       dn[2], dn[3], m);
            int w1;
            const float r_new = m.r;
            const float dtn = reference_dt(r_new, Q.reh, Q.rc.div, Q.rc.tol, w1);
            if (dtn == 0.0f) {
                finish_ray_f32(R, pix, I, Ic, steps, w1, nsamples, max_tau, ws);
                active = false;
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) { X[i] = Xn[i]; K[i] = Kn[i]; d1[i] = dn[i]; }
                const float dt_used = dt;
                dt = dtn;
                ++steps;
                const float sh[8] = {X[0].hi, X[1].hi, X[2].hi, X[3].hi, K[0].hi, K[1].hi, K[2].hi, K[3].hi};
                if (inside) sample_f32(sv, cell, Q.rc, sh, m, dt_used, I, Ic, P, Q.sc, nsamples, max_tau);
                if (SRC == SRC_QUEUE) {
                    ++queue_steps;
                    queue_samples += inside;
                }
                if (steps >= R.policy.nmax - 1) {
                    finish_ray_f32(R, pix, I, Ic, steps, MK_RAY_MAXSTEPS, nsamples, max_tau, ws);
                    active = false;
                } else if ((mode & F32_ESCAPE) && r_new > Q.sf.r_out && r_new > r_cur) {
                    // outbound beyond every snapshot cell: no sample follows
                    finish_ray_f32(R, pix, I, Ic, steps, MK_RAY_ESCAPED, nsamples, max_tau, ws);
                    active = false;
                } else if (SRC == SRC_CAMERA && (mode & (F32_HANDOFF | F32_PARK))) {
                    // near the horizon or inbound in the photon-ring region: to
                    // the near-hole queue; outbound past it (F32_PARK): to the
                    // FP32 continuation queue, whose kernel runs beside the
                    // near-hole one
                    const bool to64 = (mode & F32_HANDOFF) &&
                                      (r_new < (float)R_FP64 || (r_new < (float)R_TURN && r_new < r_cur));
                    const bool park = !to64 && (mode & F32_PARK) && r_new >= (float)R_TURN && r_new > r_cur;
                    if (to64 || park) {
                        const unsigned long long slot = atomicAdd(to64 ? &ws->q64_count : &ws->q32_count, 1ull);
                        if ((long long)slot < capacity) {
                            RayRecord &q = (to64 ? q64 : q32)[slot];
#pragma unroll
                            for (int i = 0; i < 4; i++) { q.s[i] = f2_to(X[i]); q.s[4 + i] = f2_to(K[i]); }
#pragma unroll
                            for (int ch = 0; ch < MK_MAX_NU; ch++) {
                                q.I[ch] = (double)I[ch] - (double)Ic[ch];
                                q.P[ch] = (double)P[ch];
                            }
                            q.max_tau = (double)max_tau;
                            q.ray = ray;
                            q.steps = steps;
                            q.nsamples = nsamples;
                            q.rq = rq;
                            active = false;
                        } else {
                            atomicAdd(&ws->overflow, 1ull);
                        }
                    }
                }
                r_cur = r_new;
            }
        }
    }
}

template <typename K>
static int blocks_per_sm(K kernel, int slot) {
    static int cached[64][8] = {{0}};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && cached[dev][slot]) return cached[dev][slot];
    int nb = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, RENDER_THREADS, 0);
    if (nb < 1) nb = 1;
    if (dev < 64) cached[dev][slot] = nb;
    return nb;
}

static unsigned persistent_grid(int per_sm, int64_t rays) {
    int64_t grid = (int64_t)device_sm_count() * per_sm;
    const int64_t need = (rays + RENDER_THREADS - 1) / RENDER_THREADS;
    if (grid > need) grid = need;
    return (unsigned)(grid < 1 ? 1 : grid);
}




extern "C" int mk_set_tuning(const char *name, int64_t value) {
    MK_REQUIRE(name, MK_ERR_ARG, "mk_set_tuning: null name");
    if (!strcmp(name, "fp64_rays_per_warp")) {
        MK_REQUIRE(value == 1 || value == 2 || value == 4 || value == 8 || value == 16 || value == 32, MK_ERR_ARG,
                   "mk_set_tuning: fp64_rays_per_warp must be a power of two in 1..32");
        g_fp64_rays_per_warp = (int)value;
        return MK_OK;
    }
    if (!strcmp(name, "f32_blocks_per_sm")) {
        MK_REQUIRE(value == 0 || (value >= 3 && value <= 5), MK_ERR_ARG,
                   "mk_set_tuning: f32_blocks_per_sm must be 0 (automatic), 3, 4 or 5");
        g_f32_blocks = (int)value;
        return MK_OK;
    }
    if (!strcmp(name, "phase_events")) {
        MK_REQUIRE(value == 0 || value == 1, MK_ERR_ARG, "mk_set_tuning: phase_events must be 0 or 1");
        g_phase_events = (int)value;
        return MK_OK;
    }
    if (!strcmp(name, "escape_cut")) {
        MK_REQUIRE(value == 0 || value == 1, MK_ERR_ARG, "mk_set_tuning: escape_cut must be 0 or 1");
        g_escape_cut = (int)value;
        return MK_OK;
    }
    if (!strcmp(name, "zone_wait_ns")) {
        MK_REQUIRE(value >= 1 && value <= 60000000000ll, MK_ERR_ARG,
                   "mk_set_tuning: zone_wait_ns must lie in 1 .. 6e10");
        g_zone_wait_ns = (unsigned long long)value;
        return MK_OK;
    }
    if (!strcmp(name, "zone_wait_test")) {
        MK_REQUIRE(value == 0 || value == 1, MK_ERR_ARG, "mk_set_tuning: zone_wait_test must be 0 or 1");
        g_zone_wait_test = (int)value;
        return MK_OK;
    }
    if (!strcmp(name, "fp64_zone")) {
        MK_REQUIRE(value == 0 || value == 1, MK_ERR_ARG, "mk_set_tuning: fp64_zone must be 0 or 1");
        g_fp64_zone = (int)value;
        return MK_OK;
    }
    MK_REQUIRE(false, MK_ERR_ARG, "mk_set_tuning: unknown parameter '%s'", name);
}

// Scratch of a launch: the counter header, then (mixed forms) the two ray
// queues, then -- for launches larger than one wave of phase A at 4 blocks
// per SM -- the precomputed camera states (64 bytes a ray).  A workspace of
// the size without them (ws_base) still renders: phase A then computes the
// camera states itself.
static bool mixed_form(int32_t precision) {
    return precision == MK_MIXED || precision == MK_MIXED_DF || precision == MK_MIXED_STRICT;
}
static size_t ws_base(int64_t rays, int32_t precision) {
    return mixed_form(precision) ? WS_HEADER + 2 * (size_t)rays * sizeof(RayRecord) : WS_HEADER;
}
size_t render_ws_base(int64_t rays, int32_t precision) { return ws_base(rays, precision); }
static bool camera_precompute(int64_t rays, int32_t precision) {
    return mixed_form(precision) && rays > (int64_t)device_sm_count() * 4 * RENDER_THREADS;
}

}  // namespace mk

extern "C" size_t mk_render_workspace_bytes(int64_t total_rays, int32_t precision) {
    if (total_rays < 0) return 0;
    return mk::ws_base(total_rays, precision) +
           (mk::camera_precompute(total_rays, precision) ? 8 * sizeof(double) * (size_t)total_rays : 0);
}

namespace mk {

static int launch_render(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays, int64_t max_rays,
                         const mk_job *job_dev, const mk_snapshot_view *snaps_dev, int32_t precision,
                         void *workspace_dev, size_t workspace_bytes, cudaStream_t st) {
    MK_CUDA(cudaMemsetAsync(workspace_dev, 0, WS_HEADER, st));
    if (max_rays == 0) return MK_OK;
    RenderWorkspace *ws = (RenderWorkspace *)workspace_dev;
    int rc = phase_mark(st, 0);
    if (rc != MK_OK) return rc;
    if (precision == MK_FP64) {
        const unsigned grid = persistent_grid(blocks_per_sm(render_fp64_kernel<SRC_CAMERA>, 0), max_rays);
        render_fp64_kernel<SRC_CAMERA><<<grid, RENDER_THREADS, 0, st>>>(reqs_dev, nreq, (long long)total_rays,
                                                                        snaps_dev, ws, nullptr, nullptr, 0, 1,
                                                                        job_dev);
        MK_LAUNCHED("render_fp64_kernel");
        return phase_mark(st, 1);
    }
    RayRecord *q64 = (RayRecord *)((char *)workspace_dev + WS_HEADER);
    RayRecord *q32 = q64 + max_rays;
    const long long cap = (long long)max_rays;
    float4 *cam = nullptr;
    if (camera_precompute(max_rays, precision) &&
        workspace_bytes >= ws_base(max_rays, precision) + 4 * sizeof(float4) * (size_t)max_rays) {
        cam = reinterpret_cast<float4 *>(q32 + max_rays);
        const int64_t grid = std::min<int64_t>((max_rays + RENDER_THREADS - 1) / RENDER_THREADS,
                                               (int64_t)device_sm_count() * 16);
        camera_states_kernel<<<(unsigned)grid, RENDER_THREADS, 0, st>>>(reqs_dev, nreq, (long long)total_rays,
                                                                         job_dev, cam);
        MK_LAUNCHED("camera_states_kernel");
    }
    int f32_blocks = g_f32_blocks;
    if (f32_blocks == 0)
        f32_blocks = max_rays > (int64_t)device_sm_count() * 4 * RENDER_THREADS ? 5 : 4;
    // MK_MIXED parks the outbound rays: its FP32 continuation then runs beside
    // the near-hole phase instead of after it
    const int mode = (g_fp64_zone ? F32_HANDOFF : 0) | (precision == MK_MIXED ? F32_PARK : 0) |
                     (g_escape_cut ? F32_ESCAPE : 0);
    // dynamic shared memory of the FP32 kernels: their request table
    const size_t req_smem =
        (size_t)(job_dev ? MK_MAX_REQUESTS_MIXED : std::min<int32_t>(nreq, MK_MAX_REQUESTS_MIXED)) * sizeof(ReqF32);
    if (f32_blocks == 5)
        render_f32_kernel<SRC_CAMERA, 5>
            <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_CAMERA, 5>, 5), max_rays), RENDER_THREADS, req_smem,
               st>>>(reqs_dev, nreq, (long long)total_rays, snaps_dev, ws, q64, q32, cap, job_dev, mode, cam);
    else if (f32_blocks == 4)
        render_f32_kernel<SRC_CAMERA, 4>
            <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_CAMERA, 4>, 1), max_rays), RENDER_THREADS, req_smem,
               st>>>(reqs_dev, nreq, (long long)total_rays, snaps_dev, ws, q64, q32, cap, job_dev, mode, cam);
    else
        render_f32_kernel<SRC_CAMERA, 3>
            <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_CAMERA, 3>, 2), max_rays), RENDER_THREADS, req_smem,
               st>>>(reqs_dev, nreq, (long long)total_rays, snaps_dev, ws, q64, q32, cap, job_dev, mode, cam);
    MK_LAUNCHED("render_f32_kernel (camera)");
    if ((rc = phase_mark(st, 1)) != MK_OK) return rc;
    // The FP32 continuation over the FP32 queue; its size is only known on
    // the device, so the grid is persistent.
    // MK_MIXED's FP32 queue holds parked phase-A rays; the other mixed forms'
    // hold the near-hole phase's exits
    const int qmode = (precision == MK_MIXED ? 0 : F32_RENULL) | (g_escape_cut ? F32_ESCAPE : 0);
    auto launch_f32_queue = [&](cudaStream_t s, int f32_blocks) {
        if (f32_blocks == 5)
            render_f32_kernel<SRC_QUEUE, 5>
                <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_QUEUE, 5>, 6), max_rays), RENDER_THREADS, req_smem,
                   s>>>(reqs_dev, nreq, 0, snaps_dev, ws, q64, q32, cap, job_dev, qmode, nullptr);
        else if (f32_blocks == 4)
            render_f32_kernel<SRC_QUEUE, 4>
                <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_QUEUE, 4>, 3), max_rays), RENDER_THREADS, req_smem,
                   s>>>(reqs_dev, nreq, 0, snaps_dev, ws, q64, q32, cap, job_dev, qmode, nullptr);
        else
            render_f32_kernel<SRC_QUEUE, 3>
                <<<persistent_grid(blocks_per_sm(render_f32_kernel<SRC_QUEUE, 3>, 4), max_rays), RENDER_THREADS, req_smem,
                   s>>>(reqs_dev, nreq, 0, snaps_dev, ws, q64, q32, cap, job_dev, qmode, nullptr);
    };
    // The near-hole queue: persistent grids, small blocks, so the few rays
    // near the hole spread over every SM sub-partition (they are
    // latency-bound: one FP64 warp instruction holds a sub-partition's FP64
    // unit for tens of cycles on this part).
    if (precision == MK_MIXED) {
        // phase B (near the hole, then on to each ray's end) on the caller's
        // stream and phase C (the parked outbound rays) on the side stream,
        // at the same time: they share no ray and no counter
        SideStream *side = nullptr;
        if ((rc = side_stream(&side)) != MK_OK) return rc;
        MK_CUDA(cudaEventRecord(side->fork, st));
        MK_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
        render_zone_kernel<<<(unsigned)device_sm_count() * 4, ZONE_THREADS, 0, st>>>(reqs_dev, snaps_dev, ws, q64,
                                                                                      cap, g_escape_cut,
                                                                                      g_zone_wait_ns,
                                                                                      g_zone_wait_test);
        MK_LAUNCHED("render_zone_kernel");
        // beside the near-hole pipeline (168 registers a thread) phase C runs
        // its spill-free 3-block build unless a tuning asks otherwise (phase
        // C 0.92 -> 0.84 ms at 256x256, 11.1 -> 10.9 ms on the 1024x1024
        // stress render, against the 128-register 4-block and 96-register
        // 5-block builds, which spill)
        launch_f32_queue(side->s, g_f32_blocks ? f32_blocks : 3);
        MK_LAUNCHED("render_f32_kernel (queue)");
        if ((rc = phase_mark(st, 2)) != MK_OK) return rc;
        if ((rc = phase_mark(side->s, 3, 1)) != MK_OK) return rc;
        MK_CUDA(cudaEventRecord(side->join, side->s));
        MK_CUDA(cudaStreamWaitEvent(st, side->join, 0));
        return MK_OK;
    }
    {
        const int per_warp = g_fp64_rays_per_warp;
        const int stride = 32 / per_warp;
        const unsigned grid = (unsigned)device_sm_count() * (per_warp >= 32 ? 4 : 16);
        if (precision == MK_MIXED_STRICT)
            render_fp64_kernel<SRC_QUEUE, double>
                <<<grid, 32, 0, st>>>(reqs_dev, nreq, 0, snaps_dev, ws, q64, q32, cap, stride, job_dev);
        else
            render_fp64_kernel<SRC_QUEUE, dd>
                <<<grid, 32, 0, st>>>(reqs_dev, nreq, 0, snaps_dev, ws, q64, q32, cap, stride, job_dev);
        MK_LAUNCHED("render_fp64_kernel (queue)");
    }
    if ((rc = phase_mark(st, 2)) != MK_OK) return rc;
    launch_f32_queue(st, f32_blocks);
    MK_LAUNCHED("render_f32_kernel (queue)");
    return phase_mark(st, 3);
}

}  // namespace mk

extern "C" int mk_render(const mk_request *reqs_dev, int32_t nreq, int64_t total_rays,
                         const mk_snapshot_view *snaps_dev, int32_t nsnap, int32_t precision,
                         void *workspace_dev, size_t workspace_bytes, void *stream) {
    MK_REQUIRE(reqs_dev && snaps_dev && workspace_dev, MK_ERR_ARG, "mk_render: null pointer");
    MK_REQUIRE(nreq > 0 && nsnap > 0 && total_rays >= 0, MK_ERR_ARG, "mk_render: bad sizes");
    MK_REQUIRE(precision >= MK_FP64 && precision <= MK_MIXED_STRICT, MK_ERR_ARG, "mk_render: unknown precision %d",
               (int)precision);
    const size_t need = mk::ws_base(total_rays, precision);
    MK_REQUIRE(workspace_bytes >= need, MK_ERR_ARG, "mk_render: workspace of %zu bytes, need %zu",
               workspace_bytes, need);
    MK_REQUIRE(precision == MK_FP64 || nreq <= MK_MAX_REQUESTS_MIXED, MK_ERR_LIMIT,
               "mk_render: %d requests in one mixed-form launch, at most %d", (int)nreq, MK_MAX_REQUESTS_MIXED);
    MK_REQUIRE(((uintptr_t)workspace_dev & 15) == 0, MK_ERR_ARG, "mk_render: workspace not 16-byte aligned");
    return mk::launch_render(reqs_dev, nreq, total_rays, total_rays, nullptr, snaps_dev, precision, workspace_dev,
                             workspace_bytes, mk::as_stream(stream));
}

extern "C" int mk_render_job(const mk_job *job_dev, const mk_request *reqs_dev, const mk_snapshot_view *snaps_dev,
                             int32_t precision, int64_t max_rays, void *workspace_dev, size_t workspace_bytes,
                             void *stream) {
    MK_REQUIRE(job_dev && reqs_dev && snaps_dev && workspace_dev, MK_ERR_ARG, "mk_render_job: null pointer");
    MK_REQUIRE(max_rays >= 0, MK_ERR_ARG, "mk_render_job: negative max_rays");
    MK_REQUIRE(precision >= MK_FP64 && precision <= MK_MIXED_STRICT, MK_ERR_ARG,
               "mk_render_job: unknown precision %d", (int)precision);
    const size_t need = mk::ws_base(max_rays, precision);
    MK_REQUIRE(workspace_bytes >= need, MK_ERR_ARG, "mk_render_job: workspace of %zu bytes, need %zu",
               workspace_bytes, need);
    MK_REQUIRE(((uintptr_t)workspace_dev & 15) == 0, MK_ERR_ARG, "mk_render_job: workspace not 16-byte aligned");
    return mk::launch_render(reqs_dev, 1, 0, max_rays, job_dev, snaps_dev, precision, workspace_dev,
                             workspace_bytes, mk::as_stream(stream));
}

// the allocation-free entry point sizes its static workspace from these
static_assert(mk::WS_HEADER == 256 && sizeof(mk::RayRecord) == 160, "MK_NOALLOC_MAX_MIXED_RAYS assumes 256 + 320 B/ray");

extern "C" int mk_render_phase_ms(float *ms_out, int32_t *nphases) {
    MK_REQUIRE(ms_out && nphases, MK_ERR_ARG, "mk_render_phase_ms: null pointer");
    MK_REQUIRE(mk::g_phase_dev >= 0 && mk::g_phase_n > 0, MK_ERR_ARG,
               "mk_render_phase_ms: no render recorded its phases (set the phase_events tuning first)");
    int cur = 0;
    MK_CUDA(cudaGetDevice(&cur));
    MK_REQUIRE(cur == mk::g_phase_dev, MK_ERR_ARG, "mk_render_phase_ms: the last render ran on device %d",
               mk::g_phase_dev);
    cudaEvent_t *ev = mk::g_phase_ev[mk::g_phase_dev];
    for (int i = 0; i < mk::g_phase_n; i++) {
        MK_CUDA(cudaEventSynchronize(ev[i + 1]));
        MK_CUDA(cudaEventElapsedTime(&ms_out[i], ev[mk::g_phase_from[i]], ev[i + 1]));
    }
    *nphases = mk::g_phase_n;
    return MK_OK;
}
