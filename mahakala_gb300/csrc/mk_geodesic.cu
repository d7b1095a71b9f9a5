// mk_geodesic.cu -- camera initialisation, geodesic integration and the
// shadow-bisection pass (geodesics.py), one thread per ray, FP64.
#include "mk_common.cuh"
#include "mk_kerr.cuh"

namespace mk {

constexpr int GEO_THREADS = 128;

__global__ void camera_kernel(mk_camera cam, int64_t npx, double *__restrict__ s0) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npx) return;
    double s[8];
    camera_ray(cam, p, s);
#pragma unroll
    for (int i = 0; i < 8; i++) s0[8 * p + i] = s[i];
}

__global__ void camera_points_kernel(const double *__restrict__ xs, const double *__restrict__ ys, int64_t n,
                                     double a, double ci, double si, double d, double *__restrict__ s0) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double s[8];
    camera_pixel(xs[p], ys[p], ci, si, d, a, s);
#pragma unroll
    for (int i = 0; i < 8; i++) s0[8 * p + i] = s[i];
}

// geodesic_integrator (geodesics.py:246-272) for one ray per thread.
// rows (N, npx, 8) / dts (N, npx) optional.
__global__ void __launch_bounds__(GEO_THREADS)
integrate_reference_kernel(const double *__restrict__ s0, int64_t npx, double a, int N, double div, double tol,
                           double *__restrict__ rows, double *__restrict__ dts, int32_t *__restrict__ Kout,
                           int32_t *__restrict__ why_out, double *__restrict__ state_out) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npx) return;
    double s[8], nw[8];
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = s0[8 * p + i];
    const double reh = radius_eh(a);
    int K = N, why = MK_RAY_MAXSTEPS;
    // a step's dt is the previous step's dtn (the same radius_cal of the same
    // state), carried instead of recomputed
    int w0;
    double dt = reference_dt(radius_cal(s[1], s[2], s[3], a), reh, div, tol, w0);
    for (int j = 0; j < N; j++) {
        int w1;
        rk4_step(s, dt, a, nw);
        const double dtn = reference_dt(radius_cal(nw[1], nw[2], nw[3], a), reh, div, tol, w1);
        if (dtn == 0.0) {
            K = j;
            why = (w0 != MK_RAY_ACTIVE) ? w0 : w1;
            if (rows)
                for (int r = j; r < N; r++)
#pragma unroll
                    for (int i = 0; i < 8; i++) rows[((int64_t)r * npx + p) * 8 + i] = s[i];
            if (dts)
                for (int r = j; r < N; r++) dts[(int64_t)r * npx + p] = 0.0;
            break;
        }
        if (rows)
#pragma unroll
            for (int i = 0; i < 8; i++) rows[((int64_t)j * npx + p) * 8 + i] = s[i];
        if (dts) dts[(int64_t)j * npx + p] = dt;
#pragma unroll
        for (int i = 0; i < 8; i++) s[i] = nw[i];
        dt = dtn;
        w0 = w1;
    }
    Kout[p] = K;
    why_out[p] = why;
#pragma unroll
    for (int i = 0; i < 8; i++) state_out[8 * p + i] = s[i];
}

// fixed-fraction vacuum policy: h = clamp(hfrac r, hmin, hmax), backwards
__global__ void __launch_bounds__(GEO_THREADS)
integrate_fixed_kernel(const double *__restrict__ s0, int64_t npx, double a, int N, double hfrac, double hmin,
                       double hmax, double capture, double r_escape, int32_t *__restrict__ Kout,
                       int32_t *__restrict__ why_out, double *__restrict__ state_out) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npx) return;
    double s[8], nw[8];
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = s0[8 * p + i];
    const double rcap = capture * radius_eh(a);
    double r = radius_cal(s[1], s[2], s[3], a);
    int st = MK_RAY_MAXSTEPS, j;
    for (j = 0; j < N; j++) {
        double h = hfrac * r;
        h = h < hmin ? hmin : (h > hmax ? hmax : h);
        rk4_step(s, -h, a, nw);
        const double rn = radius_cal(nw[1], nw[2], nw[3], a);
#pragma unroll
        for (int i = 0; i < 8; i++) s[i] = nw[i];
        if (isnan(rn) || isnan(s[4])) { st = MK_RAY_NAN; j++; break; }
        if (rn < rcap) { st = MK_RAY_CAPTURED; j++; break; }
        if (rn > r_escape && rn > r) { st = MK_RAY_ESCAPED; j++; break; }
        r = rn;
    }
    Kout[p] = j;
    why_out[p] = st;
#pragma unroll
    for (int i = 0; i < 8; i++) state_out[8 * p + i] = s[i];
}

__global__ void radius_kernel(const double *__restrict__ x, int64_t n, int64_t stride, double a,
                              double *__restrict__ r) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double *q = x + p * stride;
    r[p] = radius_cal(q[1], q[2], q[3], a);
}

// One bisection pass (select_photons_integrator, geodesics.py:354-378):
// integrate each polar ray with div 40, tol 1e-2 and record what the host
// needs to evaluate r[argmax(dt) - 1] on the trimmed trajectory.
__global__ void __launch_bounds__(GEO_THREADS)
shadow_pass_kernel(const double *__restrict__ ca, const double *__restrict__ sa, const double *__restrict__ mid,
                   int64_t n, double a, double ci, double si, double dist, int N, int32_t *__restrict__ Kout,
                   int32_t *__restrict__ best_out, double *__restrict__ best_dt_out, double *__restrict__ r_km1,
                   double *__restrict__ r_best, double *__restrict__ r_last) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double s[8], nw[8];
    camera_pixel(ca[p] * mid[p], sa[p] * mid[p], ci, si, dist, a, s);
    const double reh = radius_eh(a);
    int K = N, best = -1;
    double best_dt = -INFINITY, r_prev = nan(""), rb = nan(""), rk = nan(""), rl = nan("");
    int w0;
    double r_here = radius_cal(s[1], s[2], s[3], a);
    double dt = reference_dt(r_here, reh, 40.0, 1e-2, w0);  // carried from step to step, as above
    for (int j = 0; j < N; j++) {
        int w1;
        rk4_step(s, dt, a, nw);
        const double r_next = radius_cal(nw[1], nw[2], nw[3], a);
        const double dtn = reference_dt(r_next, reh, 40.0, 1e-2, w1);
        if (dtn == 0.0) {
            K = j;
            rk = r_prev;   // row K-1
            rl = r_here;   // frozen state = every later row
            break;
        }
        if (dt > best_dt) { best_dt = dt; best = j; rb = r_prev; }
        r_prev = r_here;
        if (j == N - 1) rl = r_here;  // row N-1 = state before step N-1
#pragma unroll
        for (int i = 0; i < 8; i++) s[i] = nw[i];
        r_here = r_next;
        dt = dtn;
    }
    Kout[p] = K;
    best_out[p] = best;
    best_dt_out[p] = best_dt;
    r_km1[p] = rk;
    r_best[p] = rb;
    r_last[p] = rl;
}

}  // namespace mk

using namespace mk;

extern "C" int mk_camera_init(const mk_camera *camera, double *s0_dev, void *stream) {
    MK_REQUIRE(camera && s0_dev, MK_ERR_ARG, "mk_camera_init: null pointer");
    MK_REQUIRE(camera->pixels > 0, MK_ERR_ARG, "mk_camera_init: pixels must be positive");
    MK_REQUIRE(camera->kind == MK_CAMERA_GRID || camera->kind == MK_CAMERA_EQUATOR, MK_ERR_ARG,
               "mk_camera_init: unknown camera kind %d", (int)camera->kind);
    const int64_t npx = camera->kind == MK_CAMERA_GRID ? (int64_t)camera->pixels * camera->pixels : camera->pixels;
    camera_kernel<<<grid_for(npx, 128), 128, 0, as_stream(stream)>>>(*camera, npx, s0_dev);
    MK_LAUNCHED("camera_kernel");
    return MK_OK;
}

extern "C" int mk_camera_points(const double *x_dev, const double *y_dev, int64_t n, double bhspin, double cos_inc,
                                double sin_inc, double distance, double *s0_dev, void *stream) {
    MK_REQUIRE(x_dev && y_dev && s0_dev, MK_ERR_ARG, "mk_camera_points: null pointer");
    MK_REQUIRE(n >= 0, MK_ERR_ARG, "mk_camera_points: negative size");
    if (n == 0) return MK_OK;
    camera_points_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(x_dev, y_dev, n, bhspin, cos_inc,
                                                                          sin_inc, distance, s0_dev);
    MK_LAUNCHED("camera_points_kernel");
    return MK_OK;
}

extern "C" int mk_integrate(const double *s0_dev, int64_t npx, double bhspin, const mk_step_policy *policy,
                            double *rows_dev, double *dt_dev, int32_t *K_dev, int32_t *why_dev, double *state_dev,
                            void *stream) {
    MK_REQUIRE(s0_dev && policy && K_dev && why_dev && state_dev, MK_ERR_ARG, "mk_integrate: null pointer");
    MK_REQUIRE(npx >= 0 && policy->nmax >= 0, MK_ERR_ARG, "mk_integrate: negative size");
    if (npx == 0) return MK_OK;
    cudaStream_t st = as_stream(stream);
    if (policy->kind == MK_POLICY_REFERENCE) {
        integrate_reference_kernel<<<grid_for(npx, GEO_THREADS), GEO_THREADS, 0, st>>>(
            s0_dev, npx, bhspin, policy->nmax, policy->div, policy->tol, rows_dev, dt_dev, K_dev, why_dev, state_dev);
        MK_LAUNCHED("integrate_reference_kernel");
    } else if (policy->kind == MK_POLICY_FIXED) {
        MK_REQUIRE(!rows_dev && !dt_dev, MK_ERR_UNSUPPORTED, "mk_integrate: rows only for the reference policy");
        integrate_fixed_kernel<<<grid_for(npx, GEO_THREADS), GEO_THREADS, 0, st>>>(
            s0_dev, npx, bhspin, policy->nmax, policy->hfrac, policy->hmin, policy->hmax, policy->capture,
            policy->r_escape, K_dev, why_dev, state_dev);
        MK_LAUNCHED("integrate_fixed_kernel");
    } else {
        MK_REQUIRE(false, MK_ERR_ARG, "mk_integrate: unknown policy %d", (int)policy->kind);
    }
    return MK_OK;
}

extern "C" int mk_radius_cal(const double *x_dev, int64_t npts, int64_t stride, double bhspin, double *r_dev,
                             void *stream) {
    MK_REQUIRE(x_dev && r_dev, MK_ERR_ARG, "mk_radius_cal: null pointer");
    MK_REQUIRE(npts >= 0 && stride >= 4, MK_ERR_ARG, "mk_radius_cal: bad size/stride");
    if (npts == 0) return MK_OK;
    radius_kernel<<<grid_for(npts, 256), 256, 0, as_stream(stream)>>>(x_dev, npts, stride, bhspin, r_dev);
    MK_LAUNCHED("radius_kernel");
    return MK_OK;
}

extern "C" int mk_shadow_pass(const double *cos_dev, const double *sin_dev, const double *mid_dev, int64_t n,
                              double bhspin, double cos_inc, double sin_inc, double distance, int32_t max_steps,
                              int32_t *K_dev, int32_t *best_dev, double *best_dt_dev, double *r_km1_dev,
                              double *r_best_dev, double *r_last_dev, void *stream) {
    MK_REQUIRE(cos_dev && sin_dev && mid_dev && K_dev && best_dev && best_dt_dev && r_km1_dev && r_best_dev &&
                   r_last_dev,
               MK_ERR_ARG, "mk_shadow_pass: null pointer");
    MK_REQUIRE(n >= 0 && max_steps >= 1, MK_ERR_ARG, "mk_shadow_pass: bad sizes");
    if (n == 0) return MK_OK;
    shadow_pass_kernel<<<grid_for(n, GEO_THREADS), GEO_THREADS, 0, as_stream(stream)>>>(
        cos_dev, sin_dev, mid_dev, n, bhspin, cos_inc, sin_inc, distance, max_steps, K_dev, best_dev, best_dt_dev,
        r_km1_dev, r_best_dev, r_last_dev);
    MK_LAUNCHED("shadow_pass_kernel");
    return MK_OK;
}
