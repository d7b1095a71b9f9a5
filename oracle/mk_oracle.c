/*
 * mk_oracle.c -- CPU oracle for the per-ray imaging path.  TEST
 * INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm load it as the checker.  The shipped package
 * never calls it.
 *
 * A plain-C FP64 restatement of the reference algorithm (Mahakala,
 * Python+JAX), written to follow the reference's arithmetic rather than the
 * GPU design:
 *   - the metric Jacobian is taken by forward-mode dual numbers, the rule
 *     jax.jacfwd applies (geodesics.py:305), NOT by the closed-form
 *     Christoffel symbols the CUDA kernels use;
 *   - the inverse metric is an LU solve with partial pivoting, as
 *     jnp.linalg.inv (geodesics.py:339-347);
 *   - the step rule, freeze/reject rule and trajectory rows follow
 *     geodesic_integrator (geodesics.py:233-281) step by step;
 *   - the transfer equation is solved by the reference's backward explicit
 *     Euler recursion over stored rows (transfer.py:89-119), not the GPU's
 *     forward affine accumulation.
 * Parity between the GPU path and this file is therefore a comparison of two
 * independent derivations of the same mathematics.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (see build.py).
 * -ffp-contract=off keeps a*b+c as two roundings, as NumPy evaluates it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* constants: mahakala/constants.py:22-31, electrons.py:23-29,         */
/* grmhd/grmhd.py:26-32 (MP exists only in the latter two)             */
/* ------------------------------------------------------------------ */
#define C_EE 4.8032e-10
#define C_CL 2.99792458e10
#define C_ME 9.1094e-28
#define C_MP 1.6726e-24
#define C_HPL 6.6261e-27

/* ------------------------------------------------------------------ */
/* forward-mode dual numbers with 4 tangents (jacfwd over x^mu)         */
/* The tangent rules are jax's JVP rules for mul, div, sqrt, add, sub   */
/* and integer_pow(x, 2).                                               */
/* ------------------------------------------------------------------ */
typedef struct { double v; double d[4]; } dual;

static dual dc(double v) { dual r; r.v = v; r.d[0] = r.d[1] = r.d[2] = r.d[3] = 0.0; return r; }
static dual dadd(dual a, dual b) { dual r; r.v = a.v + b.v; for (int i = 0; i < 4; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
static dual dsub(dual a, dual b) { dual r; r.v = a.v - b.v; for (int i = 0; i < 4; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
static dual dmul(dual a, dual b) { dual r; r.v = a.v * b.v; for (int i = 0; i < 4; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
static dual ddiv(dual a, dual b) {
    dual r; r.v = a.v / b.v;
    double inv2 = 1.0 / (b.v * b.v);
    for (int i = 0; i < 4; i++) r.d[i] = a.d[i] / b.v + (-b.d[i] * a.v) * inv2;
    return r;
}
static dual dsqrt(dual a) { dual r; r.v = sqrt(a.v); double h = 0.5 / r.v; for (int i = 0; i < 4; i++) r.d[i] = a.d[i] * h; return r; }
static dual dsq(dual a) { dual r; r.v = a.v * a.v; double t = 2.0 * a.v; for (int i = 0; i < 4; i++) r.d[i] = a.d[i] * t; return r; }
static dual dscale(double s, dual a) { dual r; r.v = s * a.v; for (int i = 0; i < 4; i++) r.d[i] = s * a.d[i]; return r; }

/* metric(x, a) = eta + f l l^T in Cartesian Kerr-Schild (geodesics.py:88-104) */
static void metric_dual(const double *x, double a, dual g[4][4]) {
    dual X[4];
    for (int m = 0; m < 4; m++) { X[m] = dc(x[m]); X[m].d[m] = 1.0; }
    double aa = a * a;
    dual zz = dsq(X[3]);
    dual kk = dscale(0.5, dsub(dadd(dadd(dmul(X[1], X[1]), dmul(X[2], X[2])), zz), dc(aa)));
    dual rr = dadd(dsqrt(dadd(dmul(kk, kk), dscale(aa, zz))), kk);
    dual r = dsqrt(rr);
    dual f = ddiv(dmul(dscale(2.0, rr), r), dadd(dmul(rr, rr), dscale(aa, zz)));
    dual den = dadd(rr, dc(aa));
    dual l[4];
    l[0] = dc(1.0);
    l[1] = ddiv(dadd(dmul(r, X[1]), dscale(a, X[2])), den);
    l[2] = ddiv(dsub(dmul(r, X[2]), dscale(a, X[1])), den);
    l[3] = ddiv(X[3], r);
    for (int m = 0; m < 4; m++)
        for (int n = 0; n < 4; n++) {
            dual t = dmul(f, dmul(l[m], l[n]));
            double eta = (m == n) ? (m == 0 ? -1.0 : 1.0) : 0.0;
            g[m][n] = dadd(dc(eta), t);
        }
}

static void metric_plain(const double *x, double a, double g[4][4]) {
    double aa = a * a;
    double zz = x[3] * x[3];
    double kk = 0.5 * (x[1] * x[1] + x[2] * x[2] + zz - aa);
    double rr = sqrt(kk * kk + aa * zz) + kk;
    double r = sqrt(rr);
    double f = (2.0 * rr * r) / (rr * rr + aa * zz);
    double l[4] = {1.0, (r * x[1] + a * x[2]) / (rr + aa), (r * x[2] - a * x[1]) / (rr + aa), x[3] / r};
    for (int m = 0; m < 4; m++)
        for (int n = 0; n < 4; n++)
            g[m][n] = ((m == n) ? (m == 0 ? -1.0 : 1.0) : 0.0) + f * (l[m] * l[n]);
}

/* inverse by LU with partial pivoting, then solves against the identity
   (jnp.linalg.inv -> solve(a, I)); returns 0 if singular */
static int inv4(const double A[4][4], double out[4][4]) {
    double lu[4][4];
    int piv[4];
    memcpy(lu, A, sizeof(lu));
    for (int i = 0; i < 4; i++) piv[i] = i;
    for (int k = 0; k < 4; k++) {
        int p = k;
        double best = fabs(lu[k][k]);
        for (int i = k + 1; i < 4; i++)
            if (fabs(lu[i][k]) > best) { best = fabs(lu[i][k]); p = i; }
        if (p != k) {
            for (int j = 0; j < 4; j++) { double t = lu[k][j]; lu[k][j] = lu[p][j]; lu[p][j] = t; }
            int t = piv[k]; piv[k] = piv[p]; piv[p] = t;
        }
        if (lu[k][k] == 0.0) {
            for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) out[i][j] = NAN;
            return 0;
        }
        for (int i = k + 1; i < 4; i++) {
            lu[i][k] /= lu[k][k];
            for (int j = k + 1; j < 4; j++) lu[i][j] -= lu[i][k] * lu[k][j];
        }
    }
    for (int c = 0; c < 4; c++) {
        double y[4];
        for (int i = 0; i < 4; i++) {
            double s = (piv[i] == c) ? 1.0 : 0.0;
            for (int j = 0; j < i; j++) s -= lu[i][j] * y[j];
            y[i] = s;
        }
        for (int i = 3; i >= 0; i--) {
            double s = y[i];
            for (int j = i + 1; j < 4; j++) s -= lu[i][j] * out[j][c];
            out[i][c] = s / lu[i][i];
        }
    }
    return 1;
}

/* rhs (geodesics.py:294-309): a = ig @ (-(jg@v)@v + 0.5 v@(v@jg)) */
static void rhs(const double *s, double a, double *out) {
    dual g[4][4];
    double gp[4][4], ig[4][4];
    metric_dual(s, a, g);
    for (int m = 0; m < 4; m++) for (int n = 0; n < 4; n++) gp[m][n] = g[m][n].v;
    inv4(gp, ig);
    const double *v = s + 4;
    double t1[4], t2[4], w[4];
    for (int m = 0; m < 4; m++) {
        double acc = 0.0;
        for (int b = 0; b < 4; b++) {
            double jv = 0.0;
            for (int c = 0; c < 4; c++) jv += g[m][b].d[c] * v[c];
            acc += jv * v[b];
        }
        t1[m] = acc;
    }
    for (int c = 0; c < 4; c++) {
        double acc = 0.0;
        for (int m = 0; m < 4; m++) {
            double vj = 0.0;
            for (int b = 0; b < 4; b++) vj += v[b] * g[m][b].d[c];
            acc += v[m] * vj;
        }
        t2[c] = acc;
    }
    for (int m = 0; m < 4; m++) w[m] = -t1[m] + 0.5 * t2[m];
    for (int m = 0; m < 4; m++) {
        double acc = 0.0;
        for (int n = 0; n < 4; n++) acc += ig[m][n] * w[n];
        out[m] = v[m];
        out[4 + m] = acc;
    }
}

/* RK4_gen (geodesics.py:317-336) for one ray */
static void rk4(const double *s, double dt, double a, double *out) {
    double k1[8], k2[8], k3[8], k4[8], tmp[8], d[8];
    rhs(s, a, d);
    for (int i = 0; i < 8; i++) k1[i] = dt * d[i];
    for (int i = 0; i < 8; i++) tmp[i] = s[i] + 0.5 * k1[i];
    rhs(tmp, a, d);
    for (int i = 0; i < 8; i++) k2[i] = dt * d[i];
    for (int i = 0; i < 8; i++) tmp[i] = s[i] + 0.5 * k2[i];
    rhs(tmp, a, d);
    for (int i = 0; i < 8; i++) k3[i] = dt * d[i];
    for (int i = 0; i < 8; i++) tmp[i] = s[i] + k3[i];
    rhs(tmp, a, d);
    for (int i = 0; i < 8; i++) k4[i] = dt * d[i];
    const double sixth = 1.0 / 6.0;
    for (int i = 0; i < 8; i++) out[i] = s[i] + sixth * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
}

/* radius_cal (geodesics.py:284-291) and radius_EH (:350-351) */
double orc_radius_cal(const double *x, double a) {
    double R = sqrt(x[1] * x[1] + x[2] * x[2] + x[3] * x[3]);
    double R2 = R * R;
    double aa = a * a;
    double q = R2 - aa;
    return sqrt((q + sqrt(q * q + 4.0 * aa * (x[3] * x[3]))) / 2.0);
}
static double radius_eh(double a) { return 1.0 + sqrt(1.0 - a * a); }

/* status codes shared with the CUDA path */
enum { ST_ACTIVE = 0, ST_CAPTURED = 1, ST_ESCAPED = 2, ST_MAXSTEPS = 3, ST_NAN = 4 };

/* dt rule of geodesic_step (geodesics.py:249-252); *why gets the stop reason */
static double step_dt(const double *s, double a, double rEH, double div, double tol, int *why) {
    double dt = -(orc_radius_cal(s, a) - rEH) / div;
    *why = ST_ACTIVE;
    if (isnan(dt)) { *why = ST_NAN; return 0.0; }
    if (fabs(dt) * div < tol) { *why = ST_CAPTURED; return 0.0; }
    if (fabs(dt) * div > 1500.0) { *why = ST_ESCAPED; return 0.0; }
    return dt;
}

/* ------------------------------------------------------------------ */
/* camera (geodesics.py:58-85, 107-134, 137-230)                        */
/* ------------------------------------------------------------------ */
/* _Nullify with p=1 on one ray (in place on v[4]) */
static void nullify(const double *x, double a, double *v) {
    double g[4][4];
    metric_plain(x, a, g);
    double A = (v[0] * g[0][0]) * v[0];
    double b = ((v[1] * g[1][0] + v[2] * g[2][0]) + v[3] * g[3][0]) * v[0];
    double w[3];
    for (int j = 0; j < 3; j++) w[j] = (v[1] * g[1][1 + j] + v[2] * g[2][1 + j]) + v[3] * g[3][1 + j];
    double C = (w[0] * v[1] + w[1] * v[2]) + w[2] * v[3];
    double bb = b * b, AC = A * C;
    int close = fabs(bb - AC) <= (1e-8 + 1e-5 * fabs(AC));
    double dd = close ? 0.0 : bb - AC;
    double bs = (b < 0.0) ? 0.0 : 1.0; /* heaviside(b, 1) */
    double D = -(b + bs * sqrt(dd));
    double x1 = D / A, x2 = C / D;
    double d1, d2;
    if (isnan(x1) || isnan(x2)) { d1 = d2 = NAN; }
    else { d1 = x1 < x2 ? x1 : x2; d2 = x1 < x2 ? x2 : x1; }
    double S = (d1 > 0.0) ? d1 : ((d2 > 0.0) ? d2 : NAN);
    v[1] /= S; v[2] /= S; v[3] /= S;
}

/* _Image_to_BH (geodesics.py:204-209); ci, si are cos/sin of the
   inclination in radians as NumPy evaluates them */
static void image_to_bh(double x, double y, double z, double ci, double si, double d, double *o) {
    o[0] = -y * ci + z * si + d * si;
    o[1] = x;
    o[2] = y * si + z * ci + d * ci;
}

/* one camera pixel at image-plane (x, y): position + null wavevector */
static void camera_pixel(double x, double y, double ci, double si, double d, double a, double *s) {
    double org[3], ini[3], per[3];
    image_to_bh(0.0, 0.0, 0.0, ci, si, d, org);
    image_to_bh(x, y, 0.0, ci, si, d, ini);
    image_to_bh(x + y, y - x, 0.0, ci, si, d, per);
    double v1[3], v2[3];
    for (int i = 0; i < 3; i++) { v1[i] = -ini[i] + org[i]; v2[i] = per[i] - ini[i]; }
    s[0] = 0.0; s[1] = ini[0]; s[2] = ini[1]; s[3] = ini[2];
    s[4] = 1.0;
    s[5] = v1[1] * v2[2] - v1[2] * v2[1];
    s[6] = v1[2] * v2[0] - v1[0] * v2[2];
    s[7] = v1[0] * v2[1] - v1[1] * v2[0];
    nullify(s, a, s + 4);
}

/* grid camera: grid[n] = linspace(lo, hi, 2n+1)[1::2] computed by NumPy;
   pixel p = ix*n + iy (meshgrid indexing='ij').  s0: (n*n, 8) */
void orc_camera_grid(const double *grid, int n, double ci, double si, double d, double a, double *s0) {
    for (int ix = 0; ix < n; ix++)
        for (int iy = 0; iy < n; iy++)
            camera_pixel(grid[ix], grid[iy], ci, si, d, a, s0 + 8 * ((int64_t)ix * n + iy));
}

/* polar camera of get_camera_pixel (geodesics.py:107-134); cos/sin of the
   angles are computed by NumPy and passed in */
void orc_camera_polar(const double *cosang, const double *sinang, const double *radius, int n,
                      double ci, double si, double d, double a, double *s0) {
    for (int p = 0; p < n; p++)
        camera_pixel(cosang[p] * radius[p], sinang[p] * radius[p], ci, si, d, a, s0 + 8 * p);
}

/* ------------------------------------------------------------------ */
/* integrator: reference step rule (geodesics.py:246-269)              */
/* ------------------------------------------------------------------ */
/* Integrates one ray for up to N steps.  rows (N x 8) and dts (N) are
   optional (stride `rs` between rows, in doubles).  Returns K, the index of
   the first frozen step (N if the ray never froze); *why = stop reason. */
static int integrate_ray(const double *s0, int N, double div, double tol, double a,
                         double *rows, int64_t rs, double *dts, int64_t ds,
                         double *final_state, int *why_out) {
    double s[8], nw[8];
    memcpy(s, s0, sizeof(s));
    double rEH = radius_eh(a);
    int K = N, why = ST_MAXSTEPS;
    for (int j = 0; j < N; j++) {
        int w0, w1;
        double dt = step_dt(s, a, rEH, div, tol, &w0);
        rk4(s, dt, a, nw);
        double dtn = step_dt(nw, a, rEH, div, tol, &w1);
        if (dtn == 0.0) {
            /* rejected: frozen from here on (deterministic repeat) */
            K = j;
            why = (w0 != ST_ACTIVE) ? w0 : w1;
            if (rows) for (int r = j; r < N; r++) memcpy(rows + r * rs, s, sizeof(s));
            if (dts) for (int r = j; r < N; r++) dts[r * ds] = 0.0;
            break;
        }
        if (rows) memcpy(rows + j * rs, s, sizeof(s));
        if (dts) dts[j * ds] = dt;
        memcpy(s, nw, sizeof(s));
    }
    if (final_state) memcpy(final_state, s, sizeof(s));
    *why_out = why;
    return K;
}

/* geodesic_integrator over npx rays.  S (N x npx x 8) and dt (N x npx) are
   optional full trajectories (rows beyond a ray's freeze repeat its frozen
   state).  K[p] = first frozen step, why[p] = stop reason, state[p] = the
   ray's state after K steps (its frozen state). */
void orc_integrate(const double *s0, int npx, int N, double div, double tol, double a,
                   double *S, double *dt, int *K, int *why, double *state) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int p = 0; p < npx; p++) {
        K[p] = integrate_ray(s0 + 8 * (int64_t)p, N, div, tol, a,
                             S ? S + 8 * (int64_t)p : NULL, 8 * (int64_t)npx,
                             dt ? dt + p : NULL, npx, state + 8 * (int64_t)p, &why[p]);
    }
}

/* find_shadow_bisection_angles (geodesics.py:405-435) with
   select_photons_integrator (:354-378) and get_camera_pixel (:107-134).
   cosang/sinang: NumPy cos/sin of the angles.  radii: output (inner).
   Per iteration every ray is integrated with the reference rule (div 40,
   tol 1e-2); the trajectory is trimmed as geodesic_integrator trims it
   (first all-zero dt row F over ALL rays, keep F+2 rows, or N rows when no
   such row exists or F < 1); the answer per ray is radius_cal at row
   argmax(dt) - 1, with -1 wrapping to the last kept row. */
void orc_shadow_bisection(const double *cosang, const double *sinang, int n, double ci, double si,
                          double a, double distance, int max_steps, double error_allowed,
                          int max_it, double *radii) {
    int N = max_steps;
    double *inner = radii;
    double *outer = (double *)malloc(sizeof(double) * n);
    double *mid = (double *)malloc(sizeof(double) * n);
    double *rrow = (double *)malloc(sizeof(double) * (size_t)n * N);
    double *dtrow = (double *)malloc(sizeof(double) * (size_t)n * N);
    int *Ks = (int *)malloc(sizeof(int) * n);
    for (int p = 0; p < n; p++) { inner[p] = 0.5; outer[p] = 10.0; }
    int counter = 0;
    for (;;) {
        double maxerr = -INFINITY;
        for (int p = 0; p < n; p++) { double e = outer[p] - inner[p]; if (e > maxerr) maxerr = e; }
        if (!(maxerr > error_allowed && counter < max_it)) break;
        for (int p = 0; p < n; p++) mid[p] = (outer[p] - inner[p]) / 2.0 + inner[p];
#pragma omp parallel
        {
            double *rows = (double *)malloc(sizeof(double) * 8 * (size_t)N);
#pragma omp for schedule(dynamic, 1)
            for (int p = 0; p < n; p++) {
                double s0[8], fin[8];
                int why;
                camera_pixel(cosang[p] * mid[p], sinang[p] * mid[p], ci, si, distance, a, s0);
                Ks[p] = integrate_ray(s0, N, 40.0, 1e-2, a, rows, 8, dtrow + (size_t)p * N, 1, fin, &why);
                for (int j = 0; j < N; j++) rrow[(size_t)p * N + j] = orc_radius_cal(rows + 8 * (size_t)j, a);
            }
            free(rows);
        }
        int all_frozen = 1, F = 0;
        for (int p = 0; p < n; p++) {
            if (Ks[p] >= N) all_frozen = 0;
            else if (Ks[p] > F) F = Ks[p];
        }
        int Nt = N;
        if (all_frozen && F >= 1) Nt = (F + 2 < N) ? F + 2 : N;
        for (int p = 0; p < n; p++) {
            const double *d = dtrow + (size_t)p * N;
            int am = 0;
            for (int j = 1; j < Nt; j++) if (d[j] > d[am]) am = j;
            int row = am - 1;
            if (row < 0) row = Nt - 1;
            double fin = rrow[(size_t)p * N + row];
            if (fin < 100.0) inner[p] = (outer[p] - inner[p]) / 2.0 + inner[p];
            else if (fin >= 100.0) outer[p] = (outer[p] - inner[p]) / 2.0 + inner[p];
        }
        counter++;
    }
    free(outer); free(mid); free(rrow); free(dtrow); free(Ks);
}

/* ------------------------------------------------------------------ */
/* fixed-fraction vacuum step policy (not in the reference): h = 0.05 r */
/* clamped to [hmin, hmax], captured at r < cap*r_h, escaped at r >     */
/* r_esc once r increases, at most N steps.                              */
/* ------------------------------------------------------------------ */
void orc_trace_fixed(const double *s0, int npx, int N, double a, double hfrac, double hmin,
                     double hmax, double cap, double r_esc, double *state, int *nsteps, int *why) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int p = 0; p < npx; p++) {
        double s[8], nw[8];
        memcpy(s, s0 + 8 * (int64_t)p, sizeof(s));
        double rcap = cap * radius_eh(a);
        int st = ST_MAXSTEPS, j;
        double r = orc_radius_cal(s, a);
        for (j = 0; j < N; j++) {
            double h = hfrac * r;
            if (h < hmin) h = hmin;
            if (h > hmax) h = hmax;
            rk4(s, -h, a, nw);
            double rn = orc_radius_cal(nw, a);
            memcpy(s, nw, sizeof(s));
            if (isnan(rn) || isnan(s[4])) { st = ST_NAN; j++; break; }
            if (rn < rcap) { st = ST_CAPTURED; j++; break; }
            if (rn > r_esc && rn > r) { st = ST_ESCAPED; j++; break; }
            r = rn;
        }
        memcpy(state + 8 * (int64_t)p, s, sizeof(s));
        nsteps[p] = j;
        why[p] = st;
    }
}

/* ------------------------------------------------------------------ */
/* fluid sampling (grmhd/athenak.py:639-812)                            */
/* ------------------------------------------------------------------ */
typedef struct {
    const double *mb;       /* (nmb, 8, n+2, n+2, n+2): [mb][prim][k][j][i], as the reference holds it */
    int nmb, n;
    const double *ext;      /* (nmb, 6): x1f[0], x1f[-1], x2f[0], x2f[-1], x3f[0], x3f[-1] */
    const double *left;     /* (nmb, 3): x1v[0], x2v[0], x3v[0] */
    const double *dx;       /* (nmb, 3): x?v[1] - x?v[0] */
    /* optional uniform single-level fast lookup: per-axis block faces and
       a (nb3, nb2, nb1) table of block ids; NULL -> literal O(nmb) scan */
    const double *faces[3];
    int nbx[3];
    const int32_t *table;
    double bhspin;
} orc_snapshot;

/* literal lookup (athenak.py:663-670): last block with left < x <= right */
static int lookup_scan(const orc_snapshot *m, const double *x) {
    int hit = -1;
    for (int b = 0; b < m->nmb; b++) {
        const double *e = m->ext + 6 * (int64_t)b;
        if (e[0] < x[1] && x[1] <= e[1] && e[2] < x[2] && x[2] <= e[3] && e[4] < x[3] && x[3] <= e[5])
            hit = b;
    }
    return hit;
}

static int axis_cell(const double *f, int nb, double x) {
    /* index i with f[i] < x <= f[i+1], -1 outside */
    if (!(x > f[0] && x <= f[nb])) return -1;
    int lo = 0, hi = nb; /* invariant f[lo] < x <= f[hi] */
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (x <= f[mid]) hi = mid; else lo = mid;
    }
    return lo;
}

int orc_lookup(const orc_snapshot *m, const double *x) {
    if (!m->table) return lookup_scan(m, x);
    int i = axis_cell(m->faces[0], m->nbx[0], x[1]);
    int j = axis_cell(m->faces[1], m->nbx[1], x[2]);
    int k = axis_cell(m->faces[2], m->nbx[2], x[3]);
    if (i < 0 || j < 0 || k < 0) return -1;
    return m->table[((int64_t)k * m->nbx[1] + j) * m->nbx[0] + i];
}

/* float floor_divide / remainder with Python semantics (as jnp on floats) */
static double py_floordiv(double x, double y) {
    double mod = fmod(x, y);
    double div = (x - mod) / y;
    if (mod != 0.0 && ((y < 0.0) != (mod < 0.0))) div -= 1.0;
    double fl;
    if (div != 0.0) {
        fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
    } else {
        fl = copysign(0.0, x / y);
    }
    return fl;
}
static double py_mod1(double x) {
    double m = fmod(x, 1.0);
    if (m != 0.0 && (m < 0.0)) m += 1.0;
    return m;
}

/* primitives at x (get_prims_from_geodesics body, athenak.py:712-757);
   prims[8] = dens, velx, vely, velz, eint, bcc1..3; returns block or -1 */
static int sample_prims(const orc_snapshot *m, const double *x, double *prims) {
    int b = orc_lookup(m, x);
    if (b < 0) { for (int p = 0; p < 8; p++) prims[p] = 0.0; return -1; }
    int idx[3];
    double del[3];
    for (int c = 0; c < 3; c++) {
        double d = m->dx[3 * (int64_t)b + c];
        double t = x[1 + c] - m->left[3 * (int64_t)b + c] + d;
        del[c] = py_mod1(t / d);
        idx[c] = (int)py_floordiv(t, d);
    }
    int n2 = m->n + 2;
    const double *base = m->mb + (int64_t)b * 8 * n2 * n2 * n2;
    for (int p = 0; p < 8; p++) {
        const double *q = base + (int64_t)p * n2 * n2 * n2;
#define AT(kk, jj, ii) (q[((int64_t)(idx[2] + (kk)) * n2 + (idx[1] + (jj))) * n2 + (idx[0] + (ii))])
        double aaa = AT(0, 0, 0), aab = AT(0, 0, 1), aba = AT(0, 1, 0), abb = AT(0, 1, 1);
        double baa = AT(1, 0, 0), bab = AT(1, 0, 1), bba = AT(1, 1, 0), bbb = AT(1, 1, 1);
#undef AT
        double daa = aaa + (aab - aaa) * del[0];
        double dab = aba + (abb - aba) * del[0];
        double dba = baa + (bab - baa) * del[0];
        double dbb = bba + (bbb - bba) * del[0];
        double da = daa + (dab - daa) * del[1];
        double db = dba + (dbb - dba) * del[1];
        prims[p] = da + (db - da) * del[2];
    }
    return b;
}

/* fluid scalars at one trajectory point (athenak.py:759-794).
   out[5] = dens, u, pitch_angle, kdotu, b */
static void fluid_scalars_point(const orc_snapshot *m, const double *S0, double cos_fallback, double *out) {
    double pr[8];
    sample_prims(m, S0, pr);
    double g[4][4], gi[4][4];
    metric_plain(S0, m->bhspin, g);
    inv4(g, gi);
    double alpha = sqrt(1.0 / (-gi[0][0]));
    const double *U = pr + 1;
    double w[3];
    for (int j = 0; j < 3; j++) w[j] = (U[0] * g[1][1 + j] + U[1] * g[2][1 + j]) + U[2] * g[3][1 + j];
    double gamma = sqrt(1.0 + ((w[0] * U[0] + w[1] * U[1]) + w[2] * U[2]));
    double ucon[4], ucov[4], bcon[4], bcov[4];
    ucon[0] = gamma / alpha;
    for (int i = 0; i < 3; i++) ucon[1 + i] = U[i] - gamma * alpha * gi[0][1 + i];
    for (int i = 0; i < 4; i++) ucov[i] = ((g[i][0] * ucon[0] + g[i][1] * ucon[1]) + g[i][2] * ucon[2]) + g[i][3] * ucon[3];
    const double *B = pr + 5;
    bcon[0] = (B[0] * ucov[1] + B[1] * ucov[2]) + B[2] * ucov[3];
    for (int i = 0; i < 3; i++) bcon[1 + i] = (B[i] + ucon[1 + i] * bcon[0]) / ucon[0];
    for (int i = 0; i < 4; i++) bcov[i] = ((g[i][0] * bcon[0] + g[i][1] * bcon[1]) + g[i][2] * bcon[2]) + g[i][3] * bcon[3];
    const double *k = S0 + 4;
    double kdotu = ((k[0] * ucov[0] + k[1] * ucov[1]) + k[2] * ucov[2]) + k[3] * ucov[3];
    double kdotb = ((k[0] * bcov[0] + k[1] * bcov[1]) + k[2] * bcov[2]) + k[3] * bcov[3];
    double bdotb = ((bcon[0] * bcov[0] + bcon[1] * bcov[1]) + bcon[2] * bcov[2]) + bcon[3] * bcov[3];
    double pitch = kdotb / (fabs(kdotu) * sqrt(bdotb));
    if (isnan(pitch)) pitch = cos_fallback;
    if (fabs(pitch) > 1.0) pitch = pitch / fabs(pitch);
    out[0] = pr[0];
    out[1] = pr[4];
    out[2] = acos(pitch);
    out[3] = kdotu;
    out[4] = sqrt(bdotb);
}

static void build_snapshot(orc_snapshot *m, const double *mb, int nmb, int n, const double *ext,
                           const double *left, const double *dx, const double *f1, const double *f2,
                           const double *f3, const int32_t *nb, const int32_t *table, double a) {
    m->mb = mb; m->nmb = nmb; m->n = n; m->ext = ext; m->left = left; m->dx = dx;
    m->faces[0] = f1; m->faces[1] = f2; m->faces[2] = f3;
    m->nbx[0] = nb ? nb[0] : 0; m->nbx[1] = nb ? nb[1] : 0; m->nbx[2] = nb ? nb[2] : 0;
    m->table = table; m->bhspin = a;
}

/* get_fluid_scalars_from_geodesics over npts points of S (npts x 8) */
void orc_fluid_scalars(const double *mb, int nmb, int n, const double *ext, const double *left,
                       const double *dx, const double *f1, const double *f2, const double *f3,
                       const int32_t *nb, const int32_t *table, double a,
                       const double *S, int64_t npts, double cos_fallback, double *out) {
    orc_snapshot m;
    build_snapshot(&m, mb, nmb, n, ext, left, dx, f1, f2, f3, nb, table, a);
#pragma omp parallel for schedule(static, 256)
    for (int64_t p = 0; p < npts; p++) fluid_scalars_point(&m, S + 8 * p, cos_fallback, out + 5 * p);
}

/* get_prims_from_geodesics over npts points (out: npts x 8) and the block id */
void orc_fluid_prims(const double *mb, int nmb, int n, const double *ext, const double *left,
                     const double *dx, const double *f1, const double *f2, const double *f3,
                     const int32_t *nb, const int32_t *table, double a,
                     const double *S, int64_t npts, double *out, int32_t *block) {
    orc_snapshot m;
    build_snapshot(&m, mb, nmb, n, ext, left, dx, f1, f2, f3, nb, table, a);
#pragma omp parallel for schedule(static, 256)
    for (int64_t p = 0; p < npts; p++) block[p] = sample_prims(&m, S + 8 * p, out + 8 * p);
}

/* ------------------------------------------------------------------ */
/* electrons + synchrotron + transfer                                   */
/* ------------------------------------------------------------------ */
/* rlow_rhigh_model (electrons.py:32-50); gem1 = electron_gamma - 1.,
   gim1 = ion_gamma - 1. as Python evaluates them */
static double rlow_rhigh(double dens, double u, double beta, double r_low, double r_high,
                         double gem1, double gim1) {
    double b2 = beta * beta;
    double T_ratio = (r_high * b2 + r_low) / (1.0 + b2);
    double t = (C_CL * C_CL) * (((C_MP * u) * gem1) * gim1);
    t /= dens * (gim1 + gem1 * T_ratio);
    return t / ((C_ME * C_CL) * C_CL);
}

void orc_rlow_rhigh(const double *dens, const double *u, const double *beta, int64_t n,
                    double r_low, double r_high, double gem1, double gim1, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = rlow_rhigh(dens[i], u[i], beta[i], r_low, r_high, gem1, gim1);
}

/* synchrotron_coefficients (transfer.py:30-86).  c2_11_12 = 2.0**(11./12)
   as Python evaluates it. */
static void synchrotron(double Ne, double Th, double B, double pitch, double nu, int invariant,
                        double rescale_nu, double c2_11_12, double *em_out, double *ab_out) {
    const double two_pi_me_cl = (2.0 * M_PI * C_ME) * C_CL;
    double nuc = C_EE * B / two_pi_me_cl;
    double nus = ((2.0 / 9.0) * nuc * (Th * Th)) * sin(pitch);
    double X = nu / nus;
    double var = exp(-pow(X, 1.0 / 3));
    double term = sqrt(X) + c2_11_12 * pow(X, 1.0 / 6);
    double em = Ne * nus * (term * term) / (2.0 * (Th * Th));
    em = em * var * sqrt(2.0) * M_PI * (C_EE * C_EE) / (3.0 * C_CL);
    if (X > 1.e12) em = 0.0;
    if (Th < 0.3) em = 0.0;
    double bx = C_HPL * nu / (((C_ME * C_CL) * C_CL) * Th);
    double ser = bx / 24. * (24. + bx * (12. + bx * (4. + bx)));
    double Bden = (bx < 2.e-3) ? ser : (exp(bx) - 1.0);
    double Bnu = ((2. * C_HPL) * pow(nu, 3.) / Bden) / (C_CL * C_CL);
    double ab = em / Bnu;
    if (invariant) {
        double rn = nu * rescale_nu;
        em = em / (rn * rn);
        ab = ab * rn;
    }
    if (isnan(em)) em = 0.0;
    if (isnan(ab)) ab = 0.0;
    *em_out = em;
    *ab_out = ab;
}

void orc_synchrotron(const double *Ne, const double *Th, const double *B, const double *pitch,
                     const double *nu, int64_t n, int invariant, double rescale_nu, double c2_11_12,
                     double *em, double *ab) {
    for (int64_t i = 0; i < n; i++)
        synchrotron(Ne[i], Th[i], B[i], pitch[i], nu[i], invariant, rescale_nu, c2_11_12, em + i, ab + i);
}

/* solve_specific_intensity (transfer.py:89-119) on (nsteps, npx) arrays;
   dIs (nsteps-1, npx) optional, row r = step i = nsteps-1-r */
void orc_solve_intensity(const double *em, const double *ab, const double *dt, int nsteps, int npx,
                         double L_unit, double *I, double *dIs) {
    for (int p = 0; p < npx; p++) {
        double Iv = 0.0;
        for (int i = nsteps - 1, r = 0; i >= 1; i--, r++) {
            double dI = (-dt[(int64_t)(i - 1) * npx + p]) * L_unit *
                        (em[(int64_t)i * npx + p] - (ab[(int64_t)i * npx + p] * Iv));
            Iv += dI;
            if (dIs) dIs[(int64_t)r * npx + p] = dI;
        }
        I[p] = Iv;
    }
}

/* solve_attenuated_emissivity (transfer.py:122-144); out (nsteps-1, npx) */
void orc_attenuated_emissivity(const double *em, const double *ab, const double *dt, int nsteps,
                               int npx, double L_unit, double *out) {
    for (int p = 0; p < npx; p++) {
        double tau = 0.0;
        for (int i = 1; i < nsteps; i++) {
            double dtl = dt[(int64_t)(i - 1) * npx + p];
            double src = -em[(int64_t)i * npx + p] * dtl * L_unit;
            double dtau = ab[(int64_t)i * npx + p] * dtl * L_unit;
            out[(int64_t)(i - 1) * npx + p] = exp(-tau) * src;
            tau = tau - dtau;
        }
    }
}

/* ------------------------------------------------------------------ */
/* make_image (images.py:30-144), one ray at a time                     */
/* ------------------------------------------------------------------ */
typedef struct {
    double bhspin, div, tol;
    int N;
    double fluid_gamma, r_low, r_high, gem1, gim1;
    double Ne_unit, B_unit, L_unit;
    double cos_fallback, c2_11_12, sigma_cut;
    int nnu;
    double nu[4];
} orc_render_params;

/* Renders npx rays from s0 (npx x 8).  image (nnu x npx).  nsteps[p] = the
   ray's accepted steps used by the transfer solve. */
void orc_render(const orc_render_params *P, const double *mb, int nmb, int n, const double *ext,
                const double *left, const double *dx, const double *f1, const double *f2,
                const double *f3, const int32_t *nb, const int32_t *table,
                const double *s0, int npx, double *image, int *nsteps) {
    orc_snapshot m;
    build_snapshot(&m, mb, nmb, n, ext, left, dx, f1, f2, f3, nb, table, P->bhspin);
    int N = P->N;
#pragma omp parallel
    {
        double *rows = (double *)malloc(sizeof(double) * 8 * (size_t)N);
        double *dts = (double *)malloc(sizeof(double) * (size_t)N);
#pragma omp for schedule(dynamic, 4)
        for (int p = 0; p < npx; p++) {
            int why;
            double fin[8];
            int K = integrate_ray(s0 + 8 * (int64_t)p, N, P->div, P->tol, P->bhspin, rows, 8, dts, 1, fin, &why);
            /* rows exist for steps 0..N-1 (row i = state before step i); the
               solve pairs row i with dt[i-1], so the last usable row is
               min(K, N-1) (later rows have dt = 0 and add nothing) */
            int M = (K < N - 1) ? K : N - 1;
            if (K < N) memcpy(rows + 8 * (int64_t)K, fin, sizeof(fin));
            nsteps[p] = M;
            for (int c = 0; c < P->nnu; c++) {
                double nu_obs = P->nu[c];
                double Iv = 0.0;
                for (int i = M; i >= 1; i--) {
                    double sc[5];
                    fluid_scalars_point(&m, rows + 8 * (int64_t)i, P->cos_fallback, sc);
                    double bsq = sc[4] * sc[4];
                    double beta = sc[1] * (P->fluid_gamma - 1.) / bsq / 0.5;
                    double sigma = bsq / sc[0];
                    double Th = rlow_rhigh(sc[0], sc[1], beta, P->r_low, P->r_high, P->gem1, P->gim1);
                    double Ne = P->Ne_unit * sc[0];
                    double Bg = P->B_unit * sc[4];
                    double nu = -sc[3] * nu_obs;
                    double em, ab;
                    synchrotron(Ne, Th, Bg, sc[2], nu, 1, 1. / nu_obs, P->c2_11_12, &em, &ab);
                    if (sigma > P->sigma_cut) { em = 0.0; ab = 0.0; }
                    Iv += (-dts[i - 1]) * P->L_unit * (em - (ab * Iv));
                }
                image[(int64_t)c * npx + p] = Iv;
            }
        }
        free(rows);
        free(dts);
    }
}
