// Host check of camera_ray_pair (mk_kerr.cuh), the mixed forms' camera
// ray in double-float, against the reference's construction
// (geodesics.py:121-132, 168-179, 58-85) carried out in long double: the
// three image-plane points moved to the camera, their differences, the
// cross product and the null rescaling.  Over cameras of several spins,
// inclinations, distances, fields of view and sizes, prints the largest
// relative error of the position and of the wavevector (each against its
// own norm) and whether the centre pixel of an odd grid gives NaN in both.
#include <math.h>
#include <stdio.h>

#include "mk_kerr.cuh"

typedef long double LD;

static LD L(mk::f2 v) { return (LD)v.hi + (LD)v.lo; }

static void to_bh(LD x, LD y, LD ci, LD si, LD d, LD o[3]) {
    o[0] = -y * ci + d * si;
    o[1] = x;
    o[2] = y * si + d * ci;
}

// the reference camera ray of pixel (ix, iy) in long double; false where
// the rescaling has no positive root (NaN in the reference)
static bool reference_ray(const mk_camera &c, int ix, int iy, LD X[4], LD K[4]) {
    // the image-plane grid as binary64 rounds it (grid_coord: rounded
    // product, rounded sum)
    const double step = (c.fov_upper - c.fov_lower) / (double)(2 * c.pixels);
    volatile double px = (double)(2 * ix + 1) * step, py = (double)(2 * iy + 1) * step;
    const LD x = (LD)(px + c.fov_lower), y = (LD)(py + c.fov_lower);
    const LD ci = c.cos_inc, si = c.sin_inc, d = c.distance, a = c.bhspin;
    LD org[3], ini[3], per[3];
    to_bh(0, 0, ci, si, d, org);
    to_bh(x, y, ci, si, d, ini);
    to_bh(x + y, y - x, ci, si, d, per);
    LD v1[3], v2[3], v[3];
    for (int i = 0; i < 3; i++) { v1[i] = org[i] - ini[i]; v2[i] = per[i] - ini[i]; }
    v[0] = v1[1] * v2[2] - v1[2] * v2[1];
    v[1] = v1[2] * v2[0] - v1[0] * v2[2];
    v[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const LD aa = a * a, zz = ini[2] * ini[2];
    const LD kk = 0.5L * (ini[0] * ini[0] + ini[1] * ini[1] + zz - aa);
    const LD rr = sqrtl(kk * kk + aa * zz) + kk, r = sqrtl(rr);
    const LD f = 2 * rr * r / (rr * rr + aa * zz);
    const LD l[3] = {(r * ini[0] + a * ini[1]) / (rr + aa), (r * ini[1] - a * ini[0]) / (rr + aa), ini[2] / r};
    const LD lv = l[0] * v[0] + l[1] * v[1] + l[2] * v[2];
    const LD A = f - 1, b = f * lv, C = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + f * lv * lv;
    const bool close = fabsl(b * b - A * C) <= 1e-8L + 1e-5L * fabsl(A * C);
    const LD disc = close ? 0 : b * b - A * C;
    const LD D = -(b + (b < 0 ? 0 : 1) * sqrtl(disc));
    const LD x1 = D / A, x2 = C / D;
    if (isnan(x1) || isnan(x2)) return false;
    const LD d1 = fminl(x1, x2), d2 = fmaxl(x1, x2);
    const LD S = d1 > 0 ? d1 : d2;
    if (!(S > 0)) return false;
    X[0] = 0;
    K[0] = 1;
    for (int i = 0; i < 3; i++) { X[1 + i] = ini[i]; K[1 + i] = v[i] / S; }
    return true;
}

int main() {
    double worst_x = 0, worst_k = 0;
    int rays = 0, nan_ok = 1;
    const double spins[] = {0.0, 0.5, 0.94, 0.999};
    const double incs[] = {0.0, 1.0, 17.0, 60.0, 85.0, 90.0, 180.0};
    const double fovs[] = {0.05, 20.0, 50.0};
    const double dists[] = {100.0, 1000.0, 1e4};
    const int sizes[] = {7, 64};
    for (double a : spins)
        for (double inc : incs)
            for (double fov : fovs)
                for (double dist : dists)
                    for (int n : sizes) {
                        mk_camera c = {};
                        c.kind = MK_CAMERA_GRID;
                        c.pixels = n;
                        c.bhspin = a;
                        c.cos_inc = cos(inc * M_PI / 180.0);
                        c.sin_inc = sin(inc * M_PI / 180.0);
                        c.distance = dist;
                        c.fov_lower = -fov / 2;
                        c.fov_upper = fov / 2;
                        const mk::CameraDD cd = mk::camera_dd(c);
                        for (int p = 0; p < n * n; p++) {
                            mk::f2 X[4], K[4];
                            mk::camera_ray_pair(cd, n, p, X, K);
                            LD Xr[4], Kr[4];
                            const bool ok = reference_ray(c, p / n, p % n, Xr, Kr);
                            const bool got_nan = K[1].hi != K[1].hi || K[3].hi != K[3].hi;
                            if (!ok || got_nan) {
                                if (ok == got_nan) nan_ok = 0;
                                continue;
                            }
                            LD ex = 0, nx = 0, ek = 0, nk = 0;
                            for (int i = 0; i < 4; i++) {
                                ex += (L(X[i]) - Xr[i]) * (L(X[i]) - Xr[i]);
                                nx += Xr[i] * Xr[i];
                                ek += (L(K[i]) - Kr[i]) * (L(K[i]) - Kr[i]);
                                nk += Kr[i] * Kr[i];
                            }
                            worst_x = fmax(worst_x, (double)sqrtl(ex / nx));
                            worst_k = fmax(worst_k, (double)sqrtl(ek / nk));
                            ++rays;
                        }
                        if (n % 2 == 1) {  // the centre pixel has no direction
                            mk::f2 X[4], K[4];
                            mk::camera_ray_pair(cd, n, (int64_t)(n / 2) * n + n / 2, X, K);
                            LD Xr[4], Kr[4];
                            if (reference_ray(c, n / 2, n / 2, Xr, Kr) || K[1].hi == K[1].hi) nan_ok = 0;
                        }
                    }
    printf("%.3e %.3e %d %d\n", worst_x, worst_k, rays, nan_ok);
    return 0;
}
