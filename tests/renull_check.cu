// Host check of renull_k0_dd (mk_kerr.cuh), the near-hole phase's
// double-float null renormalisation: over random Kerr-Schild points
// (r 1.3-9.3 M, spins 0-0.999) and wavevectors whose k^t is a root of
// g(k, k) = 0 perturbed by up to 1e-6, the result against the nearer root
// solved in long double from the same (rounded) inputs.  Prints the largest
// relative error away from the surface g00 = 0, the largest within
// |g00| < 1e-2 (where the quadratic's nearer root loses digits in any
// precision) and the number of such cases.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "mk_kerr.cuh"

using mk::dd;
typedef long double LD;

static LD L(dd x) { return (LD)x.hi + (LD)x.lo; }
static dd D(LD v) {
    const float h = (float)v;
    return dd(h, (float)(v - (LD)h));
}
static LD uni() { return (LD)rand() / RAND_MAX; }

// g00, 2 g0i k^i, gij k^i k^j at x
static void coefficients(LD x, LD y, LD z, LD k1, LD k2, LD k3, LD a, LD &A, LD &B, LD &C) {
    const LD aa = a * a, kk = 0.5L * (x * x + y * y + z * z - aa);
    const LD rr = sqrtl(kk * kk + aa * z * z) + kk, r = sqrtl(rr);
    const LD f = 2 * r * rr / (rr * rr + aa * z * z);
    const LD l1 = (r * x + a * y) / (rr + aa), l2 = (r * y - a * x) / (rr + aa), l3 = z / r;
    const LD lk = l1 * k1 + l2 * k2 + l3 * k3;
    A = f - 1;
    B = 2 * f * lk;
    C = k1 * k1 + k2 * k2 + k3 * k3 + f * lk * lk;
}

int main() {
    srand(7);
    double worst = 0, worst_g00 = 0;
    int near_g00 = 0;
    for (int it = 0; it < 200000; it++) {
        const LD a = rand() % 4 == 0 ? 0.0L : 0.999L * uni();
        const LD r = 1.3L + 8.0L * uni(), th = M_PI * uni(), ph = 2 * M_PI * uni();
        const LD x = (r * cosl(ph) - a * sinl(ph)) * sinl(th), y = (r * sinl(ph) + a * cosl(ph)) * sinl(th);
        const LD z = r * cosl(th);
        const dd X = D(x), Y = D(y), Z = D(z), Ad = D(a);
        const dd K1 = D(2 * uni() - 1), K2 = D(2 * uni() - 1), K3 = D(2 * uni() - 1);
        LD A, B, C;
        coefficients(L(X), L(Y), L(Z), L(K1), L(K2), L(K3), L(Ad), A, B, C);
        const LD disc = B * B - 4 * A * C;
        if (disc < 0 || A == 0) continue;
        const LD sq = sqrtl(disc), r1 = (-B + sq) / (2 * A), r2 = (-B - sq) / (2 * A);
        const LD k0 = ((rand() & 1) ? r1 : r2) * (1 + 1e-6L * (2 * uni() - 1));
        const dd got = mk::renull_k0_dd(X, Y, Z, D(k0), K1, K2, K3, Ad);
        const LD want = fabsl(r1 - k0) < fabsl(r2 - k0) ? r1 : r2;
        const double e = (double)(fabsl(L(got) - want) / fabsl(want));
        if (fabsl(A) < 1e-2L) {
            ++near_g00;
            if (!(e <= worst_g00)) worst_g00 = e;
        } else if (!(e <= worst)) {
            worst = e;
        }
    }
    printf("%.3e %.3e %d\n", worst, worst_g00, near_g00);
    return 0;
}
