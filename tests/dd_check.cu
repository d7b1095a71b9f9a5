// Host check of the double-float arithmetic in mk_dd.cuh against long
// double: prints the largest relative error of each operation over random
// operands spanning the magnitudes the geodesic step uses.
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include "mk_dd.cuh"
using mk::dd;
static long double L(dd x) { return (long double)x.hi + (long double)x.lo; }
int main() {
    srand(12345);
    double worst[6] = {0, 0, 0, 0, 0, 0};
    for (int it = 0; it < 200000; it++) {
        double a = ((double)rand() / RAND_MAX - 0.3) * pow(10.0, (rand() % 9) - 4);
        double b = ((double)rand() / RAND_MAX + 0.01) * pow(10.0, (rand() % 9) - 4);
        dd x(a), y(b);
        long double la = L(x), lb = L(y);
        long double r[6] = {la + lb, la - lb, la * lb, la / lb, 1.0L / sqrtl(lb), 0};
        dd g[6] = {x + y, x - y, x * y, x / y, mk::inv_sqrt(y), dd(0.0f, 0.0f)};
        for (int k = 0; k < 5; k++) {
            long double den = fabsl(r[k]) > 0 ? fabsl(r[k]) : 1.0L;
            long double scale = (k < 2) ? fmaxl(fabsl(la), fabsl(lb)) : den;  // add/sub: relative to operands
            double e = (double)(fabsl(L(g[k]) - r[k]) / scale);
            if (e > worst[k]) worst[k] = e;
        }
    }
    printf("%.3e %.3e %.3e %.3e %.3e\n", worst[0], worst[1], worst[2], worst[3], worst[4]);
    return 0;
}
