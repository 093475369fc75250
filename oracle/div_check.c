/*
 * Test infrastructure: checks that the FMA-corrected quotient the CUDA
 * kernels use in place of an IEEE division by a cell size,
 *
 *     y = RN(1/b)          (once per b, IEEE division on the host)
 *     q = RN(a*y)
 *     r = fma(-q, b, a)    (exact remainder)
 *     q' = fma(r, y, q)
 *
 * (Markstein's correction step: P. Markstein, "Computation of elementary
 * functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
 * 1990; correct rounding when y is the correctly rounded reciprocal and q is
 * within one ulp, outside underflow/overflow), equals RN(a/b) bit for bit on
 * the operands the kernels divide: positions and offsets by a cell size, and
 * products of shape values by a cell size.
 *
 * usage: div_check <n_random> <seed>; prints "mismatches <k> of <n>".
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s_state;
static uint64_t next_u64(void) { /* splitmix64 */
    uint64_t z = (s_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double uniform(void) { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static double corrected_div(double a, double b, double y) {
    volatile double q = a * y;
    double r = fma(-q, b, a);
    return fma(r, y, q);
}

static long check(double a, double b, double y) {
    double want = a / b;
    double got = corrected_div(a, b, y);
    uint64_t w, g;
    memcpy(&w, &want, 8);
    memcpy(&g, &got, 8);
    if (w != g && !(want == 0.0 && got == 0.0)) {
        fprintf(stderr, "mismatch a=%.17g b=%.17g want=%.17g got=%.17g\n", a, b, want, got);
        return 1;
    }
    return 0;
}

int main(int argc, char** argv) {
    long n = argc > 1 ? atol(argv[1]) : 1000000;
    s_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    const double hs[] = {1.0e-3, 0.5e-3, 0.25e-3, 0.8e-3, 1.0 / 1.25 * 1.0e-3, 0.0688 / 86.0, 0.05 / 52.0,
                         0.084 / 84.0, 0.046 / 46.0, 1.0 / 3.0 * 1.0e-3, 0.7e-3, 0.13e-3};
    const int nh = (int)(sizeof(hs) / sizeof(hs[0]));
    long bad = 0, total = 0;
    for (int ih = 0; ih < nh + 4; ++ih) {
        double b = ih < nh ? hs[ih] : 1.0e-4 + uniform() * 2.0e-3;
        double y = 1.0 / b;
        for (long i = 0; i < n; ++i) {
            /* positions in a grid of up to ~1000 cells, both signs near the origin */
            double a = (uniform() * 1.1 - 0.05) * 1000.0 * b;
            bad += check(a, b, y);
            /* near-integer quotients: a = k*b nudged by a few ulps */
            double k = floor(uniform() * 1000.0);
            double base = k * b;
            int ul = (int)(next_u64() % 9) - 4;
            double aa = base;
            for (int u = 0; u < abs(ul); ++u) aa = nextafter(aa, ul > 0 ? INFINITY : -INFINITY);
            bad += check(aa, b, y);
            /* offsets d in (-h, h) and shape-value products in [0,1] */
            bad += check((uniform() * 2.0 - 1.0) * b, b, y);
            double p = uniform() * uniform();
            bad += check(p, b, y);
            bad += check(-p, b, y);
            total += 5;
        }
    }
    printf("mismatches %ld of %ld\n", bad, total);
    return bad == 0 ? 0 : 1;
}
