/* CPU check of the integer/float-float helpers the FP32 kernels use
 * (code_mpm_gb300/csrc/fpsplit.h), compiled with gcc -O2 -ffp-contract=off:
 *   fps_cell       when it decides, floor equals floor of the IEEE quotient x/h and the
 *                  fraction is within 2e-7 of x/h - floor;
 *   fps_f2d        equals (double)f bit for bit;
 *   fps_float_threshold  (m > r) == ((double)m > t) for floats around the threshold.
 * Usage: fps_check <samples> <seed>; prints "ok decided=<fraction>" or the first mismatch. */
#include <stdio.h>
#include <stdlib.h>
#include "../../code_mpm_gb300/csrc/fpsplit.h"

static uint64_t s_state;
static uint64_t rnd(void) { /* splitmix64 */
    uint64_t z = (s_state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static double unif(void) { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); }

int main(int argc, char** argv) {
    long long n = argc > 1 ? atoll(argv[1]) : 10000000;
    s_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    long long decided = 0;
    for (long long i = 0; i < n; ++i) {
        /* cell sizes and grid lengths like the scenes' (length / cells), positions over the grid and beyond */
        int cells = 1 + (int)(rnd() % 1200);
        double len = 1e-3 + unif() * 0.5;
        double h = len / (double)cells;
        double y = 1.0 / h;
        float ih = (float)y, il = (float)(y - (double)ih);
        double x;
        switch (rnd() % 4) {
            case 0: x = (unif() * 1.2 - 0.1) * len; break;
            case 1: x = (double)(long long)(unif() * cells) * h; break;             /* on grid planes */
            case 2: x = ((double)(long long)(unif() * cells) + 0.25 * (rnd() % 4)) * h; break; /* quarter points */
            default: x = fps_u2d(rnd() & 0xbfffffffffffffffULL); break;             /* any magnitude */
        }
        float f, u;
        if (!fps_cell(x, ih, il, &f, &u)) continue;
        ++decided;
        double q = x / h;
        double fl = floor(q);
        if ((double)f != fl || fabs((double)u - (q - fl)) > 2e-7) {
            printf("mismatch x=%.17g h=%.17g q=%.17g floor=%.17g got f=%.9g u=%.9g\n", x, h, q, fl, f, u);
            return 1;
        }
    }
    for (long long i = 0; i < n; ++i) {
        float f = fps_u2f((uint32_t)rnd());
        double a = fps_f2d(f), b = (double)f;
        if (fps_d2u(a) != fps_d2u(b) && !(a != a && b != b)) {
            printf("f2d mismatch %a\n", f);
            return 1;
        }
    }
    for (long long i = 0; i < 100000; ++i) {
        double t = (rnd() % 8 == 0) ? 0.0 : unif() * pow(10.0, (double)(rnd() % 40) - 30.0);
        float r = fps_float_threshold(t);
        float m = (float)t;
        for (int k = 0; k < 4; ++k) {
            if ((m > r) != ((double)m > t)) {
                printf("threshold mismatch t=%.17g m=%a r=%a\n", t, m, r);
                return 1;
            }
            m = nextafterf(m, k < 2 ? INFINITY : -INFINITY);
        }
    }
    printf("ok decided=%.6f\n", (double)decided / (double)n);
    return 0;
}
