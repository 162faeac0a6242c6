/* The division by a divisor known ahead (div_known in
 * astrophage-microscope_gb300/csrc/dev.cuh: Markstein's correction step on a
 * precomputed reciprocal, accepted only under an exact half-ulp residual test,
 * else the IEEE division), restated operation for operation in C (fma,
 * compiled without contraction) and checked against the IEEE quotient a / b.
 * Divisors: the voxel volumes of the benchmark's CO2 grids, the deposit
 * scales, and random ones; dividends: random over many binades, and placed
 * next to quotient rounding midpoints. Test infrastructure.
 * Usage: div_known_check RANDOM_PER_DIVISOR ADVERSARIAL_PER_DIVISOR
 * Prints "checked N mismatches M fallbacks F"; exits 1 on any mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t rs = 0x9E3779B97F4A7C15ull;
static uint64_t rnd(void) { rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17; return rs; }
static double asd(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t asu(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static long fallbacks;

static double div_known(double a, double b, double y) {
    const double q = a * y;
    const double q1 = fma(fma(-b, q, a), y, q);
    const uint64_t bits = asu(q1);
    const int e = (int)((bits >> 52) & 0x7FFu);
    if (e > 53 && e < 2047 && (bits & 0xFFFFFFFFFFFFFull) != 0) {
        const double h = b * asd((uint64_t)(e - 53) << 52);
        if (h >= 2.2250738585072014e-308 && fabs(fma(-b, q1, a)) < h) return q1;
    }
    ++fallbacks;
    return a / b;
}

/* A double with a random significand and an exponent in [lo, hi]. */
static double rand_in(int lo, int hi) {
    const int e = lo + (int)(rnd() % (uint64_t)(hi - lo + 1));
    const uint64_t m = rnd() & 0xFFFFFFFFFFFFFull;
    return asd(((uint64_t)(e + 1023) << 52) | m);
}

int main(int argc, char** argv) {
    const long nr = argc > 1 ? atol(argv[1]) : 1000000, na = argc > 2 ? atol(argv[2]) : 1000000;
    double divisors[64];
    int nd = 0;
    const double edges[] = {4e-3 / 64, 4e-3 / 128, 4e-3 / 192, 4e-3 / 256, 1e-3 / 32, 1e-3 / 48, 1e-3 / 96};
    for (int k = 0; k < 7; ++k) divisors[nd++] = edges[k] * edges[k] * edges[k];     /* cubic voxels */
    divisors[nd++] = (4e-3 / 256) * (4e-3 / 256) * 60e-6;                            /* depth-averaged */
    divisors[nd++] = 1e9;
    divisors[nd++] = 1e15;
    divisors[nd++] = 1e18;
    while (nd < 40) divisors[nd++] = rand_in(-60, 60);
    long checked = 0, bad = 0;
    for (int k = 0; k < nd; ++k) {
        const double b = divisors[k], y = 1.0 / b;
        for (long i = 0; i < nr; ++i) {
            double a = rand_in(-80, 80);
            if (rnd() & 1) a = -a;
            const double got = div_known(a, b, y), want = a / b;
            ++checked;
            if (asu(got) != asu(want)) { if (bad < 5) printf("mismatch a=%a b=%a got=%a want=%a\n", a, b, got, want); ++bad; }
        }
        /* Dividends whose quotient lies next to a midpoint between two doubles:
         * a = RN(b m) for m = q + ulp(q)/2 (+- a few ulps of a), q random. */
        for (long i = 0; i < na; ++i) {
            const double q = rand_in(-40, 40);
            double a = b * ((q + nextafter(q, INFINITY)) * 0.5);
            const int wig = (int)(rnd() % 7) - 3;
            for (int w = 0; w < abs(wig); ++w) a = nextafter(a, wig > 0 ? INFINITY : -INFINITY);
            const double got = div_known(a, b, y), want = a / b;
            ++checked;
            if (asu(got) != asu(want)) { if (bad < 5) printf("mismatch a=%a b=%a got=%a want=%a\n", a, b, got, want); ++bad; }
        }
    }
    printf("checked %ld mismatches %ld fallbacks %ld\n", checked, bad, fallbacks);
    return bad ? 1 : 0;
}
