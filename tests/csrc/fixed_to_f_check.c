/* The flush's fixed-point -> float conversion (fixed_to_f in
 * astrophage-microscope_gb300/csrc/dev.cuh), restated operation for operation
 * in C (float arithmetic, fmaf, llrintf; compiled without contraction), checked
 * against the reference's (float)((double)raw / scale) (fixed_atomic.cuh:31-33,
 * diffuse.cu:57) on random deposits and on deposits placed next to float
 * rounding midpoints, at the three deposit scales. Test infrastructure.
 * Usage: fixed_to_f_check RANDOM_PER_SCALE ADVERSARIAL_PER_SCALE
 * Prints "checked N mismatches M fallbacks F"; exits 1 on any mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t rs = 88172645463325252ull;
static uint64_t rnd(void) { rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17; return rs; }
static float asf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t asu(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static long fallbacks;

static float fixed_to_f(long long raw, float inv_hi, float inv_lo, double scale) {
    const float r_hi = (float)raw;
    const float r_lo = (float)(raw - llrintf(r_hi));
    const float p = r_hi * inv_hi;
    const float e = fmaf(r_hi, inv_hi, -p);
    const float c = e + fmaf(r_hi, inv_lo, r_lo * inv_hi);
    const float f = p + c;
    const float bb = f - p;
    const float t = (p - (f - bb)) + (c - bb);
    const float af = fabsf(f);
    const uint32_t ab = asu(af);
    const float lim = asf(ab & 0x7F800000u) * ((ab & 0x7FFFFFu) ? 0x1p-24f : 0x1p-25f);
    if (fabsf(t) + af * 0x1p-43f < lim) return f;
    ++fallbacks;
    return (float)((double)raw / scale);
}

int main(int argc, char** argv) {
    const long nr = argc > 1 ? atol(argv[1]) : 1000000, na = argc > 2 ? atol(argv[2]) : 1000000;
    const double scales[] = {1e9, 1e15, 1e18};      /* temperature; CO2 and N2; irradiance */
    long n = 0, bad = 0;
    for (int si = 0; si < 3; ++si) {
        const double sc = scales[si];
        const float ih = (float)(1.0 / sc), il = (float)(1.0 / sc - (double)ih);
        for (long it = 0; it < nr; ++it) {
            const int bits = 1 + (int)(rnd() % 56);
            long long raw = (long long)(rnd() >> (64 - bits));
            if (rnd() & 1) raw = -raw;
            if (raw == 0) continue;
            if (asu((float)((double)raw / sc)) != asu(fixed_to_f(raw, ih, il, sc))) ++bad;
            ++n;
        }
        for (long it = 0; it < na; ++it) {
            float f = asf((uint32_t)(rnd() % 0x3F800000u) + 0x20000000u);
            if (it % 7 == 0) f = asf(asu(f) & 0xFF800000u);
            double m = (double)f + (double)(nextafterf(f, INFINITY) - f) * 0.5;
            if (it & 1) m = (double)f - (double)(f - nextafterf(f, 0.0f)) * 0.5;
            const double rr = m * sc;
            if (fabs(rr) > 9.0e15 || fabs(rr) < 1.0) continue;
            const long long raw = llround(rr) + (long long)(rnd() % 5) - 2;
            if (raw == 0) continue;
            if (asu((float)((double)raw / sc)) != asu(fixed_to_f(raw, ih, il, sc))) ++bad;
            ++n;
        }
    }
    printf("checked %ld mismatches %ld fallbacks %ld\n", n, bad, fallbacks);
    return bad != 0;
}
