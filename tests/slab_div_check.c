/* Checks the slab division of the traversal (slab_div in
 * aurora_gb300/csrc/aur_traverse.cuh): with y = RN(1/d) and q = RN(a*y),
 * RN(q + fma(-q, d, a) * y) must equal RN(a/d) bit for bit whenever
 * |y| is in [2^-40, 2^40] and the result's magnitude is in [2^-59, 2^100]
 * (the only cases the traversal takes it). Random numerators from subnormal
 * to near overflow, with mantissa patterns that stress the rounding.
 * Usage: slab_div_check N  -> prints "<cases> <accepted> <mismatches>". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint64_t next(void) {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}
static float from_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float make(int emin, int emax, uint32_t mant) {
    const int e = emin + (int)(next() % (uint64_t)(emax - emin + 1));
    const uint32_t sign = (uint32_t)(next() & 1u) << 31;
    if (e < -126) return from_bits(sign | (mant & 0x7FFFFFu));
    return from_bits(sign | ((uint32_t)(e + 127) << 23) | (mant & 0x7FFFFFu));
}

int main(int argc, char** argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 10000000LL;
    long long accepted = 0, bad = 0;
    for (long long i = 0; i < n; ++i) {
        uint32_t md = (uint32_t)next(), ma = (uint32_t)next();
        switch (i & 7) {
            case 0: md = 0x7FFFFFu; break;   /* divisor mantissa all ones */
            case 1: md = 0u; break;          /* divisor a power of two */
            case 2: ma = md; break;          /* equal mantissas */
            case 3: ma = 0x7FFFFFu; break;
            case 4: ma = md ^ 1u; break;
            default: break;
        }
        const float d = make(-45, 45, md);
        const float a = make(-140, 127, ma);
        const float y = 1.0f / d;
        const float q = a * y;
        const float f = fmaf(fmaf(-q, d, a), y, q);
        const float my = fabsf(y), m = fabsf(f);
        if (!(my >= 0x1p-40f && my <= 0x1p40f && m >= 0x1p-59f && m <= 0x1p100f)) continue;
        ++accepted;
        if (to_bits(f) != to_bits(a / d)) ++bad;
    }
    printf("%lld %lld %lld\n", n, accepted, bad);
    return bad != 0;
}
