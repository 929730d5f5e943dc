/*
 * oracle_math.c — RNG and elementary functions for the oracle (test
 * infrastructure only; see oracle.h).  Written independently of the
 * library's device code so that the two can be compared bit for bit.
 *
 * Build with -ffp-contract=off: every float operation below must be a single
 * IEEE-754 binary32 operation rounded to nearest.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include "oracle.h"

/* PCG-style hash of res/shader/random.wgsl:14-20.  The reference computes an
 * LCG step into `rng_state` (random.wgsl:17) and never uses it; the output is
 * derived from the raw input state (random.wgsl:18-19). */
uint32_t orc_pcg(uint32_t s) {
    uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (word >> 22u) ^ word;
}

/* Xorshift 13/17/5 of random.wgsl:32-45 (one round, no LCG). */
uint32_t orc_xorshift(uint32_t s) {
    s ^= s << 13u;
    s ^= s >> 17u;
    s ^= s << 5u;
    return s;
}

/* UniformFloat = f32(UniformUint(s)) * 2^-32, random.wgsl:27-29,47-49.
 * The u32 -> f32 conversion rounds to nearest, so 1.0 is reachable. */
float orc_uniform_float(uint32_t s) {
    return (float)orc_xorshift(s) * 0x1p-32f;
}

static inline float bits_to_float(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t float_to_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

/*
 * exp(x) in binary32 by Cody-Waite reduction and a Taylor polynomial:
 *   x = n*ln2 + r, n = rint(x/ln2), |r| <= ln2/2,  exp(x) = 2^n * P(r),
 *   P(r) = sum_{k=0..7} r^k/k!  (truncation error < 6e-9 relative).
 * ln2 is split as LN2_HI = 2839/4096 (12 significant bits, so n*LN2_HI is
 * exact for |n| <= 2^12) and LN2_LO = ln2 - LN2_HI rounded to binary32.
 * Results below FLT_MIN are returned as 0 and above FLT_MAX as +inf.
 * The library's device copy performs the same operation sequence.
 */
#define ORC_LN2_HI 0.693115234375f
#define ORC_LN2_LO 3.19461849452998e-05f   /* ln2 - 2839/4096 */
#define ORC_INV_LN2 1.4426950408889634f      /* 1/ln2 */

float orc_expf(float x) {
    if (!(x == x)) return x;
    if (x > 88.72283f) return INFINITY;
    if (x < -87.33654f) return 0.0f;
    float t = x * ORC_INV_LN2;
    float nf = rintf(t);
    int n = (int)nf;
    float r = x - nf * ORC_LN2_HI;
    r = r - nf * ORC_LN2_LO;
    float p = 1.98412698e-4f;           /* 1/5040 */
    p = p * r + 1.38888889e-3f;         /* 1/720  */
    p = p * r + 8.33333377e-3f;         /* 1/120  */
    p = p * r + 4.16666679e-2f;         /* 1/24   */
    p = p * r + 1.66666672e-1f;         /* 1/6    */
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    if (n == 128) return (p * bits_to_float((uint32_t)(127 + 127) << 23)) * 2.0f;
    return p * bits_to_float((uint32_t)(n + 127) << 23);
}

/*
 * log(x) in binary32: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
 * log(m) = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716, series to s^9.
 * Subnormal inputs are pre-scaled by 2^23.
 */
float orc_logf(float x) {
    if (!(x == x)) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return INFINITY;
    int e_adj = 0;
    if (x < 0x1p-126f) { x = x * 0x1p23f; e_adj = -23; }
    uint32_t b = float_to_bits(x);
    int e = (int)((b >> 23) & 0xFFu) - 127 + e_adj;
    uint32_t mb = (b & 0x7FFFFFu) | 0x3F800000u;
    if (mb > 0x3FB504F3u) { mb -= 0x00800000u; e += 1; }
    float m = bits_to_float(mb);
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float q = 0.222222224f;              /* 2/9 */
    q = q * z + 0.285714298f;            /* 2/7 */
    q = q * z + 0.400000006f;            /* 2/5 */
    q = q * z + 0.666666687f;            /* 2/3 */
    q = q * z + 2.0f;
    float poly = s * q;
    float ef = (float)e;
    return ef * ORC_LN2_HI + (ef * ORC_LN2_LO + poly);
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
 * as easy as 1, 2, 3").  Multipliers and Weyl key increments are the
 * published constants of that algorithm. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        if (r < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
