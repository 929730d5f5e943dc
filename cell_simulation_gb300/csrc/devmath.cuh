// devmath.cuh — device RNG and elementary functions.  Every floating-point
// operation uses an explicit round-to-nearest intrinsic so that no multiply
// is contracted into an FMA: the results are the IEEE-754 binary32 values of
// the written expression, identical on every run and on any IEEE host.
#pragma once
#include <cstdint>

namespace cellsim {

// PCG-style hash of res/shader/random.wgsl:14-20 (the LCG step the shader
// stores in `rng_state` is unused; the output comes from the raw state).
__device__ __forceinline__ uint32_t d_pcg(uint32_t s) {
    uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (word >> 22u) ^ word;
}

// UniformUint, random.wgsl:32-45: one xorshift 13/17/5 round.
__device__ __forceinline__ uint32_t d_xorshift(uint32_t s) {
    s ^= s << 13u;
    s ^= s >> 17u;
    s ^= s << 5u;
    return s;
}

// UniformFloat, random.wgsl:27-29,47-49: f32(u) * 2^-32 (round to nearest).
__device__ __forceinline__ float d_uniform_float(uint32_t s) {
    return __fmul_rn(__uint2float_rn(d_xorshift(s)), 0x1p-32f);
}

// exp(x): Cody-Waite reduction x = n ln2 + r with ln2 = 2839/4096 + lo and a
// degree-7 Taylor polynomial, results below FLT_MIN flushed to 0.
__device__ __forceinline__ float d_expf(float x) {
    const float LN2_HI = 0.693115234375f;        // 2839/4096
    const float LN2_LO = 3.19461849452998e-05f;  // ln2 - 2839/4096
    const float INV_LN2 = 1.4426950408889634f;
    if (!(x == x)) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -87.33654f) return 0.0f;
    float nf = rintf(__fmul_rn(x, INV_LN2));
    int n = (int)nf;
    float r = __fsub_rn(x, __fmul_rn(nf, LN2_HI));
    r = __fsub_rn(r, __fmul_rn(nf, LN2_LO));
    float p = 1.98412698e-4f;
    p = __fadd_rn(__fmul_rn(p, r), 1.38888889e-3f);
    p = __fadd_rn(__fmul_rn(p, r), 8.33333377e-3f);
    p = __fadd_rn(__fmul_rn(p, r), 4.16666679e-2f);
    p = __fadd_rn(__fmul_rn(p, r), 1.66666672e-1f);
    p = __fadd_rn(__fmul_rn(p, r), 0.5f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f);
    if (n == 128) return __fmul_rn(__fmul_rn(p, __int_as_float((127 + 127) << 23)), 2.0f);
    return __fmul_rn(p, __int_as_float((n + 127) << 23));
}

// log(x): x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
// s = (m-1)/(m+1), odd series to s^9.
__device__ __forceinline__ float d_logf(float x) {
    const float LN2_HI = 0.693115234375f;
    const float LN2_LO = 3.19461849452998e-05f;
    if (!(x == x)) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e_adj = 0;
    if (x < 0x1p-126f) { x = __fmul_rn(x, 0x1p23f); e_adj = -23; }
    uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xFFu) - 127 + e_adj;
    uint32_t mb = (b & 0x7FFFFFu) | 0x3F800000u;
    if (mb > 0x3FB504F3u) { mb -= 0x00800000u; e += 1; }
    float m = __uint_as_float(mb);
    float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    float z = __fmul_rn(s, s);
    float q = 0.222222224f;
    q = __fadd_rn(__fmul_rn(q, z), 0.285714298f);
    q = __fadd_rn(__fmul_rn(q, z), 0.400000006f);
    q = __fadd_rn(__fmul_rn(q, z), 0.666666687f);
    q = __fadd_rn(__fmul_rn(q, z), 2.0f);
    float poly = __fmul_rn(s, q);
    float ef = (float)e;
    return __fadd_rn(__fmul_rn(ef, LN2_HI), __fadd_rn(__fmul_rn(ef, LN2_LO), poly));
}

// Philox4x32-10 (Salmon et al., SC'11), published multipliers and Weyl
// increments.
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 d_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        if (r < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
    return U4{c0, c1, c2, c3};
}

}  // namespace cellsim
