// rng.cuh -- the reference's per-path seeding and the exactly specified arithmetic of the camera.
//
// Seeding. Every NL-PF / NL-NRC path slot i starts from Pcg32::new_seq_offset(i, seed_i) where
// seed_i is the i-th `gen::<u64>()` of `StdRng::seed_from_u64(seed)` (init_pcg32_buffer_with_seed,
// crates/akari_render/src/sampler/mod.rs:157-173). The reference pins rand 0.8.5 / rand_chacha
// 0.3.1 / rand_core 0.6.4 (Cargo.lock:1716-1738): StdRng is ChaCha12Rng, so
//   - seed_from_u64 (rand_core 0.6.4) expands the u64 into the 32-byte key with the PCG32 output
//     function applied to a 64-bit LCG state that is advanced before each 4-byte word is taken
//     (multiplier 6364136223846793005, increment 11634580027462260723), words little-endian;
//   - ChaCha12Rng (rand_chacha 0.3.1) is Bernstein's ChaCha with 12 rounds, a 64-bit block counter
//     in state words 12-13 starting at 0 and a zero 64-bit stream id in words 14-15; its output is
//     the keystream read as little-endian u32 words in block order;
//   - gen::<u64>() (BlockRng::next_u64) takes two consecutive words, the first as the low half.
//     Starting from an empty buffer every u64 takes an aligned word pair, so the i-th u64 is words
//     (2i, 2i + 1) of the keystream: block i / 8, words 2 (i % 8) and 2 (i % 8) + 1.
// Each path therefore derives its seed from one ChaCha block, with no sequential generator.
//
// Camera arithmetic. The camera ray of a path (camera/mod.rs:73-126 with the pixel filter of
// film.rs:30-48) is written with explicitly rounded operations (__fmul_rn, __fadd_rn, __fmaf_rn,
// ...), so the compiler cannot contract or reorder it and a CPU restatement with the same
// operations reproduces every ray bit for bit. The Gaussian filter's logarithm, sine and cosine
// are computed here from their series (below), not by the CUDA math library, for the same reason.
#pragma once

#include <stdint.h>

namespace sty {

// ---- ChaCha (D. J. Bernstein, "ChaCha, a variant of Salsa20", 2008) --------------------------
__host__ __device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
__host__ __device__ __forceinline__ void chacha_qr(uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d) {
    a += b; d ^= a; d = rotl32(d, 16);
    c += d; b ^= c; b = rotl32(b, 12);
    a += b; d ^= a; d = rotl32(d, 8);
    c += d; b ^= c; b = rotl32(b, 7);
}
// out = rounds / 2 double rounds (column then diagonal quarter rounds) of `in`, plus `in`
__host__ __device__ __forceinline__ void chacha_block(const uint32_t in[16], uint32_t out[16], int rounds) {
    uint32_t x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = in[k];
    for (int r = 0; r < rounds; r += 2) {
        chacha_qr(x[0], x[4], x[8], x[12]);
        chacha_qr(x[1], x[5], x[9], x[13]);
        chacha_qr(x[2], x[6], x[10], x[14]);
        chacha_qr(x[3], x[7], x[11], x[15]);
        chacha_qr(x[0], x[5], x[10], x[15]);
        chacha_qr(x[1], x[6], x[11], x[12]);
        chacha_qr(x[2], x[7], x[8], x[13]);
        chacha_qr(x[3], x[4], x[9], x[14]);
    }
#pragma unroll
    for (int k = 0; k < 16; k++) out[k] = x[k] + in[k];
}

// rand_core 0.6.4 SeedableRng::seed_from_u64 for a 32-byte seed: 8 little-endian key words
__host__ __device__ inline void std_rng_key(uint64_t seed, uint32_t key[8]) {
    uint64_t s = seed;
    for (int k = 0; k < 8; k++) {
        s = s * 6364136223846793005ull + 11634580027462260723ull;
        const uint32_t xs = (uint32_t)(((s >> 18) ^ s) >> 27);
        const uint32_t rot = (uint32_t)(s >> 59);
        key[k] = (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
}

// The i-th gen::<u64>() of ChaCha12Rng keyed by `key` (block i / 8 of the keystream)
__host__ __device__ inline uint64_t std_rng_u64(const uint32_t key[8], uint64_t i) {
    const uint64_t blk = i >> 3;
    uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,  // "expand 32-byte k"
                       key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                       (uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u};
    uint32_t out[16];
    chacha_block(in, out, 12);
    const int w = 2 * (int)(i & 7);
    return (uint64_t)out[w] | ((uint64_t)out[w + 1] << 32);
}

// ---- exactly specified logarithm and sine / cosine ---------------------------------------
// ln(x) for finite x > 0: x = m 2^e with m in [sqrt(2)/2, sqrt(2)), ln m = 2 atanh(s),
// s = (m - 1) / (m + 1), |s| <= 0.1716, by its series to s^11 (truncation below 1e-10 relative);
// ln x = e ln 2 + ln m. x = 0 gives -inf.
__device__ __forceinline__ float ex_ln(float x) {
    if (x == 0.0f) return __int_as_float(0xff800000);
    const uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    float p = 0.18181818f;                      // 2/11
    p = __fmaf_rn(p, s2, 0.22222222f);          // 2/9
    p = __fmaf_rn(p, s2, 0.28571429f);          // 2/7
    p = __fmaf_rn(p, s2, 0.4f);                 // 2/5
    p = __fmaf_rn(p, s2, 0.66666667f);          // 2/3
    const float lm = __fmaf_rn(__fmul_rn(s, s2), p, __fmul_rn(2.0f, s));
    return __fmaf_rn((float)e, 0.69314718f, lm);
}
// sin and cos of 2 pi t for t in [0, 1] (t in turns): quadrant k = rint(4t), f = t - k / 4 in
// [-1/8, 1/8] (exact), x = 2 pi f, Taylor series of sin to x^11 and cos to x^12 (|x| <= pi / 4:
// truncation below 1e-11), then the quadrant's symmetry.
__device__ __forceinline__ void ex_sincos_turns(float t, float *sn, float *cs) {
    const float k = rintf(__fmul_rn(t, 4.0f));
    const float f = __fsub_rn(t, __fmul_rn(k, 0.25f));
    const float x = __fmul_rn(f, 6.28318531f);
    const float x2 = __fmul_rn(x, x);
    float ps = -2.5052108e-08f;                 // -1/11!
    ps = __fmaf_rn(ps, x2, 2.7557319e-06f);     // 1/9!
    ps = __fmaf_rn(ps, x2, -1.9841270e-04f);    // -1/7!
    ps = __fmaf_rn(ps, x2, 8.3333333e-03f);     // 1/5!
    ps = __fmaf_rn(ps, x2, -1.6666667e-01f);    // -1/3!
    const float s = __fmaf_rn(__fmul_rn(x, x2), ps, x);
    float pc = 2.0876757e-09f;                  // 1/12!
    pc = __fmaf_rn(pc, x2, -2.7557319e-07f);    // -1/10!
    pc = __fmaf_rn(pc, x2, 2.4801587e-05f);     // 1/8!
    pc = __fmaf_rn(pc, x2, -1.3888889e-03f);    // -1/6!
    pc = __fmaf_rn(pc, x2, 4.1666667e-02f);     // 1/4!
    pc = __fmaf_rn(pc, x2, -0.5f);              // -1/2!
    const float c = __fmaf_rn(x2, pc, 1.0f);
    const int q = ((int)k) & 3;
    *sn = q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
    *cs = q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}

}  // namespace sty
