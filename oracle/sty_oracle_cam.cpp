// sty_oracle_cam.cpp -- TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference's path
// seeding and camera rays, the checker of the library's device-side versions.
//
// Seeding (crates/akari_render/src/sampler/mod.rs:157-173, init_pcg32_buffer_with_seed): path slot i
// starts from Pcg32::new_seq_offset(i, seed_i), seed_i = the i-th rng.gen::<u64>() of
// StdRng::seed_from_u64(seed). The reference pins rand 0.8.5, rand_chacha 0.3.1 and rand_core
// 0.6.4 (Cargo.lock:1716-1738); none of them is in the reference tree, so their published
// algorithms are restated here as those crates define them:
//   - rand_core 0.6.4 SeedableRng::seed_from_u64: a 64-bit LCG (multiplier 6364136223846793005,
//     increment 11634580027462260723) advanced before each 4-byte chunk, the chunk being the PCG
//     XSH-RR output of the advanced state, little-endian, 8 chunks for the 32-byte key;
//   - rand 0.8.5 StdRng = rand_chacha 0.3.1 ChaCha12Rng: ChaCha (Bernstein 2008) with 12 rounds,
//     key = the seed, 64-bit block counter (state words 12-13) from 0, stream id 0 (words 14-15);
//     the generator fills a buffer of 4 consecutive blocks (64 words) at a time;
//   - rand_core BlockRng::next_u64 reads two words (low word first) and refills when fewer than
//     two remain, consuming the buffer sequentially.
// This file follows those definitions literally (sequential generator with a 64-word buffer); the
// library computes seed_i from block i / 8 directly. Pinning: the ChaCha block function is checked
// at 20 rounds against the published RFC 8439 test vectors (tests/test_oracle.py); the seed
// expansion constants are restated from rand_core's published source and have no vector.
//
// Camera rays (PerspectiveCamera::generate_ray, crates/akari_render/src/camera/mod.rs:73-126, and
// PixelFilter::sample, crates/akari_render/src/film.rs:30-48): the same explicitly rounded float
// operations as the library's camera (std::fmaf where it fuses, one rounding per operation
// otherwise; this file is compiled with -ffp-contract=off), and the same series logarithm and
// sine / cosine (their Taylor coefficients are the mathematical constants written out).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sty_oracle.h"

namespace {

inline uint32_t rotl(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

#define QR(a, b, c, d)             \
    a += b; d ^= a; d = rotl(d, 16); \
    c += d; b ^= c; b = rotl(b, 12); \
    a += b; d ^= a; d = rotl(d, 8);  \
    c += d; b ^= c; b = rotl(b, 7);

void block(const uint32_t in[16], uint32_t out[16], int rounds) {
    uint32_t x[16];
    memcpy(x, in, sizeof(x));
    for (int r = 0; r < rounds; r += 2) {
        QR(x[0], x[4], x[8], x[12]);
        QR(x[1], x[5], x[9], x[13]);
        QR(x[2], x[6], x[10], x[14]);
        QR(x[3], x[7], x[11], x[15]);
        QR(x[0], x[5], x[10], x[15]);
        QR(x[1], x[6], x[11], x[12]);
        QR(x[2], x[7], x[8], x[13]);
        QR(x[3], x[4], x[9], x[14]);
    }
    for (int k = 0; k < 16; k++) out[k] = x[k] + in[k];
}

// rand_core::SeedableRng::seed_from_u64 for a 32-byte seed
void seed_from_u64(uint64_t state, uint8_t seed[32]) {
    for (int c = 0; c < 8; c++) {
        state = state * 6364136223846793005ull + 11634580027462260723ull;
        const uint64_t s = state;
        const uint32_t xorshifted = (uint32_t)(((s >> 18) ^ s) >> 27);
        const uint32_t rot = (uint32_t)(s >> 59);
        const uint32_t x = (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
        for (int b = 0; b < 4; b++) seed[4 * c + b] = (uint8_t)(x >> (8 * b));
    }
}

// ChaCha12Rng behind rand_core's BlockRng: a buffer of 4 blocks, consumed word by word
struct ChaCha12Rng {
    uint32_t key[8];
    uint64_t counter = 0;
    uint32_t results[64];
    size_t index = 64;
    explicit ChaCha12Rng(const uint8_t seed[32]) {
        for (int k = 0; k < 8; k++)
            key[k] = (uint32_t)seed[4 * k] | ((uint32_t)seed[4 * k + 1] << 8) | ((uint32_t)seed[4 * k + 2] << 16) |
                     ((uint32_t)seed[4 * k + 3] << 24);
    }
    void generate() {
        for (int b = 0; b < 4; b++) {
            const uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2],
                                     key[3], key[4], key[5], key[6], key[7], (uint32_t)counter,
                                     (uint32_t)(counter >> 32), 0u, 0u};
            block(in, results + 16 * b, 12);
            counter++;
        }
    }
    uint64_t next_u64() {
        if (index < 63) {
            const uint64_t v = (uint64_t)results[index] | ((uint64_t)results[index + 1] << 32);
            index += 2;
            return v;
        }
        if (index >= 64) {
            generate();
            index = 2;
            return (uint64_t)results[0] | ((uint64_t)results[1] << 32);
        }
        const uint64_t lo = results[63];
        generate();
        index = 1;
        return lo | ((uint64_t)results[0] << 32);
    }
};

inline uint32_t pcg_next(sty_pcg32 &g) {
    const uint64_t old = g.state;
    g.state = old * 0x5851f42d4c957f2dull + g.inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}
inline float next_1d(sty_pcg32 &g) { return (float)pcg_next(g) * 2.3283064e-10f; }

// the series logarithm of the library's camera (atanh series of ln m, m in [sqrt(2)/2, sqrt(2)))
float ex_ln(float x) {
    if (x == 0.0f) return -INFINITY;
    uint32_t b;
    memcpy(&b, &x, 4);
    int e = (int)((b >> 23) & 0xffu) - 127;
    const uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.18181818f;
    p = std::fmaf(p, s2, 0.22222222f);
    p = std::fmaf(p, s2, 0.28571429f);
    p = std::fmaf(p, s2, 0.4f);
    p = std::fmaf(p, s2, 0.66666667f);
    const float lm = std::fmaf(s * s2, p, 2.0f * s);
    return std::fmaf((float)e, 0.69314718f, lm);
}
// sine and cosine of 2 pi t (t in turns) by quadrant reduction and Taylor series
void ex_sincos_turns(float t, float *sn, float *cs) {
    const float k = std::rint(t * 4.0f);
    const float f = t - k * 0.25f;
    const float x = f * 6.28318531f;
    const float x2 = x * x;
    float ps = -2.5052108e-08f;
    ps = std::fmaf(ps, x2, 2.7557319e-06f);
    ps = std::fmaf(ps, x2, -1.9841270e-04f);
    ps = std::fmaf(ps, x2, 8.3333333e-03f);
    ps = std::fmaf(ps, x2, -1.6666667e-01f);
    const float s = std::fmaf(x * x2, ps, x);
    float pc = 2.0876757e-09f;
    pc = std::fmaf(pc, x2, -2.7557319e-07f);
    pc = std::fmaf(pc, x2, 2.4801587e-05f);
    pc = std::fmaf(pc, x2, -1.3888889e-03f);
    pc = std::fmaf(pc, x2, 4.1666667e-02f);
    pc = std::fmaf(pc, x2, -0.5f);
    const float c = std::fmaf(x2, pc, 1.0f);
    const int q = ((int)k) & 3;
    *sn = q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
    *cs = q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}

}  // namespace

extern "C" {

void orc_chacha_block(const uint32_t *in, uint32_t *out, int32_t rounds) { block(in, out, rounds); }

void orc_std_rng_key(uint64_t seed, uint32_t *key) {
    uint8_t s[32];
    seed_from_u64(seed, s);
    for (int k = 0; k < 8; k++)
        key[k] = (uint32_t)s[4 * k] | ((uint32_t)s[4 * k + 1] << 8) | ((uint32_t)s[4 * k + 2] << 16) |
                 ((uint32_t)s[4 * k + 3] << 24);
}

void orc_std_rng_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t *out) {
    uint8_t s[32];
    seed_from_u64(seed, s);
    ChaCha12Rng rng(s);
    for (uint64_t i = 0; i < first; i++) rng.next_u64();
    for (uint64_t i = 0; i < n; i++) out[i] = rng.next_u64();
}

// Depth-0 rays of every slot i = b * W * H + px (origin, direction, 0, 1e20), as sty_scene_camera_rays.
void orc_camera_rays(const sty_camera *cam, uint32_t branch, uint64_t seed, float *rays) {
    const uint32_t W = cam->width, H = cam->height;
    const uint64_t npx = (uint64_t)W * H, n = npx * branch;
    // camera frame in double, rounded once (as the library's make_camera)
    double f[3], r[3], u[3];
    for (int a = 0; a < 3; a++) f[a] = (double)cam->target[a] - (double)cam->eye[a];
    double l = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (int a = 0; a < 3; a++) f[a] /= l;
    r[0] = f[1] * cam->up[2] - f[2] * cam->up[1];
    r[1] = f[2] * cam->up[0] - f[0] * cam->up[2];
    r[2] = f[0] * cam->up[1] - f[1] * cam->up[0];
    l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int a = 0; a < 3; a++) r[a] /= l;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    float fw[3], rt[3], up[3];
    for (int a = 0; a < 3; a++) {
        fw[a] = (float)f[a];
        rt[a] = (float)r[a];
        up[a] = (float)u[a];
    }
    const float tan_half = (float)std::tan((double)cam->fov_y * 0.5 * 3.14159265358979323846 / 180.0);
    const float aspect = (float)((double)W / (double)H);
    const float rad = cam->filter_radius;
    std::vector<uint64_t> seeds(n);
    orc_std_rng_u64(seed, 0, n, seeds.data());
    for (uint64_t i = 0; i < n; i++) {
        sty_pcg32 g;  // Pcg32::new_seq_offset(i, seed_i), sampler/mod.rs:94-100
        g.state = 0;
        g.inc = (i << 1) | 1ull;
        pcg_next(g);
        g.state += seeds[i];
        pcg_next(g);
        const uint64_t px = i % npx;
        const float fx = (float)(px % W) + 0.5f, fy = (float)(px / W) + 0.5f;
        const float u0 = next_1d(g), u1 = next_1d(g);
        float ox, oy;
        if (cam->filter == STY_FILTER_GAUSSIAN) {
            const float sigma = rad / 3.0f;
            const float rr = std::sqrt(-2.0f * ex_ln(u0));
            float sn, cs;
            ex_sincos_turns(u1, &sn, &cs);
            ox = std::fmin(std::fmax((rr * cs) * sigma, -rad), rad);
            oy = std::fmin(std::fmax((rr * sn) * sigma, -rad), rad);
        } else {
            ox = (u0 - 0.5f) * rad;
            oy = (u1 - 0.5f) * rad;
        }
        const float ndx = (2.0f * (fx + ox)) / (float)W - 1.0f;
        const float ndy = 1.0f - (2.0f * (fy + oy)) / (float)H;
        const float sx = (ndx * tan_half) * aspect, sy = ndy * tan_half;
        const float dx = std::fmaf(up[0], sy, std::fmaf(rt[0], sx, fw[0]));
        const float dy = std::fmaf(up[1], sy, std::fmaf(rt[1], sx, fw[1]));
        const float dz = std::fmaf(up[2], sy, std::fmaf(rt[2], sx, fw[2]));
        const float inv = 1.0f / std::sqrt(std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx)));
        float *o = rays + 8 * i;
        o[0] = cam->eye[0];
        o[1] = cam->eye[1];
        o[2] = cam->eye[2];
        o[3] = dx * inv;
        o[4] = dy * inv;
        o[5] = dz * inv;
        o[6] = 0.0f;
        o[7] = 1e20f;
    }
}

}  // extern "C"
