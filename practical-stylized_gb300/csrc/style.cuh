// style.cuh -- device implementation of the nonlinear style nodes.
//
// Each node restates the corresponding reference `apply_stylization`
// (crates/akari_render/src/svm/surface/mod.rs) in FP32 with CUDA math functions; node
// parameters are laid out as documented in include/sty_gb300.h.
#pragma once

#include "common.cuh"

namespace sty {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 scale3(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ f3 clamp3(f3 a, float lo, float hi) {
    return {clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi)};
}
// Color::lum (crates/akari_render/src/color.rs:356-361)
__device__ __forceinline__ float lum709(f3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
// linear_to_srgb1 / srgb_to_linear1 (color.rs:536-549)
__device__ __forceinline__ float lin2srgb(float v) {
    return v <= 0.0031308f ? v * 12.92f : powf(v, 1.0f / 2.4f) * 1.055f - 0.055f;
}
__device__ __forceinline__ float srgb2lin(float v) {
    return v <= 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
}
__device__ __forceinline__ f3 lin2srgb3(f3 c) { return {lin2srgb(c.x), lin2srgb(c.y), lin2srgb(c.z)}; }
__device__ __forceinline__ f3 srgb2lin3(f3 c) { return {srgb2lin(c.x), srgb2lin(c.y), srgb2lin(c.z)}; }
__device__ __forceinline__ float rem_euclid(float a, float b) {
    float r = fmodf(a, b);
    return r < 0.0f ? r + fabsf(b) : r;
}
// rgb_to_hsv / hsv_to_rgb (color.rs:551-590)
__device__ inline f3 rgb2hsv(f3 c) {
    float mx = fmaxf(c.x, fmaxf(c.y, c.z)), mn = fminf(c.x, fminf(c.y, c.z));
    float diff = mx - mn, h;
    if (mx == mn)
        h = 0.0f;
    else if (mx == c.x)
        h = rem_euclid((c.y - c.z) / diff, 6.0f);
    else if (mx == c.y)
        h = (c.z - c.x) / diff + 2.0f;
    else
        h = (c.x - c.y) / diff + 4.0f;
    h = h / 6.0f;
    float s = mx == 0.0f ? 0.0f : diff / mx;
    return {h, s, mx};
}
__device__ inline f3 hsv2rgb(f3 hsv) {
    auto f = [&](int n) {
        float k = rem_euclid((float)n + hsv.x * 6.0f, 6.0f);
        float m = fmaxf(fminf(fminf(k, 4.0f - k), 1.0f), 0.0f);
        return hsv.z - hsv.z * hsv.y * m;
    };
    return {f(5), f(3), f(1)};
}

__device__ inline f3 style_node(const sty_style_node &nd, uint32_t depth, f3 li, f3 pos) {
    switch (nd.kind) {
        case STY_STYLE_HALF_TONE: {  // mod.rs:1180-1232
            if ((float)depth > nd.p[4]) return li;
            const float lum = (li.x + li.y + li.z) / 3.0f;
            if (lum == 0.0f) return li;
            float r = depth == 0 ? lum / nd.p[1] : roundf(lum / nd.p[0]) / nd.p[1];
            r = 1.0f - clampf(r, 0.0f, 1.0f);
            const float d = nd.p[3];
            r = r * d * 0.5f * nd.p[2];
            const float *A = nd.p + 12;
            const float tp[3] = {A[0] * pos.x + A[1] * pos.y + A[2] * pos.z + A[3],
                                 A[4] * pos.x + A[5] * pos.y + A[6] * pos.z + A[7],
                                 A[8] * pos.x + A[9] * pos.y + A[10] * pos.z + A[11]};
            const float ip[3] = {floorf(tp[0] / d) * d, floorf(tp[1] / d) * d, floorf(tp[2] / d) * d};
            float mind = 1e16f;
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++)
                    for (int k = 0; k < 2; k++) {
                        const float qx = ip[0] + (float)i * d - pos.x, qy = ip[1] + (float)j * d - pos.y,
                                    qz = ip[2] + (float)k * d - pos.z;
                        const float dist = sqrtf(qx * qx + qy * qy + qz * qz);
                        if (dist < mind) mind = dist;
                    }
            const float *tone = mind < r ? nd.p + 6 : nd.p + 9;
            const float b = nd.p[5];
            return {li.x + (tone[0] * li.x - li.x) * b, li.y + (tone[1] * li.y - li.y) * b,
                    li.z + (tone[2] * li.z - li.z) * b};
        }
        case STY_STYLE_TOON: {  // mod.rs:573-610
            const float w = nd.p[0];
            f3 c = clamp3(li, 0.0f, 1e5f);
            float lum = lum709(c);
            if (lum <= 0.0f) return c;
            f3 hue = {c.x / lum, c.y / lum, c.z / lum};
            float nl;
            if (lum > 1.0f) {
                nl = floorf(lum / w) * w;
            } else {
                nl = srgb2lin(floorf(lin2srgb(lum) / w) * w);
            }
            return scale3(hue, nl);
        }
        case STY_STYLE_PALETTE: {  // mod.rs:697-735
            const float indirect_scale = nd.p[0], gamma = nd.p[1];
            f3 c = li;
            float lum = (c.x + c.y + c.z) / 3.0f;
            if (depth != 0) c = {c.x / indirect_scale, c.y / indirect_scale, c.z / indirect_scale};
            c = clamp3(c, 0.0f, 1.0f);
            c = {powf(c.x, gamma), powf(c.y, gamma), powf(c.z, gamma)};
            float min_dist = 1e16f;
            f3 best = {0.0f, 0.0f, 0.0f};
            for (int k = 0; k < nd.n; k++) {
                f3 q = {nd.p[2 + 3 * k], nd.p[3 + 3 * k], nd.p[4 + 3 * k]};
                float dx = q.x - c.x, dy = q.y - c.y, dz = q.z - c.z;
                float dist = dx * dx + dy * dy + dz * dz;
                if (dist < min_dist) {
                    min_dist = dist;
                    best = q;
                }
            }
            float ig = 1.0f / gamma;
            c = {powf(best.x, ig), powf(best.y, ig), powf(best.z, ig)};
            if (depth != 0) {
                float nl = (c.x + c.y + c.z) / 3.0f;
                if (nl != 0.0f) c = scale3(c, lum / nl);
            }
            return c;
        }
        case STY_STYLE_SAT_ADJUST: {  // mod.rs:821-851
            const float power = nd.p[0], indirect_scale = nd.p[1];
            float lum = fmaxf(li.x, fmaxf(li.y, li.z));
            if (lum == 0.0f) return li;
            f3 c = li;
            if (depth != 0) c = {c.x / indirect_scale, c.y / indirect_scale, c.z / indirect_scale};
            c = lin2srgb3(clamp3(c, 0.0f, 1.0f));
            f3 hsv = rgb2hsv(c);
            hsv.y = powf(hsv.y, power);
            c = srgb2lin3(hsv2rgb(hsv));
            if (depth != 0) c = scale3(c, indirect_scale);
            return c;
        }
        case STY_STYLE_SAT_REX: {  // mod.rs:1060-1089
            const float blend = nd.p[0];
            float lum = (li.x + li.y + li.z) / 3.0f;
            float cmin = fminf(li.x, fminf(li.y, li.z));
            if (lum <= 0.0f || cmin < 0.0f) return li;
            float cmax = fmaxf(li.x, fmaxf(li.y, li.z));
            f3 im = {(li.x - cmin) / cmax, (li.y - cmin) / cmax, (li.z - cmin) / cmax};
            float u = (im.x + im.y + im.z) / 3.0f;
            if (u != 0.0f) {
                float k = 1.0f - blend;
                return {blend * lum + k * im.x * lum / u, blend * lum + k * im.y * lum / u,
                        blend * lum + k * im.z * lum / u};
            }
            float v = blend * lum + (1.0f - blend) * lum;
            return {v, v, v};
        }
        case STY_STYLE_EIGHT_BIT: {  // mod.rs:1316-1345
            const float indirect_scale = nd.p[0];
            auto map8 = [](f3 c) {
                f3 s = lin2srgb3(c);
                f3 q = {roundf(s.x * 8.0f) / 8.0f, roundf(s.y * 8.0f) / 8.0f, roundf(s.z * 4.0f) / 4.0f};
                return srgb2lin3(q);
            };
            float lum = fmaxf(li.x, fmaxf(li.y, li.z));
            if (lum == 0.0f) return li;
            if (depth > 0) {
                f3 m = map8({li.x / indirect_scale, li.y / indirect_scale, li.z / indirect_scale});
                return scale3(m, indirect_scale);
            }
            float nl = fminf(lum, 1.0f);
            return map8({li.x / lum * nl, li.y / lum * nl, li.z / lum * nl});
        }
        case STY_STYLE_TOON_STEPS: {
            f3 c = clamp3(li, 0.0f, 1e5f);
            float lum = lum709(c);
            if (lum <= 0.0f) return c;
            int k = 0;
            for (int t = 0; t < nd.n; t++) k += (nd.p[t] <= lum) ? 1 : 0;
            float level = nd.p[8 + k];
            return {c.x / lum * level, c.y / lum * level, c.z / lum * level};
        }
        case STY_STYLE_RAMP_SMOOTH: {
            f3 c = clamp3(li, 0.0f, 1e5f);
            float lum = lum709(c);
            const float s = nd.p[0];
            f3 o = {0.0f, 0.0f, 0.0f}, prev = {0.0f, 0.0f, 0.0f};
            for (int k = 0; k < nd.n; k++) {
                f3 ck = {nd.p[9 + 3 * k], nd.p[10 + 3 * k], nd.p[11 + 3 * k]};
                float sg = 1.0f / (1.0f + expf(-s * (lum - nd.p[1 + k])));
                o.x += sg * (ck.x - prev.x);
                o.y += sg * (ck.y - prev.y);
                o.z += sg * (ck.z - prev.z);
                prev = ck;
            }
            return o;
        }
        default:
            return li;
    }
}

// pos: the shaded point (read by STY_STYLE_HALF_TONE only)
__device__ inline f3 style_apply(const sty_style_program &prog, uint32_t depth, f3 li, f3 pos) {
    const uint32_t bit = depth > 31u ? 31u : depth;
    for (int i = 0; i < prog.n_nodes && i < STY_STYLE_MAX_NODES; i++) {
        const sty_style_node &nd = prog.nodes[i];
        if ((nd.depth_mask >> bit) & 1u) li = style_node(nd, depth, li, pos);
    }
    return li;
}
__device__ inline f3 style_apply(const sty_style_program &prog, uint32_t depth, f3 li) {
    return style_apply(prog, depth, li, f3{0.0f, 0.0f, 0.0f});
}

// Host-side validation of a style program's sizes.
bool style_program_valid(const sty_style_program *p);

}  // namespace sty
