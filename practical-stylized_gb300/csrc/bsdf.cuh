// bsdf.cuh -- the reference's principled BSDF (crates/akari_render/src/svm/surface/principled.rs:
// 118-330) restated on the device, in the shading frame (z = normal), FP32.
//
// Composition (outermost first; "add" = BsdfBlendMode::Addictive: f_a + f_b, pdf lerp(pdf_a, pdf_b,
// frac); "mix" = BsdfBlendMode::Mix: lerp of f and pdf, a skipped when frac >= 1 - 1e-4, b when
// frac <= 1e-4; mod.rs:1536-1690):
//   L5 = add(coat_w * A(coat_rough, |cos_o|, coat_ior), scaled(L4, lerp(1, coat_tint (1 - A), coat_w)), coat)
//   L4 = emissive(L3)                                   (emission is the material's; pass-through here)
//   L3 = mix(metallic, L2, metal)
//   L2 = add(f0 lum(spec_tint) A(rough, |cos_o|, eta_s), scaled(L1, 1 - spec_tint f0 A), spec)
//   L1 = mix(transmission, diffuse, dielectric)
//   dielectric = add(Fr_dielectric(cos_o, ior), transmission(sqrt(base)), reflection(base))
// with f0 = ((ior - 1) / (ior + 1))^2 (times 2 specular_ior_level when that is not 0.5, eta_s =
// ior_from_f0(f0)), spec = microfacet reflection of colour spec_tint f0 and dielectric Fresnel
// eta_s, metal = microfacet reflection with the complex Fresnel of Gulbrandsen's
// artistic_to_conductor_fresnel(base, spec_tint), coat = microfacet reflection of colour coat_w with
// dielectric Fresnel coat_ior; Trowbridge-Reitz alpha = max(roughness^2, 1e-4), visible-normal
// sampling (mod.rs:1871-2097, microfacet.rs:24-211). A(r, mu, eta) is the table
// ggx_dielectric_s (precompute.rs:56-145): the mean of f/pdf of a unit-colour dielectric GGX
// reflection sampled at (roughness r, cos mu, ior), over a 16^3 grid read trilinearly.
// Sampling picks a lobe per mixture with weighted_discrete_choice2_and_remap (b when u < frac,
// u remapped; sampling.rs:61-71), samples it with the remaining 2-D sample, and the closure is then
// evaluated at the sampled direction (SurfaceClosure::sample, mod.rs:1846-1869).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sty_gb300.h"

namespace sty {
namespace bsdf {

constexpr float kPiB = 3.14159265358979323846f;
constexpr int kTabN = 16;  // ggx_dielectric_s is kTabN^3

struct B3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ B3 b3(float x, float y, float z) { return {x, y, z}; }
__host__ __device__ __forceinline__ B3 add(B3 a, B3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ B3 sub(B3 a, B3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ B3 mul(B3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ float dot(B3 a, B3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ B3 cross(B3 a, B3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ B3 normalize(B3 a) { return mul(a, 1.0f / sqrtf(dot(a, a))); }
__host__ __device__ __forceinline__ bool same_hemi(B3 a, B3 b) { return a.z * b.z > 0.0f; }
__host__ __device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }
__host__ __device__ __forceinline__ float lum709(const float c[3]) {
    return c[0] * 0.2126f + c[1] * 0.7152f + c[2] * 0.0722f;
}

// ---- Trowbridge-Reitz, isotropic -------------------------------------------------------------
__host__ __device__ __forceinline__ float tr_d(B3 wh, float a) {
    const float c2 = wh.z * wh.z, s2 = fmaxf(0.0f, 1.0f - c2);
    const float tan2 = s2 / c2, e = tan2 / (a * a);
    const float inv_d = kPiB * a * a * c2 * c2 * (1.0f + e) * (1.0f + e);
    if (!isfinite(tan2) || !isfinite(inv_d) || inv_d == 0.0f) return 0.0f;
    return 1.0f / inv_d;
}
__host__ __device__ __forceinline__ float tr_lambda(B3 w, float a) {
    const float c2 = w.z * w.z, s2 = fmaxf(0.0f, 1.0f - c2);
    const float at = fabsf(sqrtf(s2) / w.z);
    const float l = (-1.0f + sqrtf(1.0f + a * a * at * at)) * 0.5f;
    return isfinite(at) ? l : 0.0f;
}
__host__ __device__ __forceinline__ float tr_pdf(B3 wo, B3 wh, float a) {  // visible normals
    return tr_d(wh, a) * (1.0f / (1.0f + tr_lambda(wo, a))) * fabsf(dot(wo, wh)) / fabsf(wo.z);
}
// visible-normal sample (microfacet.rs:117-139)
__host__ __device__ __forceinline__ B3 tr_sample_wh(B3 w, float a, float u0, float u1) {
    B3 wh = normalize(b3(a * w.x, a * w.y, w.z));
    if (wh.z < 0.0f) wh = mul(wh, -1.0f);
    const B3 t1 = wh.z < 0.99999f ? normalize(cross(b3(0.0f, 0.0f, 1.0f), wh)) : b3(1.0f, 0.0f, 0.0f);
    const B3 t2 = normalize(cross(wh, t1));
    const float r = sqrtf(u0), phi = u1 * 2.0f * kPiB;
    float px = r * cosf(phi), py = r * sinf(phi);
    const float h = sqrtf(1.0f - px * px);
    py = h + (py - h) * ((1.0f + wh.z) * 0.5f);
    const float pz = sqrtf(fmaxf(1.0f - (px * px + py * py), 0.0f));
    const B3 nh = add(add(mul(t1, px), mul(t2, py)), mul(wh, pz));
    return normalize(b3(a * nh.x, a * nh.y, fmaxf(nh.z, 1e-6f)));
}
__host__ __device__ __forceinline__ B3 reflect(B3 w, B3 n) { return sub(mul(n, 2.0f * dot(w, n)), w); }
// geometry.rs:287-306
__host__ __device__ __forceinline__ bool refract(B3 w, B3 n, float eta, B3 *wt) {
    float ci = dot(w, n);
    const float e = ci >= 0.0f ? eta : 1.0f / eta;
    const B3 nn = ci >= 0.0f ? n : mul(n, -1.0f);
    ci = fabsf(ci);
    const float s2i = fmaxf(1.0f - ci * ci, 0.0f), s2t = s2i / (e * e);
    if (s2t >= 1.0f) return false;
    const float ct = sqrtf(1.0f - s2t);
    *wt = add(mul(w, -1.0f / e), mul(nn, ci / e - ct));
    return true;
}

// ---- Fresnel (mod.rs:2098-2190) -----------------------------------------------------------------
__host__ __device__ __forceinline__ float fr_dielectric(float ci, float eta) {
    ci = fminf(fmaxf(ci, -1.0f), 1.0f);
    const float e = ci > 0.0f ? eta : 1.0f / eta;
    ci = fabsf(ci);
    const float s2i = 1.0f - ci * ci, s2t = s2i / (e * e);
    if (s2t >= 1.0f) return 1.0f;
    const float ct = sqrtf(fmaxf(1.0f - s2t, 0.0f));
    const float rpa = (e * ci - ct) / (e * ci + ct), rpe = (ci - e * ct) / (ci + e * ct);
    return fminf(fmaxf((rpa * rpa + rpe * rpe) * 0.5f, 0.0f), 1.0f);
}
struct Cx {
    float re, im;
};
__host__ __device__ __forceinline__ Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ __forceinline__ Cx cdiv(Cx a, Cx b) {
    const float d = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__host__ __device__ __forceinline__ Cx csqrt(Cx z) {  // principal root
    const float n = sqrtf(z.re * z.re + z.im * z.im);
    if (n == 0.0f) return {0.0f, 0.0f};
    const float t1 = sqrtf(0.5f * (n + fabsf(z.re))), t2 = 0.5f * z.im / t1;
    if (z.re >= 0.0f) return {t1, t2};
    return {fabsf(t2), copysignf(t1, z.im)};
}
__host__ __device__ __forceinline__ float fr_complex(float ci, float n, float k) {
    ci = fminf(fmaxf(ci, 0.0f), 0.999f);
    const Cx eta = {n, k};
    const float s2 = 1.0f - ci * ci;
    const Cx s2t = cdiv(Cx{s2, 0.0f}, cmul(eta, eta));
    const Cx ct = csqrt(Cx{1.0f - s2t.re, -s2t.im});
    const Cx ec = {eta.re * ci, eta.im * ci};
    const Cx rpa = cdiv(Cx{ec.re - ct.re, ec.im - ct.im}, Cx{ec.re + ct.re, ec.im + ct.im});
    const Cx ect = cmul(eta, ct);
    const Cx rpe = cdiv(Cx{ci - ect.re, -ect.im}, Cx{ci + ect.re, ect.im});
    return (rpa.re * rpa.re + rpa.im * rpa.im + rpe.re * rpe.re + rpe.im * rpe.im) * 0.5f;
}
__host__ __device__ __forceinline__ float ior_from_f0(float f0) {
    const float s = sqrtf(fminf(fmaxf(f0, 0.0f), 0.99f));
    return (1.0f + s) / (1.0f - s);
}

// ---- the ggx_dielectric_s table ----------------------------------------------------------------
// A(roughness, mu, eta): trilinear read (PreComputedTable::read_3d, mod.rs:2318-2380) at
// (roughness, |mu| clamped to 0.999, sqrt(|eta - 1| / (eta + 1)))
__host__ __device__ __forceinline__ float tab_1d(const float *t, float x, int off) {
    x = fminf(fmaxf(x, 0.0f), 1.0f) * (float)(kTabN - 1);
    const int i = (int)floorf(x), j = min(i + 1, kTabN - 1);
    const float w = x - (float)i;
    return (1.0f - w) * t[off + i] + w * t[off + j];
}
__host__ __device__ __forceinline__ float tab_2d(const float *t, float x, float y, int off) {
    y = fminf(fmaxf(y, 0.0f), 1.0f) * (float)(kTabN - 1);
    const int i = (int)floorf(y), j = min(i + 1, kTabN - 1);
    const float w = y - (float)i;
    return (1.0f - w) * tab_1d(t, x, off + kTabN * i) + w * tab_1d(t, x, off + kTabN * j);
}
__host__ __device__ __forceinline__ float tab_3d(const float *t, float x, float y, float z) {
    z = fminf(fmaxf(z, 0.0f), 1.0f) * (float)(kTabN - 1);
    const int i = (int)floorf(z), j = min(i + 1, kTabN - 1);
    const float w = z - (float)i;
    return (1.0f - w) * tab_2d(t, x, y, kTabN * kTabN * i) + w * tab_2d(t, x, y, kTabN * kTabN * j);
}
__host__ __device__ __forceinline__ float ggx_albedo(const float *t, float rough, float mu, float eta) {
    const float z = sqrtf(fabsf((eta - 1.0f) / (eta + 1.0f)));
    mu = fabsf(fminf(fmaxf(mu, -0.999f), 0.999f));
    return tab_3d(t, rough, mu, z);
}
// the table's integrand: f/pdf of a unit-colour GGX reflection with dielectric Fresnel `ior`,
// sampled at wo = (sqrt(1 - mu^2), 0, mu) with the visible-normal sample (u0, u1); 0 when the
// sample is invalid (precompute_ggx_dielectric, precompute.rs:56-98)
__host__ __device__ __forceinline__ float ggx_albedo_sample(float rough, float mu, float ior, float u0, float u1) {
    const float a = fmaxf(rough * rough, 1e-4f);
    const B3 wo = b3(sqrtf(1.0f - mu * mu), 0.0f, mu);
    const B3 wh = tr_sample_wh(wo, a, u0, u1);
    const B3 wi = reflect(wo, wh);
    if (!same_hemi(wo, wi)) return 0.0f;
    B3 h = add(wo, wi);
    const float co = wo.z, ci = wi.z;
    if (dot(h, wo) * dot(wi, h) < 0.0f || (h.x == 0.0f && h.y == 0.0f && h.z == 0.0f) || ci == 0.0f || co == 0.0f)
        return 0.0f;
    h = normalize(h);
    const float F = fr_dielectric(dot(wi, h.z < 0.0f ? mul(h, -1.0f) : h), ior);
    const float D = tr_d(h, a), G = 1.0f / (1.0f + tr_lambda(wo, a) + tr_lambda(wi, a));
    const float f = F * fabsf(0.25f * D * G / (ci * co)) * fabsf(ci);
    const float pdf = tr_pdf(wo, h, a) / (4.0f * fabsf(dot(wo, h)));
    return pdf > 0.0f ? f / pdf : 0.0f;
}

// ---- the closure --------------------------------------------------------------------------------
struct PClosure {
    float base[3], tcol[3];
    float alpha, rough, rough_d;          // GGX alpha, the input roughness, sqrt(alpha)
    float metallic, transmission, ior;
    float spec_eta, spec_f0, spec_tint[3], spec_tint_lum;
    float cn[3], ck[3];                    // conductor n, k
    float coat_w, coat_alpha, coat_rough, coat_rough_d, coat_ior, coat_tint[3];
};
// kinds evaluated through PClosure
__host__ __device__ __forceinline__ bool closure_kind(int32_t kind) {
    return kind == STY_MAT_PRINCIPLED || kind == STY_MAT_GLASS;
}
// STY_MAT_PRINCIPLED: the principled layers. STY_MAT_GLASS (glass.rs:13-44) is the dielectric layer
// alone -- transmission 1, no specular, metal or coat layer -- with the transmitted lobe tinted by
// the colour itself rather than its square root.
template <class M>
__host__ __device__ __forceinline__ PClosure make_closure(const M &m) {
    PClosure c;
    for (int i = 0; i < 3; i++) {
        c.base[i] = m.albedo[i];
        c.tcol[i] = sqrtf(m.albedo[i]);
        c.spec_tint[i] = m.specular_tint[i];
        c.coat_tint[i] = m.coat_tint[i];
    }
    c.rough = m.roughness;
    c.alpha = fmaxf(m.roughness * m.roughness, 1e-4f);
    c.rough_d = sqrtf(c.alpha);
    c.metallic = m.metallic;
    c.transmission = m.transmission;
    c.ior = m.ior;
    float f0 = (m.ior - 1.0f) / (m.ior + 1.0f);
    f0 *= f0;
    float eta_s = m.ior;
    if (m.specular_ior_level != 0.5f) {
        f0 *= 2.0f * m.specular_ior_level;
        eta_s = ior_from_f0(f0);
    }
    c.spec_f0 = f0;
    c.spec_eta = eta_s;
    c.spec_tint_lum = lum709(m.specular_tint);
    // Gulbrandsen 2014 (artistic_to_conductor_fresnel, mod.rs:2128-2142)
    for (int i = 0; i < 3; i++) {
        const float r = fminf(fmaxf(m.albedo[i], 0.0f), 0.99f), g = m.specular_tint[i], rs = sqrtf(r);
        const float nmin = (1.0f - r) / (1.0f + r), nmax = (1.0f + rs) / (1.0f - rs);
        const float n = nmax + (nmin - nmax) * g;
        const float k2 = fmaxf(((n + 1.0f) * (n + 1.0f) * r - (n - 1.0f) * (n - 1.0f)) / (1.0f - r), 0.0f);
        c.cn[i] = n;
        c.ck[i] = sqrtf(k2);
    }
    c.coat_w = m.coat_weight;
    c.coat_rough = m.coat_roughness;
    c.coat_alpha = fmaxf(m.coat_roughness * m.coat_roughness, 1e-4f);
    c.coat_rough_d = sqrtf(c.coat_alpha);
    c.coat_ior = m.coat_ior;
    if (m.kind == STY_MAT_GLASS) {
        for (int i = 0; i < 3; i++) {
            c.tcol[i] = m.albedo[i];
            c.spec_tint[i] = 0.0f;
        }
        c.spec_tint_lum = 0.0f;
        c.transmission = 1.0f;
        c.metallic = 0.0f;
        c.coat_w = 0.0f;
    }
    return c;
}

// microfacet reflection (mod.rs:1877-1910); fresnel: 0 dielectric(eta), 1 conductor (n, k)
__host__ __device__ __forceinline__ float mf_reflect(B3 wo, B3 wi, float a, int fkind, float eta, const float *n,
                                                     const float *k, const float col[3], float f[3]) {
    f[0] = f[1] = f[2] = 0.0f;
    B3 wh = add(wo, wi);
    const float co = wo.z, ci = wi.z;
    if (dot(wh, wo) * dot(wi, wh) < 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) || ci == 0.0f ||
        co == 0.0f || !same_hemi(wo, wi))
        return 0.0f;
    wh = normalize(wh);
    const float cf = dot(wi, wh.z < 0.0f ? mul(wh, -1.0f) : wh);
    const float D = tr_d(wh, a), G = 1.0f / (1.0f + tr_lambda(wo, a) + tr_lambda(wi, a));
    const float s = fabsf(0.25f * D * G / (ci * co)) * fabsf(ci);
    for (int i = 0; i < 3; i++) {
        const float F = fkind == 0 ? fr_dielectric(cf, eta) : fr_complex(fabsf(cf), n[i], k[i]);
        f[i] = col[i] * F * s;
    }
    return tr_pdf(wo, wh, a) / (4.0f * fabsf(dot(wo, wh)));
}
// microfacet transmission (mod.rs:1979-2036), dielectric Fresnel
__host__ __device__ __forceinline__ float mf_transmit(B3 wo, B3 wi, float a, float eta, const float col[3],
                                                      float f[3]) {
    f[0] = f[1] = f[2] = 0.0f;
    const float co = wo.z, ci = wi.z;
    const float e = co > 0.0f ? eta : 1.0f / eta;
    B3 wh = normalize(add(wo, mul(wi, e)));
    if (wh.z < 0.0f) wh = mul(wh, -1.0f);
    const bool backfacing = dot(wh, wi) * ci < 0.0f || dot(wh, wo) * co < 0.0f;
    if (dot(wh, wo) * dot(wi, wh) > 0.0f || ci == 0.0f || co == 0.0f || backfacing || same_hemi(wo, wi)) return 0.0f;
    const float F = fr_dielectric(dot(wo, wh), eta);
    const float q = dot(wi, wh) + dot(wo, wh) / e;
    const float denom = q * q * ci * co;
    const float D = tr_d(wh, a), G = 1.0f / (1.0f + tr_lambda(wo, a) + tr_lambda(wi, a));
    if (denom != 0.0f) {
        const float s = fabsf(D * G / (e * e) * fabsf(dot(wi, wh)) * fabsf(dot(wo, wh)) / denom) * fabsf(ci);
        for (int i = 0; i < 3; i++) f[i] = (1.0f - F) * col[i] * s;
    }
    const float d2 = q * q;
    return d2 == 0.0f ? 0.0f : tr_pdf(wo, wh, a) * (fabsf(dot(wi, wh)) / d2);
}

__host__ __device__ __forceinline__ void lerp3(float a[3], const float b[3], float t) {
    for (int i = 0; i < 3; i++) a[i] = a[i] + (b[i] - a[i]) * t;
}
constexpr float kMixEps = 1e-4f;

// f * |cos_i| (rgb) and pdf of the closure for wo, wi in the shading frame (z = normal)
__host__ __device__ inline float eval(const PClosure &c, const float *tab, B3 wo, B3 wi, float f[3]) {
    const float mu = fabsf(wo.z);
    // L1 = mix(transmission, diffuse, dielectric)
    float f1[3] = {0.0f, 0.0f, 0.0f}, p1 = 0.0f;
    {
        float fa[3] = {0.0f, 0.0f, 0.0f}, fb[3] = {0.0f, 0.0f, 0.0f}, pa = 0.0f, pb = 0.0f;
        if (c.transmission < 1.0f - kMixEps && same_hemi(wo, wi)) {
            const float k = fabsf(wi.z) / kPiB;
            for (int i = 0; i < 3; i++) fa[i] = c.base[i] * k;
            pa = k;
        }
        if (c.transmission > kMixEps) {
            float ft[3], fr[3];
            const float pt = mf_transmit(wo, wi, c.alpha, c.ior, c.tcol, ft);
            const float pr = mf_reflect(wo, wi, c.alpha, 0, c.ior, nullptr, nullptr, c.base, fr);
            const float frd = fr_dielectric(wo.z, c.ior);
            for (int i = 0; i < 3; i++) fb[i] = ft[i] + fr[i];
            pb = lerpf(pt, pr, frd);
        }
        for (int i = 0; i < 3; i++) f1[i] = lerpf(fa[i], fb[i], c.transmission);
        p1 = lerpf(pa, pb, c.transmission);
    }
    // L2 = add(spec weight, scaled(L1), spec)
    float f2[3], p2;
    {
        const float A = ggx_albedo(tab, c.rough, mu, c.spec_eta);
        const float frac = c.spec_f0 * c.spec_tint_lum * A;
        const float col[3] = {c.spec_tint[0] * c.spec_f0, c.spec_tint[1] * c.spec_f0, c.spec_tint[2] * c.spec_f0};
        float fs[3];
        const float ps = mf_reflect(wo, wi, c.alpha, 0, c.spec_eta, nullptr, nullptr, col, fs);
        for (int i = 0; i < 3; i++) f2[i] = f1[i] * (1.0f - c.spec_tint[i] * c.spec_f0 * A) + fs[i];
        p2 = lerpf(p1, ps, frac);
    }
    // L3 = mix(metallic, L2, metal)
    float f3[3] = {0.0f, 0.0f, 0.0f}, p3;
    {
        float fa[3] = {0.0f, 0.0f, 0.0f}, fm[3] = {0.0f, 0.0f, 0.0f}, pa = 0.0f, pm = 0.0f;
        if (c.metallic < 1.0f - kMixEps) {
            for (int i = 0; i < 3; i++) fa[i] = f2[i];
            pa = p2;
        }
        if (c.metallic > kMixEps) {
            const float one[3] = {1.0f, 1.0f, 1.0f};
            pm = mf_reflect(wo, wi, c.alpha, 1, 0.0f, c.cn, c.ck, one, fm);
        }
        for (int i = 0; i < 3; i++) f3[i] = lerpf(fa[i], fm[i], c.metallic);
        p3 = lerpf(pa, pm, c.metallic);
    }
    // L5 = add(coat weight, scaled(L4 = L3), coat)
    {
        const float A = ggx_albedo(tab, c.coat_rough, mu, c.coat_ior);
        const float frac = c.coat_w * A;
        const float col[3] = {c.coat_w, c.coat_w, c.coat_w};
        float fc[3];
        const float pc = mf_reflect(wo, wi, c.coat_alpha, 0, c.coat_ior, nullptr, nullptr, col, fc);
        for (int i = 0; i < 3; i++) f[i] = f3[i] * lerpf(1.0f, c.coat_tint[i] * (1.0f - A), c.coat_w) + fc[i];
        return lerpf(p3, pc, frac);
    }
}

// b when u < frac (remapped u / frac), else a (remapped (u - frac) / (1 - frac))
__host__ __device__ __forceinline__ bool choose_b(float frac, float &u) {
    if (u < frac) {
        u = u / frac;
        return true;
    }
    u = (u - frac) / (1.0f - frac);
    return false;
}
// sample_wi of the closure: the sampled direction and its validity (the caller evaluates)
__host__ __device__ inline bool sample(const PClosure &c, const float *tab, B3 wo, float u, float u0, float u1,
                                       B3 *wi) {
    const float mu = fabsf(wo.z);
    if (choose_b(c.coat_w * ggx_albedo(tab, c.coat_rough, mu, c.coat_ior), u)) {  // coat
        *wi = reflect(wo, tr_sample_wh(wo, c.coat_alpha, u0, u1));
        return same_hemi(wo, *wi);
    }
    if (choose_b(c.metallic, u) ||  // metal
        choose_b(c.spec_f0 * c.spec_tint_lum * ggx_albedo(tab, c.rough, mu, c.spec_eta), u)) {  // specular
        *wi = reflect(wo, tr_sample_wh(wo, c.alpha, u0, u1));
        return same_hemi(wo, *wi);
    }
    if (choose_b(c.transmission, u)) {  // dielectric
        const B3 wh = tr_sample_wh(wo, c.alpha, u0, u1);
        if (choose_b(fr_dielectric(wo.z, c.ior), u)) {
            *wi = reflect(wo, wh);
            return same_hemi(wo, *wi);
        }
        if (!refract(wo, wh, c.ior, wi)) return false;
        return !same_hemi(wo, *wi);
    }
    // diffuse: cosine hemisphere (polar disk), on wo's side
    const float r = sqrtf(u0), phi = u1 * 2.0f * kPiB;
    const float x = r * cosf(phi), y = r * sinf(phi);
    B3 w = b3(x, y, sqrtf(fmaxf(1.0f - x * x - y * y, 0.0f)));
    if (!same_hemi(wo, w)) w = mul(w, -1.0f);
    *wi = w;
    return true;
}
// avg_roughness (BsdfMixture: lerp of the lobes' by frac; diffuse 1, microfacet sqrt(alpha))
__host__ __device__ inline float avg_roughness(const PClosure &c, const float *tab, B3 wo) {
    const float mu = fabsf(wo.z);
    const float r1 = lerpf(1.0f, c.rough_d, c.transmission);
    const float r2 = lerpf(r1, c.rough_d, c.spec_f0 * c.spec_tint_lum * ggx_albedo(tab, c.rough, mu, c.spec_eta));
    const float r3 = lerpf(r2, c.rough_d, c.metallic);
    return lerpf(r3, c.coat_rough_d, c.coat_w * ggx_albedo(tab, c.coat_rough, mu, c.coat_ior));
}

// ---- world space (SurfaceClosure, mod.rs:1693-1869) -----------------------------------------------
struct BFrame {
    B3 t, s, n;
};
__host__ __device__ __forceinline__ BFrame frame_n(B3 n) {  // Frame::from_n (geometry.rs:163-171)
    B3 t;
    if (fabsf(n.x) > fabsf(n.y)) t = mul(b3(-n.z, 0.0f, n.x), 1.0f / sqrtf(n.x * n.x + n.z * n.z));
    else t = mul(b3(0.0f, n.z, -n.y), 1.0f / sqrtf(n.y * n.y + n.z * n.z));
    return {t, cross(n, t), n};
}
__host__ __device__ __forceinline__ B3 to_local(const BFrame &f, B3 v) { return b3(dot(f.t, v), dot(f.s, v), dot(f.n, v)); }
__host__ __device__ __forceinline__ B3 to_world(const BFrame &f, B3 v) {
    return add(add(mul(f.t, v.x), mul(f.s, v.y)), mul(f.n, v.z));
}
__host__ __device__ __forceinline__ bool closure_valid(B3 ns, B3 ng, B3 wo, B3 wi) {  // check_wo_wi_valid
    auto sgn = [](float x) { return x > 0.0f ? 1.0f : -1.0f; };
    const float fl = sgn(dot(ng, ns));
    return sgn(fl * dot(wo, ns)) * sgn(dot(wo, ng)) > 0.0f && sgn(fl * dot(wi, ns)) * sgn(dot(wi, ng)) > 0.0f;
}
__host__ __device__ inline float eval_world(const PClosure &c, const float *tab, B3 ns, B3 ng, B3 wo, B3 wi, float f[3]) {
    f[0] = f[1] = f[2] = 0.0f;
    if (!closure_valid(ns, ng, wo, wi)) return 0.0f;
    const BFrame fr = frame_n(ns);
    return eval(c, tab, to_local(fr, wo), to_local(fr, wi), f);
}
// SurfaceClosure::sample: the direction, f * |cos| and pdf at it (false / pdf 0 when invalid)
__host__ __device__ inline bool sample_world(const PClosure &c, const float *tab, B3 ns, B3 ng, B3 wo, float u, float u0,
                                             float u1, B3 *wi, float f[3], float *pdf) {
    f[0] = f[1] = f[2] = 0.0f;
    *pdf = 0.0f;
    const BFrame fr = frame_n(ns);
    B3 wl;
    if (!sample(c, tab, to_local(fr, wo), u, u0, u1, &wl)) return false;
    *wi = to_world(fr, wl);
    if (!closure_valid(ns, ng, wo, *wi)) return false;
    *pdf = eval_world(c, tab, ns, ng, wo, *wi, f);
    return *pdf > 0.0f;
}
__host__ __device__ inline float avg_roughness_world(const PClosure &c, const float *tab, B3 ns, B3 wo) {
    return avg_roughness(c, tab, to_local(frame_n(ns), wo));
}

}  // namespace bsdf

// The ggx_dielectric_s table of the current device (computed once per device; 16^3 floats,
// x = roughness fastest, then mu, then z = (ior - 1) / (ior + 1) parameter).
const float *principled_table();

}  // namespace sty
