// tracer.cuh -- device building blocks of the wavefront tracers (trace.cu: NL-PF / NL-NRC paths;
// brpt.cu: the branching path tracer): vector helpers, PCG32 sampling, the camera ray, emitter
// radiance with its MIS weight, stylization flags, BSDF sampling / evaluation, NEE, and the per-path
// state planes of the NL-PF wavefront.
#pragma once

#include <cmath>

#include "bsdf.cuh"
#include "common.cuh"
#include "rng.cuh"
#include "scene.cuh"
#include "style.cuh"

namespace sty {
namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr float kPi = 3.14159265358979323846f;

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3m(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ F3 normalize(F3 a) { return a * (1.0f / sqrtf(dot(a, a))); }

__device__ __forceinline__ uint32_t pcg_next(sty_pcg32 &s) {
    const uint64_t old = s.state;
    s.state = old * 0x5851f42d4c957f2dULL + s.inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}
// IndependentSampler::next_1d (sampler/mod.rs:208-212): u32 * (1 / u32::MAX as f32)
__device__ __forceinline__ float next_1d(sty_pcg32 &s) { return (float)pcg_next(s) * 2.3283064e-10f; }

// Wachter & Binder, "A Fast and Robust Method for Avoiding Self-Intersection" (Ray Tracing Gems,
// ch. 6): offset along the normal in integer ulps, absolute offset near the origin.
__device__ __forceinline__ F3 offset_ray_origin(F3 p, F3 n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    const float pv[3] = {p.x, p.y, p.z}, nv[3] = {n.x, n.y, n.z};
    float o[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int of = (int)(int_scale * nv[a]);
        const float pi = __int_as_float(__float_as_int(pv[a]) + (pv[a] < 0.0f ? -of : of));
        o[a] = fabsf(pv[a]) < origin ? pv[a] + float_scale * nv[a] : pi;
    }
    return {o[0], o[1], o[2]};
}
__device__ __forceinline__ F3 face_forward(F3 n, F3 v) { return dot(n, v) < 0.0f ? -n : n; }

// Frame::from_n (geometry.rs:163-171)
struct Frame {
    F3 t, s, n;
};
__device__ __forceinline__ Frame frame_from_n(F3 n) {
    F3 t;
    if (fabsf(n.x) > fabsf(n.y))
        t = f3m(-n.z, 0.0f, n.x) * (1.0f / sqrtf(n.x * n.x + n.z * n.z));
    else
        t = f3m(0.0f, n.z, -n.y) * (1.0f / sqrtf(n.y * n.y + n.z * n.z));
    return {t, cross(n, t), n};
}
__device__ __forceinline__ F3 to_local(const Frame &f, F3 v) { return {dot(f.t, v), dot(f.s, v), dot(f.n, v)}; }
__device__ __forceinline__ F3 to_world(const Frame &f, F3 v) { return f.t * v.x + f.s * v.y + f.n * v.z; }

__device__ __forceinline__ float2 uniform_sample_disk(float u0, float u1) {  // sampling.rs:5-9
    const float r = sqrtf(u0), phi = u1 * 2.0f * kPi;
    return make_float2(r * cosf(phi), r * sinf(phi));
}
__device__ __forceinline__ float2 uniform_sample_triangle(float u0, float u1) {  // sampling.rs:32-44
    if (u0 < u1) {
        const float b0 = u0 / 2.0f;
        return make_float2(b0, u1 - b0);
    }
    const float b1 = u1 / 2.0f;
    return make_float2(u0 - b1, b1);
}

__device__ __forceinline__ uint32_t style_index(uint32_t f) {
    uint32_t i = 0;
    if (f & 2u) i = 1;
    if (f & 4u) i = 2;
    if (f & 8u) i = 3;
    return i;
}

// ---- BSDF (same forms as pf_ref.cu's evaluation; sampling restated here) --------------------
__device__ __forceinline__ bool wo_wi_valid(F3 ns, F3 ng, F3 wo, F3 wi) {
    auto sgn = [](float x) { return x > 0.0f ? 1.0f : -1.0f; };
    const float fl = sgn(dot(ng, ns));
    return sgn(fl * dot(wo, ns)) * sgn(dot(wo, ng)) > 0.0f && sgn(fl * dot(wi, ns)) * sgn(dot(wi, ng)) > 0.0f;
}
__device__ __forceinline__ float tr_d(float ch, float a) {
    const float c2 = ch * ch, s2 = fmaxf(0.0f, 1.0f - c2);
    const float tan2 = s2 / c2, e = tan2 / (a * a);
    const float inv_d = kPi * a * a * c2 * c2 * (1.0f + e) * (1.0f + e);
    if (!isfinite(tan2) || !isfinite(inv_d) || inv_d == 0.0f) return 0.0f;
    return 1.0f / inv_d;
}
__device__ __forceinline__ float tr_lambda(float cw, float a) {
    const float c2 = cw * cw, s2 = fmaxf(0.0f, 1.0f - c2);
    const float at = fabsf(sqrtf(s2) / cw);
    const float l = (-1.0f + sqrtf(1.0f + a * a * at * at)) * 0.5f;
    return isfinite(at) ? l : 0.0f;
}
__device__ __forceinline__ bsdf::B3 tob(F3 v) { return bsdf::b3(v.x, v.y, v.z); }
// STY_MAT_PRINCIPLED / STY_MAT_GLASS through the shared closure (bsdf.cuh); tab = the scene's
// albedo table
__device__ __forceinline__ float princ_eval(const sty_scene_material &m, const float *tab, F3 ns, F3 ng, F3 wo, F3 wi,
                                            F3 *f) {
    float fv[3];
    const float p = bsdf::eval_world(bsdf::make_closure(m), tab, tob(ns), tob(ng), tob(wo), tob(wi), fv);
    *f = f3m(fv[0], fv[1], fv[2]);
    return p;
}
// PRINC = false: a kernel variant for scenes without closure materials (SceneView::any_closure),
// which then carries none of the closure's code, registers or stack.
template <bool PRINC = true>
__device__ __forceinline__ float bsdf_pdf(const sty_scene_material &m, F3 ns, F3 ng, F3 wo, F3 wi, const float *tab) {
    if constexpr (PRINC) {
        if (bsdf::closure_kind(m.kind)) {
            F3 f;
            return princ_eval(m, tab, ns, ng, wo, wi, &f);
        }
    }
    if (!wo_wi_valid(ns, ng, wo, wi)) return 0.0f;
    const float co = dot(wo, ns), ci = dot(wi, ns);
    if (m.kind == STY_MAT_DIFFUSE) return co * ci >= 0.0f ? fabsf(ci) / kPi : 0.0f;
    const float a = fmaxf(m.alpha, 1e-4f);
    F3 wh = wo + wi;
    if (dot(wh, wo) * dot(wi, wh) < 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) || ci == 0.0f ||
        co == 0.0f || !(co * ci >= 0.0f))
        return 0.0f;
    wh = normalize(wh);
    const float d = tr_d(dot(wh, ns), a), g1 = 1.0f / (1.0f + tr_lambda(co, a));
    const float owh = fabsf(dot(wo, wh));
    return d * g1 * owh / fabsf(co) / (4.0f * owh);
}
// Surface::sample: wi (world) and its pdf (0 = invalid)
template <bool PRINC = true>
__device__ __forceinline__ F3 bsdf_sample(const sty_scene_material &m, F3 ns, F3 ng, F3 wo, float u_sel, float u0, float u1,
                          float *pdf, const float *tab) {
    if constexpr (PRINC) {
        if (bsdf::closure_kind(m.kind)) {
            bsdf::B3 w = bsdf::b3(0.0f, 0.0f, 0.0f);
            float fv[3];
            bsdf::sample_world(bsdf::make_closure(m), tab, tob(ns), tob(ng), tob(wo), u_sel, u0, u1, &w, fv, pdf);
            return f3m(w.x, w.y, w.z);
        }
    }
    const Frame fr = frame_from_n(ns);
    const F3 wol = to_local(fr, wo);
    F3 wil;
    bool valid = true;
    if (m.kind == STY_MAT_DIFFUSE) {  // cos_sample_hemisphere, flipped into wo's hemisphere
        const float2 d = uniform_sample_disk(u0, u1);
        const float z = sqrtf(fmaxf(1.0f - d.x * d.x - d.y * d.y, 0.0f));
        wil = f3m(d.x, d.y, z);
        if (!(wol.z * wil.z >= 0.0f)) wil = -wil;
    } else {  // visible-normal sampling (microfacet.rs:117-152) + reflect
        const float a = fmaxf(m.alpha, 1e-4f);
        F3 wh = normalize(f3m(a * wol.x, a * wol.y, wol.z));
        if (wh.z < 0.0f) wh = -wh;
        const F3 t1 = wh.z < 0.99999f ? normalize(cross(f3m(0.0f, 0.0f, 1.0f), wh)) : f3m(1.0f, 0.0f, 0.0f);
        const F3 t2 = normalize(cross(wh, t1));
        float2 p = uniform_sample_disk(u0, u1);
        const float h = sqrtf(1.0f - p.x * p.x);
        p.y = h + (p.y - h) * ((1.0f + wh.z) * 0.5f);
        const float pz = sqrtf(fmaxf(1.0f - (p.x * p.x + p.y * p.y), 0.0f));
        const F3 nh = t1 * p.x + t2 * p.y + wh * pz;
        wh = normalize(f3m(a * nh.x, a * nh.y, fmaxf(nh.z, 1e-6f)));
        wil = wh * (2.0f * dot(wol, wh)) - wol;
        valid = wol.z * wil.z >= 0.0f;
    }
    const F3 wi = to_world(fr, wil);
    valid = valid && wo_wi_valid(ns, ng, wo, wi);
    *pdf = valid ? bsdf_pdf(m, ns, ng, wo, wi, tab) : 0.0f;
    return wi;
}

// ---- per-path state (SoA) and per-depth vertex planes ---------------------------------------
struct PathState {
    float *o[3], *d[3];
    float *prev_p[3];
    float *prev_pdf;
    uint32_t *flags, *exclude, *terminated;
    uint32_t *split;  // depth of the vertex a final-gathering render stopped at, NONE otherwise
};
struct VertOut {  // mutable view of one depth's sty_pf_vertices planes
    int32_t *active;
    float *p[3], *wo[3], *ns[3], *ng[3], *le[3], *mis, *dir_wi[3], *dir_l[3], *dir_pdf, *ind_wi[3], *ind_mis;
    uint32_t *flags, *material;
};
struct CamArgs {
    float eye[3], fwd[3], right[3], up[3];
    float tan_half, aspect, radius;
    uint32_t W, H;
    uint32_t random_px;  // 1: path tid starts at pixel pcg32() % (W*H) (training paths, nrc_pt.rs:1394)
    uint32_t filter;     // STY_FILTER_BOX / STY_FILTER_GAUSSIAN (PixelFilter, film.rs:20-48)
    uint32_t pixel_major;  // k > 0: path slot tid is sample tid % k of pixel tid / k (screen-record order)
};

// One light sample for a vertex at p (sample_light, lm_path_filtering.rs:1261-1316): emitter chosen
// by the area x luminance CDF, uniform point on it, Li styled at depth + 1 by the emitter's program
// (flags = the vertex's updated flags), shadow ray. Returns false when the sample carries nothing.
__device__ bool nee_sample(const SceneView &sc, F3 p, F3 ng, uint32_t prim, uint32_t new_flags, uint32_t depth,
                           const sty_style_program *progs, uint32_t n_progs, sty_pcg32 &st, F3 *wi_out, f3 *li_out,
                           float *pdf_out) {
    const float ux = next_1d(st), uy = next_1d(st), uz = next_1d(st);
    if (sc.n_lights == 0) return false;
    uint32_t lo = 0, hi = sc.n_lights - 1;
    while (lo < hi) {  // first k with cdf[k+1] > ux
        const uint32_t mid = (lo + hi) >> 1;
        if (sc.light_cdf[mid + 1] > ux) hi = mid;
        else lo = mid + 1;
    }
    const uint32_t lt = sc.light_tris[lo];
    const float sel = sc.light_cdf[lo + 1] - sc.light_cdf[lo];
    const float2 bb = uniform_sample_triangle(uy, uz);
    const float *lp = sc.tri_pos + 9 * (size_t)lt;
    const float c0 = 1.0f - bb.x - bb.y;
    const F3 q = f3m(c0 * lp[0] + bb.x * lp[3] + bb.y * lp[6], c0 * lp[1] + bb.x * lp[4] + bb.y * lp[7],
                     c0 * lp[2] + bb.x * lp[5] + bb.y * lp[8]);
    const F3 ln = f3m(sc.tri_normal[3 * lt], sc.tri_normal[3 * lt + 1], sc.tri_normal[3 * lt + 2]);
    F3 wi = q - p;
    const float dist2 = dot(wi, wi);
    if (!(dist2 > 0.0f)) return false;
    const float dist = sqrtf(dist2);
    wi = wi * (1.0f / dist);
    const sty_scene_material lm = sc.materials[sc.tri_material[lt]];
    f3 li = {0.0f, 0.0f, 0.0f};
    if (dot(wi, ln) < 0.0f) li = {lm.emission[0], lm.emission[1], lm.emission[2]};
    const float lpdf = sel / sc.tri_area[lt] * dist2 / fabsf(dot(ln, wi));
    if (!(isfinite(lpdf) && lpdf > 0.0f)) return false;
    if (!(new_flags & 1u)) {  // the light's style node at the next depth (sample_light :1286-1305)
        const int32_t pi = lm.style[style_index(new_flags)];
        if (pi >= 0 && (uint32_t)pi < n_progs) li = style_apply(progs[pi], depth + 1, li, f3{q.x, q.y, q.z});
    }
    const F3 so = offset_ray_origin(p, face_forward(ng, wi));
    const float s3[3] = {so.x, so.y, so.z}, w3[3] = {wi.x, wi.y, wi.z};
    if (trace_any(sc, s3, w3, 0.0f, dist * (1.0f - 1e-3f), prim, lt)) return false;
    *wi_out = wi;
    *li_out = li;
    *pdf_out = lpdf;
    return true;
}
// Surface::avg_roughness: diffuse 1, the GGX lobe its alpha (as the NL-PF paths have used it), the
// principled closure the frac-weighted mean of its lobes' (which depends on wo)
template <bool PRINC = true>
__device__ __forceinline__ float lobe_roughness(const sty_scene_material &m, const float *tab, F3 ns, F3 wo) {
    if constexpr (PRINC) {
        if (bsdf::closure_kind(m.kind))
            return bsdf::avg_roughness_world(bsdf::make_closure(m), tab, tob(ns), tob(wo));
    }
    return m.kind == STY_MAT_DIFFUSE ? 1.0f : m.alpha;
}

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
// init_pcg32_buffer_with_seed (sampler/mod.rs:157-173): path slot i gets
// Pcg32::new_seq_offset(i, seed_i), seed_i the i-th gen::<u64>() of StdRng::seed_from_u64(seed);
// `key` is that generator's ChaCha12 key (std_rng_key)
struct StdRngKey {
    uint32_t k[8];
};
inline StdRngKey std_rng_key_of(uint64_t seed) {
    StdRngKey r;
    std_rng_key(seed, r.k);
    return r;
}
// With pixel_major = k > 0 the slots are stored pixel-major (slot = px * k + b) but each keeps the
// stream of the reference's slot b * npx + px, so a pixel sample draws the same numbers in either
// order.
__global__ void k_rng_init(uint32_t n, StdRngKey key, uint32_t pixel_major, uint32_t npx, sty_pcg32 *rng) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t seq = pixel_major ? (i % pixel_major) * npx + i / pixel_major : i;
    sty_pcg32 g;
    g.state = 0;
    g.inc = ((uint64_t)seq << 1) | 1ull;
    pcg_next(g);
    g.state += std_rng_u64(key.k, seq);
    pcg_next(g);
    rng[i] = g;
}

// f * |cos| (rgb) and pdf of a scene material (Surface::evaluate; diffuse.rs:17-48,
// svm/surface/mod.rs:1877-1910 with unit Fresnel)
template <bool PRINC = true>
__device__ __forceinline__ float bsdf_eval(const sty_scene_material &m, F3 ns, F3 ng, F3 wo, F3 wi, F3 *f, const float *tab) {
    if constexpr (PRINC) {
        if (bsdf::closure_kind(m.kind)) return princ_eval(m, tab, ns, ng, wo, wi, f);
    }
    *f = f3m(0.0f, 0.0f, 0.0f);
    if (!wo_wi_valid(ns, ng, wo, wi)) return 0.0f;
    const float co = dot(wo, ns), ci = dot(wi, ns);
    if (m.kind == STY_MAT_DIFFUSE) {
        if (!(co * ci >= 0.0f)) return 0.0f;
        const float k = fabsf(ci) / kPi;
        *f = f3m(m.albedo[0] * k, m.albedo[1] * k, m.albedo[2] * k);
        return k;
    }
    const float a = fmaxf(m.alpha, 1e-4f);
    F3 wh = wo + wi;
    if (dot(wh, wo) * dot(wi, wh) < 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) || ci == 0.0f ||
        co == 0.0f || !(co * ci >= 0.0f))
        return 0.0f;
    wh = normalize(wh);
    const float d = tr_d(dot(wh, ns), a);
    const float g = 1.0f / (1.0f + tr_lambda(co, a) + tr_lambda(ci, a)), g1 = 1.0f / (1.0f + tr_lambda(co, a));
    const float k = fabsf(0.25f * d * g / (ci * co)) * fabsf(ci);
    *f = f3m(m.albedo[0] * k, m.albedo[1] * k, m.albedo[2] * k);
    const float owh = fabsf(dot(wo, wh));
    return d * g1 * owh / fabsf(co) / (4.0f * owh);
}

// PixelFilter::sample (film.rs:30-48) of the sampler draw (u0, u1): box (u - 0.5) r; Gaussian
// Box-Muller offset sigma (r cos 2 pi u1, r sin 2 pi u1), r = sqrt(-2 ln u0), sigma = radius / 3,
// clamped to [-radius, radius] (u0 = 0 gives an infinite r; min(max(., -radius), radius) maps the
// resulting infinities and NaNs to -radius or radius)
__device__ __forceinline__ float2 pixel_filter_offset(const CamArgs &cam, float u0, float u1) {
    if (cam.filter != STY_FILTER_GAUSSIAN)
        return make_float2(__fmul_rn(__fsub_rn(u0, 0.5f), cam.radius), __fmul_rn(__fsub_rn(u1, 0.5f), cam.radius));
    const float sigma = __fdiv_rn(cam.radius, 3.0f);
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, ex_ln(u0)));
    float sn, cs;
    ex_sincos_turns(u1, &sn, &cs);
    const float ox = __fmul_rn(__fmul_rn(r, cs), sigma), oy = __fmul_rn(__fmul_rn(r, sn), sigma);
    return make_float2(fminf(fmaxf(ox, -cam.radius), cam.radius), fminf(fmaxf(oy, -cam.radius), cam.radius));
}
// Camera ray of pixel px (PerspectiveCamera::generate_ray, camera/mod.rs:73-126): 2 sampler draws
// for the pixel filter; film point (px + 0.5 + offset) mapped to the pinhole's direction; every
// operation explicitly rounded (a CPU restatement reproduces it bit for bit)
__device__ __forceinline__ void camera_ray(const CamArgs &cam, uint32_t px, sty_pcg32 &st, F3 *ro, F3 *rd) {
    const float fx = (float)(px % cam.W) + 0.5f, fy = (float)(px / cam.W) + 0.5f;
    const float u0 = next_1d(st), u1 = next_1d(st);
    const float2 o = pixel_filter_offset(cam, u0, u1);
    const float ndx = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn(fx, o.x)), (float)cam.W), 1.0f);
    const float ndy = __fsub_rn(1.0f, __fdiv_rn(__fmul_rn(2.0f, __fadd_rn(fy, o.y)), (float)cam.H));
    const float sx = __fmul_rn(__fmul_rn(ndx, cam.tan_half), cam.aspect), sy = __fmul_rn(ndy, cam.tan_half);
    const float dx = __fmaf_rn(cam.up[0], sy, __fmaf_rn(cam.right[0], sx, cam.fwd[0]));
    const float dy = __fmaf_rn(cam.up[1], sy, __fmaf_rn(cam.right[1], sx, cam.fwd[1]));
    const float dz = __fmaf_rn(cam.up[2], sy, __fmaf_rn(cam.right[2], sx, cam.fwd[2]));
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)))));
    *ro = f3m(cam.eye[0], cam.eye[1], cam.eye[2]);
    *rd = f3m(__fmul_rn(dx, inv), __fmul_rn(dy, inv), __fmul_rn(dz, inv));
}
// Emitter radiance at a hit and its balance-heuristic weight against the light pdf seen from the
// previous vertex (handle_surface_light, lm_path_filtering.rs:388-426 / branching_pt.rs:199-238;
// pdf_direct, light/area.rs:108-130); weight 1 at depth 0 or when the hit is not an emitter.
__device__ __forceinline__ bool emitter_le(const SceneView &sc, const sty_scene_material &m, uint32_t prim, F3 p,
                                           F3 ng, F3 rd, uint32_t depth, F3 prev_p, float prev_pdf, F3 *le,
                                           float *mis) {
    *le = f3m(0.0f, 0.0f, 0.0f);
    *mis = 1.0f;
    const bool emitter = m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f;
    if (!emitter) return false;
    if (dot(ng, rd) < 0.0f) *le = f3m(m.emission[0], m.emission[1], m.emission[2]);
    if (depth > 0) {
        float sel = 0.0f;
        for (uint32_t k = 0; k < sc.n_lights; k++)
            if (sc.light_tris[k] == prim) sel = sc.light_cdf[k + 1] - sc.light_cdf[k];
        const F3 w = p - prev_p;
        const float dist2 = dot(w, w);
        const F3 wn = w * (1.0f / sqrtf(dist2));
        const float lpdf = sel / sc.tri_area[prim] * dist2 / fmaxf(fabsf(dot(ng, wn)), 1e-6f);
        *mis = prev_pdf / (prev_pdf + lpdf);
    }
    return true;
}
// stylization flags after a hit (update_stylization_flags via sty_set_idx): bit 0 = disabled,
// bits 1-3 = style index 1-3
__device__ __forceinline__ uint32_t update_flags(const sty_scene_material &m, uint32_t flags) {
    uint32_t f = flags;
    if (m.set_style >= 0) {
        f &= 1u;
        if (m.set_style == 1) f |= 2u;
        if (m.set_style == 2) f |= 4u;
        if (m.set_style == 3) f |= 8u;
    }
    return f;
}

// The camera frame in double, rounded once to float (no host FMA contraction or libm difference
// between machines can change a bit of it).
inline CamArgs make_camera(const sty_camera &cam) {
    CamArgs ca;
    double f[3], r[3], u[3];
    for (int a = 0; a < 3; a++) f[a] = (double)cam.target[a] - (double)cam.eye[a];
    double l = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (int a = 0; a < 3; a++) f[a] /= l;
    r[0] = f[1] * cam.up[2] - f[2] * cam.up[1];
    r[1] = f[2] * cam.up[0] - f[0] * cam.up[2];
    r[2] = f[0] * cam.up[1] - f[1] * cam.up[0];
    l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int a = 0; a < 3; a++) r[a] /= l;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    for (int a = 0; a < 3; a++) {
        ca.eye[a] = cam.eye[a];
        ca.fwd[a] = (float)f[a];
        ca.right[a] = (float)r[a];
        ca.up[a] = (float)u[a];
    }
    ca.tan_half = (float)std::tan((double)cam.fov_y * 0.5 * 3.14159265358979323846 / 180.0);
    ca.aspect = (float)((double)cam.width / (double)cam.height);
    ca.radius = cam.filter_radius;
    ca.W = cam.width;
    ca.H = cam.height;
    ca.random_px = 0;
    ca.filter = (uint32_t)cam.filter;
    ca.pixel_major = 0;
    return ca;
}

}  // namespace
}  // namespace sty
