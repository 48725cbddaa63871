// trace.cu -- wavefront tracer and the end-to-end NL-PF render.
//
// k_trace restates one bounce of kernel_mk_trace (crates/akari_integrator/src/lm_path_filtering.rs:
// 1063-1218) for every path slot: camera ray at depth 0 (camera/mod.rs:73-126, box pixel filter
// film.rs:31-33), closest hit, emitter radiance with balance MIS against the light pdf
// (handle_surface_light :388-426, mis_weight :305-316), stylization-flag update, NEE with the
// light's style node applied at the next depth (sample_light :1261-1316, light/area.rs:51-132),
// BSDF sampling (diffuse.rs:40-53, microfacet.rs:117-152) and the continuation ray
// (offset_ray_origin, face_forward). Sampler draws follow the reference order: 2 for the camera,
// then per bounce 3 for the light and 1 + 2 for the BSDF. Each depth's vertices are written as SoA
// planes (sty_pf_vertices) that stay on the device; the record the reference's kernel_propagate
// copies into the parent (wi = -wo, mis) is written into the parent depth's slot when the child
// vertex is found.
#include <cub/cub.cuh>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "scene.cuh"
#include "style.cuh"
#include "tracer.cuh"

namespace sty {
const sty_camera &scene_camera(const sty_scene *s);
void scene_bounds(const sty_scene *s, float mn[3], float mx[3]);
const std::vector<sty_scene_material> &scene_materials(const sty_scene *s);
void *&scene_render_cache(sty_scene *s);
uint32_t nrc_batch_size(const sty_nrc *nr);
uint32_t nrc_input_dims(const sty_nrc *nr);
}  // namespace sty

namespace sty {
namespace {


// Screen-space record planes of one depth that the tracer writes in STY_PF_MODE_SCREEN (the
// position, normal and valid planes are the vertex planes themselves); rad[0] == nullptr: none.
struct RecOut {
    float *rad[3], *thr[3];
    uint32_t *prim;
};

__global__ void k_trace(SceneView sc, CamArgs cam, uint32_t n_paths, uint32_t depth, uint32_t max_depth,
                        PathState ps, VertOut v, VertOut parent, sty_pcg32 *rng, const sty_style_program *progs,
                        uint32_t n_progs, unsigned long long *vcount, float split_rough, RecOut rec,
                        RecOut rec_parent) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n_paths) return;
    sty_pcg32 st = rng[tid];
    F3 ro, rd;
    uint32_t flags, exclude;
    float prev_pdf;
    F3 prev_p;
    const bool recs = rec.rad[0] != nullptr;
    if (depth == 0) {
        const uint32_t npx = cam.W * cam.H;
        const uint32_t px = cam.random_px ? pcg_next(st) % npx : cam.pixel_major ? tid / cam.pixel_major : tid % npx;
        camera_ray(cam, px, st, &ro, &rd);
        flags = 0;
        exclude = NONE;
        prev_pdf = 0.0f;
        prev_p = ro;
        ps.terminated[tid] = 0;
        ps.split[tid] = NONE;
    } else {
        if (ps.terminated[tid]) return;
        ro = f3m(ps.o[0][tid], ps.o[1][tid], ps.o[2][tid]);
        rd = f3m(ps.d[0][tid], ps.d[1][tid], ps.d[2][tid]);
        flags = ps.flags[tid];
        exclude = ps.exclude[tid];
        prev_pdf = ps.prev_pdf[tid];
        prev_p = f3m(ps.prev_p[0][tid], ps.prev_p[1][tid], ps.prev_p[2][tid]);
    }
    const float o3[3] = {ro.x, ro.y, ro.z}, d3[3] = {rd.x, rd.y, rd.z};
    const Hit h = trace_closest(sc, o3, d3, 0.0f, 1e20f, exclude);
    if (h.prim == NONE) {
        ps.terminated[tid] = 1;
        rng[tid] = st;
        return;
    }
    atomicAdd(vcount, 1ull);
    const uint32_t prim = h.prim;
    const float *tp = sc.tri_pos + 9 * (size_t)prim;
    const float b0 = 1.0f - h.b1 - h.b2;
    const F3 p = f3m(b0 * tp[0] + h.b1 * tp[3] + h.b2 * tp[6], b0 * tp[1] + h.b1 * tp[4] + h.b2 * tp[7],
                     b0 * tp[2] + h.b1 * tp[5] + h.b2 * tp[8]);
    const F3 ng = f3m(sc.tri_normal[3 * prim], sc.tri_normal[3 * prim + 1], sc.tri_normal[3 * prim + 2]);
    const F3 ns = ng;
    const F3 wo = -rd;
    const uint32_t mi = sc.tri_material[prim];
    const sty_scene_material m = sc.materials[mi];
    // emitter (handle_surface_light) and stylization flags (update_stylization_flags)
    F3 le;
    float mis;
    emitter_le(sc, m, prim, p, ng, rd, depth, prev_p, prev_pdf, &le, &mis);
    const uint32_t new_flags = update_flags(m, flags);
    v.active[tid] = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float pa = a == 0 ? p.x : a == 1 ? p.y : p.z;
        v.p[a][tid] = pa;
    }
    v.wo[0][tid] = wo.x; v.wo[1][tid] = wo.y; v.wo[2][tid] = wo.z;
    v.ns[0][tid] = ns.x; v.ns[1][tid] = ns.y; v.ns[2][tid] = ns.z;
    v.ng[0][tid] = ng.x; v.ng[1][tid] = ng.y; v.ng[2][tid] = ng.z;
    v.le[0][tid] = le.x; v.le[1][tid] = le.y; v.le[2][tid] = le.z;
    v.mis[tid] = mis;
    v.flags[tid] = new_flags;
    v.material[tid] = mi;
    v.dir_pdf[tid] = 0.0f;
    v.dir_wi[0][tid] = v.dir_wi[1][tid] = v.dir_wi[2][tid] = 0.0f;
    v.dir_l[0][tid] = v.dir_l[1][tid] = v.dir_l[2][tid] = 0.0f;
    v.ind_wi[0][tid] = v.ind_wi[1][tid] = v.ind_wi[2][tid] = 0.0f;
    v.ind_mis[tid] = 0.0f;
    if (depth > 0) {  // the parent's indirect record: wi = -wo, mis (kernel_filter :1043-1047)
        parent.ind_wi[0][tid] = rd.x;
        parent.ind_wi[1][tid] = rd.y;
        parent.ind_wi[2][tid] = rd.z;
        parent.ind_mis[tid] = mis;
        if (recs && mis != 1.0f)  // the parent's throughput carries this vertex's emission MIS weight
            for (int c = 0; c < 3; c++) rec_parent.thr[c][tid] *= mis;
    }
    F3 rad = le;  // screen record: emission (with its MIS weight) + light sample (balance MIS)
    if (recs) {
        if (rec.prim) rec.prim[tid] = prim;
        rec.rad[0][tid] = le.x; rec.rad[1][tid] = le.y; rec.rad[2][tid] = le.z;
        rec.thr[0][tid] = 0.0f; rec.thr[1][tid] = 0.0f; rec.thr[2][tid] = 0.0f;
    }
    if (depth >= max_depth) {
        ps.terminated[tid] = 1;
        rng[tid] = st;
        return;
    }
    // NEE (sample_light)
    {
        F3 lwi;
        f3 li;
        float lpdf;
        if (nee_sample(sc, p, ng, prim, new_flags, depth, progs, n_progs, st, &lwi, &li, &lpdf)) {
            v.dir_wi[0][tid] = lwi.x;
            v.dir_wi[1][tid] = lwi.y;
            v.dir_wi[2][tid] = lwi.z;
            v.dir_l[0][tid] = li.x;
            v.dir_l[1][tid] = li.y;
            v.dir_l[2][tid] = li.z;
            v.dir_pdf[tid] = lpdf;
            if (recs) {  // the direct term of the reference's filter with the vertex as its own neighbour
                F3 f;
                const float bp = bsdf_eval(m, ns, ng, wo, lwi, &f, sc.ggx_tab);
                const float w = lpdf / (lpdf + bp) / lpdf;
                rad = rad + f3m(f.x * li.x, f.y * li.y, f.z * li.z) * w;
                rec.rad[0][tid] = rad.x; rec.rad[1][tid] = rad.y; rec.rad[2][tid] = rad.z;
            }
        }
    }
    // final-gathering renders stop at the first rough vertex (splitting, nrc_pt.rs:372-375)
    if (split_rough > 0.0f && lobe_roughness(m, sc.ggx_tab, ns, wo) > split_rough) {
        ps.split[tid] = depth;
        ps.exclude[tid] = prim;  // the split vertex's triangle, skipped by its gather rays
        ps.terminated[tid] = 1;
        rng[tid] = st;
        return;
    }
    // BSDF sample and continuation
    const float usel = next_1d(st), us0 = next_1d(st), us1 = next_1d(st);
    float pdf = 0.0f;
    const F3 wi = bsdf_sample(m, ns, ng, wo, usel, us0, us1, &pdf, sc.ggx_tab);
    if (recs && pdf > 0.0f) {  // throughput to the child: f |cos| / pdf (times the child's MIS weight, above)
        F3 f;
        const float bp = bsdf_eval(m, ns, ng, wo, wi, &f, sc.ggx_tab);
        if (bp > 0.0f) {
            const float k = 1.0f / bp;
            rec.thr[0][tid] = f.x * k; rec.thr[1][tid] = f.y * k; rec.thr[2][tid] = f.z * k;
        }
    }
    if (pdf > 0.0f) {
        const F3 no = offset_ray_origin(p, face_forward(ng, wi));
        ps.o[0][tid] = no.x; ps.o[1][tid] = no.y; ps.o[2][tid] = no.z;
        ps.d[0][tid] = wi.x; ps.d[1][tid] = wi.y; ps.d[2][tid] = wi.z;
        ps.prev_p[0][tid] = p.x; ps.prev_p[1][tid] = p.y; ps.prev_p[2][tid] = p.z;
        ps.prev_pdf[tid] = pdf;
        ps.flags[tid] = new_flags;
        ps.exclude[tid] = prim;
    } else {
        ps.terminated[tid] = 1;
    }
    rng[tid] = st;
}

// splat + first-hit stylization + film (kernel_splat / kernel_update_film, :429-506)
__global__ void k_splat(uint32_t npx, uint32_t branch, const float *out0, VertOut v0, const sty_scene_material *mats,
                        const sty_style_program *progs, uint32_t n_progs, int no_first_hit, double weight,
                        double *film) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npx) return;
    const size_t n = (size_t)npx * branch;
    f3 sum = {0.0f, 0.0f, 0.0f};
    for (uint32_t b = 0; b < branch; b++) {
        const size_t i = (size_t)b * npx + px;
        if (!v0.active[i]) continue;
        sum.x += out0[i];
        sum.y += out0[n + i];
        sum.z += out0[2 * n + i];
    }
    const float sc = 1.0f / (float)branch;
    const f3 mean = {sum.x * sc, sum.y * sc, sum.z * sc};
    double acc[3] = {0, 0, 0};
    uint32_t cnt = 0;
    for (uint32_t b = 0; b < branch; b++) {
        const size_t i = (size_t)b * npx + px;
        if (!v0.active[i]) continue;
        f3 c = mean;
        if (!no_first_hit) {
            // the path's flags before its first hit are all clear: style index 0
            const int32_t pi = mats[v0.material[i]].style[0];
            if (pi >= 0 && (uint32_t)pi < n_progs) c = style_apply(progs[pi], 0, c, f3{v0.p[0][i], v0.p[1][i], v0.p[2][i]});
        }
        acc[0] += c.x;
        acc[1] += c.y;
        acc[2] += c.z;
        cnt++;
    }
    if (cnt)
        for (int c = 0; c < 3; c++) film[3 * (size_t)px + c] += weight * acc[c] / cnt;
}


// Per-vertex radiance estimate reusing only the vertex itself: le + own NEE (balance MIS) +
// f * L_next * mis_next / pdf (evaluate_filtered_radiance :758-972 with a one-element neighbour set)
__global__ void k_self_radiance(SceneView sc, uint32_t n, VertOut v, const float *next, float *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!v.active[i]) {
        out[i] = out[n + i] = out[2 * (size_t)n + i] = 0.0f;
        return;
    }
    const sty_scene_material m = sc.materials[v.material[i]];
    const F3 ns = f3m(v.ns[0][i], v.ns[1][i], v.ns[2][i]), ng = f3m(v.ng[0][i], v.ng[1][i], v.ng[2][i]);
    const F3 wo = f3m(v.wo[0][i], v.wo[1][i], v.wo[2][i]);
    F3 rad = f3m(v.le[0][i], v.le[1][i], v.le[2][i]);
    const float dpdf = v.dir_pdf[i];
    if (dpdf > 0.0f) {
        F3 f;
        const float bp = bsdf_eval(m, ns, ng, wo, f3m(v.dir_wi[0][i], v.dir_wi[1][i], v.dir_wi[2][i]), &f, sc.ggx_tab);
        const float w = dpdf / (dpdf + bp) / dpdf;
        rad = rad + f3m(f.x * v.dir_l[0][i], f.y * v.dir_l[1][i], f.z * v.dir_l[2][i]) * w;
    }
    const F3 wi = f3m(v.ind_wi[0][i], v.ind_wi[1][i], v.ind_wi[2][i]);
    if (next && dot(wi, wi) != 0.0f) {
        F3 f;
        const float bp = bsdf_eval(m, ns, ng, wo, wi, &f, sc.ggx_tab);
        if (bp > 0.0f) {
            const float s = v.ind_mis[i] / bp;
            rad = rad + f3m(f.x * next[i], f.y * next[n + i], f.z * next[2 * (size_t)n + i]) * s;
        }
    }
    out[i] = rad.x;
    out[n + i] = rad.y;
    out[2 * (size_t)n + i] = rad.z;
}

// NRC input rows. Layout STY_NRC_ROWS_REF follows write_nrc_inputs (nrc_pt.rs:583-663): position
// normalised to the scene box, ns * 0.5 + 0.5, wo * 0.5 + 0.5, roughness (diffuse 1, GGX alpha),
// albedo, [disabled, enabled], one-hot style index (4), one-hot depth (max_depth + 1):
// 20 + max_depth floats. Layout STY_NRC_ROWS_SPHERICAL is the 11-input row of the frequency-encoded
// cache: normalised position, normal and wo as (theta / pi, (phi + pi) / 2pi)
// (xyz_to_spherical_normalized, geometry.rs:342-346), roughness, albedo.
struct FeatArgs {
    float bmin[3], bext[3];
    uint32_t max_depth, dims, layout;
};
__device__ __forceinline__ void sph(F3 w, float *t, float *p) {
    *t = acosf(fminf(fmaxf(w.z, -1.0f), 1.0f)) * (1.0f / kPi);
    *p = (atan2f(w.y, w.x) + kPi) * (0.5f / kPi);
}
__device__ void write_features(const SceneView &sc, const FeatArgs &fa, F3 p, F3 wo, F3 ns, uint32_t mi,
                               uint32_t flags, uint32_t depth, float *row) {
    const sty_scene_material m = sc.materials[mi];
    row[0] = (p.x - fa.bmin[0]) / fa.bext[0];
    row[1] = (p.y - fa.bmin[1]) / fa.bext[1];
    row[2] = (p.z - fa.bmin[2]) / fa.bext[2];
    const float rough = lobe_roughness(m, sc.ggx_tab, ns, wo);
    if (fa.layout == STY_NRC_ROWS_SPHERICAL) {
        sph(ns, &row[3], &row[4]);
        sph(wo, &row[5], &row[6]);
        row[7] = rough;
        row[8] = m.albedo[0];
        row[9] = m.albedo[1];
        row[10] = m.albedo[2];
        return;
    }
    row[3] = ns.x * 0.5f + 0.5f;
    row[4] = ns.y * 0.5f + 0.5f;
    row[5] = ns.z * 0.5f + 0.5f;
    row[6] = wo.x * 0.5f + 0.5f;
    row[7] = wo.y * 0.5f + 0.5f;
    row[8] = wo.z * 0.5f + 0.5f;
    row[9] = rough;
    row[10] = m.albedo[0];
    row[11] = m.albedo[1];
    row[12] = m.albedo[2];
    const bool off = (flags & 1u) != 0;
    row[13] = off ? 1.0f : 0.0f;
    row[14] = off ? 0.0f : 1.0f;
    const uint32_t si = style_index(flags);
    for (uint32_t k = 0; k < 4; k++) row[15 + k] = k == si ? 1.0f : 0.0f;
    for (uint32_t k = 0; k <= fa.max_depth; k++) row[19 + k] = k == depth ? 1.0f : 0.0f;
}
// Rows of one depth, in path order after the rows of the earlier depths: row = *base + idx[i],
// idx the exclusive prefix sum of the active flags.
__global__ void k_nrc_train_rows(SceneView sc, FeatArgs fa, uint32_t n, uint32_t depth, VertOut v, const float *rad,
                                 const uint32_t *idx, const unsigned long long *base, float *inputs, float *targets,
                                 uint64_t capacity) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !v.active[i]) return;
    const unsigned long long k = *base + idx[i];
    if (k >= capacity) return;
    write_features(sc, fa, f3m(v.p[0][i], v.p[1][i], v.p[2][i]), f3m(v.wo[0][i], v.wo[1][i], v.wo[2][i]),
                   f3m(v.ns[0][i], v.ns[1][i], v.ns[2][i]), v.material[i], v.flags[i], depth, inputs + k * fa.dims);
    targets[k * 3] = rad[i];
    targets[k * 3 + 1] = rad[n + i];
    targets[k * 3 + 2] = rad[2 * (size_t)n + i];
}
__global__ void k_advance_rows(uint32_t n, const uint32_t *idx, const int32_t *active, unsigned long long *base) {
    *base += (unsigned long long)idx[n - 1] + (active[n - 1] ? 1u : 0u);
}
__global__ void k_nrc_query_rows(SceneView sc, FeatArgs fa, uint32_t n, VertOut v, float *inputs, float *targets,
                                 uint32_t depth = 0) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float *row = inputs + (size_t)i * fa.dims;
    float le[3] = {0.0f, 0.0f, 0.0f};
    if (v.active[i]) {
        write_features(sc, fa, f3m(v.p[0][i], v.p[1][i], v.p[2][i]), f3m(v.wo[0][i], v.wo[1][i], v.wo[2][i]),
                       f3m(v.ns[0][i], v.ns[1][i], v.ns[2][i]), v.material[i], v.flags[i], depth, row);
        le[0] = v.le[0][i];
        le[1] = v.le[1][i];
        le[2] = v.le[2][i];
    } else {
        for (uint32_t c = 0; c < fa.dims; c++) row[c] = 0.0f;
    }
    for (int c = 0; c < 3; c++) targets[(size_t)i * 3 + c] = le[c];
}

// The cache's predictions for the vertices of one depth (rows [n][3], dense in path order) as
// radiance planes [3][n], styled at that depth by the vertex's material and flags unless the cache
// learns styled radiance (nrc_pt.rs:748-775); inactive slots give 0.
__global__ void k_nrc_style_pred(SceneView sc, uint32_t n, VertOut v, const float *pred, const sty_style_program *progs,
                                 uint32_t n_progs, uint32_t depth, int stylize, float *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 c = {0.0f, 0.0f, 0.0f};
    if (v.active[i]) {
        c = {pred[3 * (size_t)i], pred[3 * (size_t)i + 1], pred[3 * (size_t)i + 2]};
        const uint32_t fl = v.flags[i];
        if (stylize && !(fl & 1u)) {
            const int32_t pi = sc.materials[v.material[i]].style[style_index(fl)];
            if (pi >= 0 && (uint32_t)pi < n_progs) c = style_apply(progs[pi], depth, c, f3{v.p[0][i], v.p[1][i], v.p[2][i]});
        }
    }
    out[i] = c.x;
    out[n + i] = c.y;
    out[2 * (size_t)n + i] = c.z;
}
// Rendering pass: one first hit per pixel (path i = pixel i); the cache's prediction there, styled
// at depth 0 unless no_first_hit_stylization, into the FP64 film (kernel_inference_stage_gathering,
// nrc_pt.rs:877-965).
__global__ void k_nrc_splat_pred(uint32_t npx, VertOut v0, const float *pred, const sty_scene_material *mats,
                                 const sty_style_program *progs, uint32_t n_progs, int no_first_hit, double weight,
                                 double *film) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npx || !v0.active[px]) return;
    f3 c = {pred[3 * (size_t)px], pred[3 * (size_t)px + 1], pred[3 * (size_t)px + 2]};
    const uint32_t fl = v0.flags[px];
    if (!no_first_hit && !(fl & 1u)) {
        const int32_t pi = mats[v0.material[px]].style[style_index(fl)];
        if (pi >= 0 && (uint32_t)pi < n_progs) c = style_apply(progs[pi], 0, c, f3{v0.p[0][px], v0.p[1][px], v0.p[2][px]});
    }
    film[3 * (size_t)px] += weight * c.x;
    film[3 * (size_t)px + 1] += weight * c.y;
    film[3 * (size_t)px + 2] += weight * c.z;
}
// zero the targets that are not finite (the reference drops such rows, :790-793)
__global__ void k_finite_targets(size_t n3, float *t) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3 && !isfinite(t[i])) t[i] = 0.0f;
}

// ---- final gathering (nrc_pt.rs:436-582, 877-965, 969-1047) -------------------------------------
// The split vertex of every path, gathered from the per-depth planes into per-path planes.
struct SplitPlanes {
    float *p[3], *wo[3], *ns[3], *ng[3];
    uint32_t *material, *flags, *prim;
};
__global__ void k_split_collect(uint32_t n, uint32_t d, VertOut v, const uint32_t *split, const uint32_t *prim_of,
                                SplitPlanes sp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || split[i] != d) return;
    for (int a = 0; a < 3; a++) {
        sp.p[a][i] = v.p[a][i];
        sp.wo[a][i] = v.wo[a][i];
        sp.ns[a][i] = v.ns[a][i];
        sp.ng[a][i] = v.ng[a][i];
    }
    sp.material[i] = v.material[i];
    sp.flags[i] = v.flags[i];
    sp.prim[i] = prim_of[i];
}
// One gather iteration for every split path: another light sample at the split vertex (added to
// acc_direct) and one BSDF-sampled ray; its hit becomes a cache query row (zero row if none) with
// the sample's throughput f |cos| / pdf and the hit's emission MIS weight.
__global__ void k_fg_step(SceneView sc, FeatArgs fa, uint32_t n, const uint32_t *split, SplitPlanes sp, sty_pcg32 *rng,
                          const sty_style_program *progs, uint32_t n_progs, float *rows, float *thr, float *gmis,
                          uint32_t *gmat, uint32_t *gflags, float *gpos, float *acc_direct) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float *row = rows + (size_t)i * fa.dims;
    for (uint32_t c = 0; c < fa.dims; c++) row[c] = 0.0f;
    thr[i] = thr[n + i] = thr[2 * (size_t)n + i] = 0.0f;
    const uint32_t s = split[i];
    if (s == NONE) return;
    sty_pcg32 st = rng[i];
    const sty_scene_material m = sc.materials[sp.material[i]];
    const F3 p = f3m(sp.p[0][i], sp.p[1][i], sp.p[2][i]), wo = f3m(sp.wo[0][i], sp.wo[1][i], sp.wo[2][i]);
    const F3 ns = f3m(sp.ns[0][i], sp.ns[1][i], sp.ns[2][i]), ng = f3m(sp.ng[0][i], sp.ng[1][i], sp.ng[2][i]);
    const uint32_t fl = sp.flags[i], prim = sp.prim[i];
    {
        F3 lwi;
        f3 li;
        float lpdf;
        if (nee_sample(sc, p, ng, prim, fl, s, progs, n_progs, st, &lwi, &li, &lpdf)) {
            F3 f;
            const float bp = bsdf_eval(m, ns, ng, wo, lwi, &f, sc.ggx_tab);
            const float w = lpdf / (lpdf + bp) / lpdf;
            acc_direct[i] += f.x * li.x * w;
            acc_direct[n + i] += f.y * li.y * w;
            acc_direct[2 * (size_t)n + i] += f.z * li.z * w;
        }
    }
    const float usel = next_1d(st), us0 = next_1d(st), us1 = next_1d(st);
    float pdf = 0.0f;
    const F3 wi = bsdf_sample(m, ns, ng, wo, usel, us0, us1, &pdf, sc.ggx_tab);
    rng[i] = st;
    if (!(pdf > 0.0f)) return;
    const F3 o = offset_ray_origin(p, face_forward(ng, wi));
    const float o3[3] = {o.x, o.y, o.z}, d3[3] = {wi.x, wi.y, wi.z};
    const Hit h = trace_closest(sc, o3, d3, 0.0f, 1e20f, prim);
    if (h.prim == NONE) return;
    const float *tp = sc.tri_pos + 9 * (size_t)h.prim;
    const float b0 = 1.0f - h.b1 - h.b2;
    const F3 q = f3m(b0 * tp[0] + h.b1 * tp[3] + h.b2 * tp[6], b0 * tp[1] + h.b1 * tp[4] + h.b2 * tp[7],
                     b0 * tp[2] + h.b1 * tp[5] + h.b2 * tp[8]);
    const F3 qn = f3m(sc.tri_normal[3 * h.prim], sc.tri_normal[3 * h.prim + 1], sc.tri_normal[3 * h.prim + 2]);
    const uint32_t qm = sc.tri_material[h.prim];
    const sty_scene_material mq = sc.materials[qm];
    float mis = 1.0f;
    if (mq.emission[0] > 0.0f || mq.emission[1] > 0.0f || mq.emission[2] > 0.0f) {  // handle_surface_light
        float sel = 0.0f;
        for (uint32_t k = 0; k < sc.n_lights; k++)
            if (sc.light_tris[k] == h.prim) sel = sc.light_cdf[k + 1] - sc.light_cdf[k];
        const F3 w = q - p;
        const float dist2 = dot(w, w);
        const float lpdf = sel / sc.tri_area[h.prim] * dist2 / fmaxf(fabsf(dot(qn, w * (1.0f / sqrtf(dist2)))), 1e-6f);
        mis = pdf / (pdf + lpdf);
    }
    uint32_t qf = fl;  // update_stylization_flags at the gather hit
    if (mq.set_style >= 0) {
        qf &= 1u;
        if (mq.set_style == 1) qf |= 2u;
        if (mq.set_style == 2) qf |= 4u;
        if (mq.set_style == 3) qf |= 8u;
    }
    F3 f;
    const float bp = bsdf_eval(m, ns, ng, wo, wi, &f, sc.ggx_tab);
    if (!(bp > 0.0f)) return;
    thr[i] = f.x / bp;
    thr[n + i] = f.y / bp;
    thr[2 * (size_t)n + i] = f.z / bp;
    gmis[i] = mis;
    gmat[i] = qm;
    gflags[i] = qf;
    gpos[i] = q.x;
    gpos[n + i] = q.y;
    gpos[2 * (size_t)n + i] = q.z;
    write_features(sc, fa, q, -wi, qn, qm, qf, s + 1, row);
}
// acc_indirect += style_{s+1}(cache prediction at the gather hit) * throughput * mis; every
// iteration counts (a miss contributes 0)
__global__ void k_fg_accumulate(SceneView sc, uint32_t n, const uint32_t *split, const float *pred, const float *thr,
                                const float *gmis, const uint32_t *gmat, const uint32_t *gflags, const float *gpos,
                                const sty_style_program *progs, uint32_t n_progs, int stylize, float *acc_ind,
                                float *ngath) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || split[i] == NONE) return;
    ngath[i] += 1.0f;
    if (thr[i] == 0.0f && thr[n + i] == 0.0f && thr[2 * (size_t)n + i] == 0.0f) return;
    f3 c = {pred[3 * (size_t)i], pred[3 * (size_t)i + 1], pred[3 * (size_t)i + 2]};
    const uint32_t fl = gflags[i];
    if (stylize && !(fl & 1u)) {
        const int32_t pi = sc.materials[gmat[i]].style[style_index(fl)];
        const f3 q = {gpos[i], gpos[n + i], gpos[2 * (size_t)n + i]};
        if (pi >= 0 && (uint32_t)pi < n_progs) c = style_apply(progs[pi], split[i] + 1, c, q);
    }
    const float w = gmis[i];
    if (!(isfinite(c.x) && isfinite(c.y) && isfinite(c.z))) return;
    acc_ind[i] += c.x * thr[i] * w;
    acc_ind[n + i] += c.y * thr[n + i] * w;
    acc_ind[2 * (size_t)n + i] += c.z * thr[2 * (size_t)n + i] * w;
}
// Backward sweep over depth d (propagate_and_splat :969-1047): at the split vertex
// Le + direct / (n + 1) + indirect / n, elsewhere Le + direct + f L_{d+1} mis / pdf; styled at
// depth d when `stylize` (style applies at d > 0, and at 0 unless no_first_hit_stylization).
__global__ void k_fg_sweep(SceneView sc, uint32_t n, uint32_t d, VertOut v, const float *next, const uint32_t *split,
                           const float *acc_direct, const float *acc_ind, const float *ngath,
                           const sty_style_program *progs, uint32_t n_progs, int stylize, float *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 r = {0.0f, 0.0f, 0.0f};
    if (v.active[i]) {
        const sty_scene_material m = sc.materials[v.material[i]];
        const F3 ns = f3m(v.ns[0][i], v.ns[1][i], v.ns[2][i]), ng = f3m(v.ng[0][i], v.ng[1][i], v.ng[2][i]);
        const F3 wo = f3m(v.wo[0][i], v.wo[1][i], v.wo[2][i]);
        F3 dir = f3m(0.0f, 0.0f, 0.0f);
        const float dpdf = v.dir_pdf[i];
        if (dpdf > 0.0f) {
            F3 f;
            const float bp = bsdf_eval(m, ns, ng, wo, f3m(v.dir_wi[0][i], v.dir_wi[1][i], v.dir_wi[2][i]), &f, sc.ggx_tab);
            const float w = dpdf / (dpdf + bp) / dpdf;
            dir = f3m(f.x * v.dir_l[0][i] * w, f.y * v.dir_l[1][i] * w, f.z * v.dir_l[2][i] * w);
        }
        r = {v.le[0][i], v.le[1][i], v.le[2][i]};
        if (split[i] == d) {
            const float ng_ = ngath[i];
            const float kd = 1.0f / (ng_ + 1.0f), ki = ng_ > 0.0f ? 1.0f / ng_ : 0.0f;
            r.x += (dir.x + acc_direct[i]) * kd + acc_ind[i] * ki;
            r.y += (dir.y + acc_direct[n + i]) * kd + acc_ind[n + i] * ki;
            r.z += (dir.z + acc_direct[2 * (size_t)n + i]) * kd + acc_ind[2 * (size_t)n + i] * ki;
        } else {
            r.x += dir.x;
            r.y += dir.y;
            r.z += dir.z;
            const F3 wi = f3m(v.ind_wi[0][i], v.ind_wi[1][i], v.ind_wi[2][i]);
            if (next && dot(wi, wi) != 0.0f) {
                F3 f;
                const float bp = bsdf_eval(m, ns, ng, wo, wi, &f, sc.ggx_tab);
                if (bp > 0.0f) {
                    const float k = v.ind_mis[i] / bp;
                    r.x += f.x * next[i] * k;
                    r.y += f.y * next[n + i] * k;
                    r.z += f.z * next[2 * (size_t)n + i] * k;
                }
            }
        }
        const uint32_t fl = v.flags[i];
        if (stylize && !(fl & 1u)) {
            const int32_t pi = m.style[style_index(fl)];
            if (pi >= 0 && (uint32_t)pi < n_progs) r = style_apply(progs[pi], d, r, f3{v.p[0][i], v.p[1][i], v.p[2][i]});
        }
    }
    out[i] = r.x;
    out[n + i] = r.y;
    out[2 * (size_t)n + i] = r.z;
}
__global__ void k_fg_splat(uint32_t npx, const int32_t *active0, const float *rad0, double weight, double *film) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npx || !active0[px]) return;
    for (int c = 0; c < 3; c++) film[3 * (size_t)px + c] += weight * rad0[(size_t)c * npx + px];
}

}  // namespace
}  // namespace sty

using namespace sty;

namespace {


// Device buffers a scene keeps between renders (grown on demand, freed with the scene): renders
// of one scene reuse them, so calls on one scene are serialised by the caller.
enum CacheSlot {
    kVerts, kOuts, kPathState, kRng, kPrograms, kVertexCount, kRowCount, kRowIndex, kScanTmp,
    kQueryIn, kQueryPred, kQueryScratch, kTargets, kRowsIn, kRowsTgt, kFinalGather, kRecords, kSlots
};
struct RenderCache {
    void *p[kSlots] = {};
    size_t bytes[kSlots] = {};
    sty_pf_ref_ctx *ctx = nullptr;
    uint64_t ctx_cap = 0;
    ~RenderCache() {
        for (void *q : p)
            if (q) cudaFree(q);
        if (ctx) sty_pf_ref_destroy(ctx);
    }
};
RenderCache &render_cache(sty_scene *scene) {
    void *&c = scene_render_cache(scene);
    if (!c) c = new RenderCache();
    return *static_cast<RenderCache *>(c);
}

// Per-depth vertex planes, path state, per-path Pcg32 and per-depth radiance planes of one
// wavefront trace, in the scene's cached buffers.
struct TraceJob {
    static constexpr size_t kPlanes = 30;  // per depth: active, 27 float planes, flags, material
    uint32_t npx = 0, n = 0, D = 0, max_depth = 0, n_programs = 0;
    CamArgs ca;
    SceneView sv;
    RenderCache *cache = nullptr;
    float *verts = nullptr, *outs = nullptr, *psb = nullptr;
    sty_pcg32 *rng = nullptr;
    sty_style_program *dprog = nullptr;
    unsigned long long *vc = nullptr;
    std::vector<VertOut> vo;
    std::vector<sty_pf_vertices> vin;
    PathState ps;
    float bmin[3], bmax[3];
    float split_rough = 0.0f;  // > 0: stop paths at the first vertex rougher than this
    // STY_PF_MODE_SCREEN: slots in pixel-major order, and the screen-space record planes the tracer
    // writes (each plane D * n, sty_pf_records order); the vertex planes p, ns and active alias them
    uint32_t pixel_major = 0;
    sty_pf_records_out rp{};
    std::vector<RecOut> ro;
    sty_status s = STY_OK;

    void *alloc(CacheSlot k, size_t bytes, const char *what) {
        if (s != STY_OK) return nullptr;
        if (cache->bytes[k] < bytes) {
            if (cache->p[k]) cudaFree(cache->p[k]);
            cache->p[k] = nullptr;
            cache->bytes[k] = 0;
            s = check_cuda(cudaMalloc(&cache->p[k], bytes), what);
            if (s != STY_OK) return nullptr;
            cache->bytes[k] = bytes;
        }
        return cache->p[k];
    }
    sty_status init(sty_scene *scene, uint32_t branch, uint32_t maxd, const sty_style_program *programs,
                    uint32_t nprog, uint64_t seed, cudaStream_t st, uint32_t paths = 0, uint32_t pmajor = 0) {
        const sty_camera &cam = scene_camera(scene);
        npx = cam.width * cam.height;
        const uint64_t np64 = paths ? (uint64_t)paths : (uint64_t)npx * branch;
        if (np64 >= (1ull << 31)) {
            set_error("too many paths (%llu)", (unsigned long long)np64);
            return STY_ERR_ARG;
        }
        n = (uint32_t)np64;
        max_depth = maxd;
        D = maxd + 1;
        n_programs = nprog;
        cache = &render_cache(scene);
        ca = make_camera(cam);
        ca.pixel_major = pixel_major = pmajor;
        sv = scene_view(scene);
        scene_bounds(scene, bmin, bmax);
        verts = (float *)alloc(kVerts, (size_t)D * kPlanes * n * 4, "alloc vertices");
        outs = (float *)alloc(kOuts, (size_t)D * 3 * n * 4, "alloc outputs");
        psb = (float *)alloc(kPathState, (size_t)14 * n * 4, "alloc path state");
        rng = (sty_pcg32 *)alloc(kRng, (size_t)n * sizeof(sty_pcg32), "alloc rng");
        dprog = (sty_style_program *)alloc(kPrograms, 64 * sizeof(sty_style_program), "alloc programs");
        vc = (unsigned long long *)alloc(kVertexCount, 8, "alloc counter");
        if (s != STY_OK) return s;
        if (nprog)
            STY_TRY(check_cuda(cudaMemcpyAsync(dprog, programs, nprog * sizeof(sty_style_program),
                                               cudaMemcpyHostToDevice, st), "upload programs"));
        STY_TRY(check_cuda(cudaMemsetAsync(vc, 0, 8, st), "zero counter"));
        vo.resize(D);
        vin.resize(D);
        for (uint32_t d = 0; d < D; d++) {
            float *b = verts + (size_t)d * kPlanes * n;
            int k = 0;
            auto pl = [&]() { return b + (size_t)(k++) * n; };
            VertOut &w = vo[d];
            w.active = (int32_t *)pl();
            for (int a = 0; a < 3; a++) w.p[a] = pl();
            for (int a = 0; a < 3; a++) w.wo[a] = pl();
            for (int a = 0; a < 3; a++) w.ns[a] = pl();
            for (int a = 0; a < 3; a++) w.ng[a] = pl();
            for (int a = 0; a < 3; a++) w.le[a] = pl();
            w.mis = pl();
            for (int a = 0; a < 3; a++) w.dir_wi[a] = pl();
            for (int a = 0; a < 3; a++) w.dir_l[a] = pl();
            w.dir_pdf = pl();
            for (int a = 0; a < 3; a++) w.ind_wi[a] = pl();
            w.ind_mis = pl();
            w.flags = (uint32_t *)pl();
            w.material = (uint32_t *)pl();
            sty_pf_vertices &r = vin[d];
            r.active = w.active;
            for (int a = 0; a < 3; a++) {
                r.p[a] = w.p[a];
                r.wo[a] = w.wo[a];
                r.ns[a] = w.ns[a];
                r.ng[a] = w.ng[a];
                r.le[a] = w.le[a];
                r.dir_wi[a] = w.dir_wi[a];
                r.dir_l[a] = w.dir_l[a];
                r.ind_wi[a] = w.ind_wi[a];
            }
            r.mis = w.mis;
            r.dir_pdf = w.dir_pdf;
            r.ind_mis = w.ind_mis;
            r.flags = w.flags;
            r.material = w.material;
            r.n = n;
        }
        int k = 0;
        auto pl = [&]() { return psb + (size_t)(k++) * n; };
        for (int a = 0; a < 3; a++) ps.o[a] = pl();
        for (int a = 0; a < 3; a++) ps.d[a] = pl();
        for (int a = 0; a < 3; a++) ps.prev_p[a] = pl();
        ps.prev_pdf = pl();
        ps.flags = (uint32_t *)pl();
        ps.exclude = (uint32_t *)pl();
        ps.terminated = (uint32_t *)pl();
        ps.split = (uint32_t *)pl();
        ro.assign(D, RecOut{});
        k_rng_init<<<(n + 255) / 256, 256, 0, st>>>(n, std_rng_key_of(seed), pixel_major, npx, rng);
        return check_launch("k_rng_init");
    }
    // SCREEN mode: the tracer writes screen records, into `ext` (caller planes) or into the scene's
    // cache; the vertex planes p, ns and active of every depth become views of the record planes
    sty_status init_records(const sty_pf_records_out *ext) {
        if (ext) {
            rp = *ext;
        } else {
            float *b = (float *)alloc(kRecords, (size_t)13 * D * n * 4, "alloc records");
            if (s != STY_OK) return s;
            for (int a = 0; a < 3; a++) {
                rp.pos[a] = b + (size_t)a * D * n;
                rp.nrm[a] = b + (size_t)(3 + a) * D * n;
                rp.rad[a] = b + (size_t)(6 + a) * D * n;
                rp.thr[a] = b + (size_t)(9 + a) * D * n;
            }
            rp.valid = (int32_t *)(b + (size_t)12 * D * n);
            rp.prim = nullptr;
        }
        for (uint32_t d = 0; d < D; d++) {
            const size_t o = (size_t)d * n;
            VertOut &w = vo[d];
            sty_pf_vertices &r = vin[d];
            w.active = rp.valid + o;
            r.active = w.active;
            for (int a = 0; a < 3; a++) {
                w.p[a] = rp.pos[a] + o;
                w.ns[a] = rp.nrm[a] + o;
                r.p[a] = w.p[a];
                r.ns[a] = w.ns[a];
                ro[d].rad[a] = rp.rad[a] + o;
                ro[d].thr[a] = rp.thr[a] + o;
            }
            ro[d].prim = rp.prim ? rp.prim + o : nullptr;
        }
        return STY_OK;
    }
    sty_pf_records records(uint32_t spp) const {
        sty_pf_records r;
        for (int a = 0; a < 3; a++) {
            r.pos[a] = rp.pos[a];
            r.nrm[a] = rp.nrm[a];
            r.rad[a] = rp.rad[a];
            r.thr[a] = rp.thr[a];
        }
        r.valid = rp.valid;
        r.width = (int32_t)ca.W;
        r.height = (int32_t)ca.H;
        r.spp = (int32_t)spp;
        r.depths = (int32_t)D;
        return r;
    }
    // all depths of one wavefront (kernel_trace dispatch loop, lm_path_filtering.rs:1646-1654)
    sty_status trace(cudaStream_t st) {
        STY_TRY(check_cuda(cudaMemsetAsync(verts, 0, (size_t)D * kPlanes * n * 4, st), "reset vertices"));
        if (rp.valid) {  // records of slots without a hit read as invalid zeros
            const size_t pl = (size_t)D * n * 4;
            for (int a = 0; a < 3; a++) {
                STY_TRY(check_cuda(cudaMemsetAsync(rp.pos[a], 0, pl, st), "reset records"));
                STY_TRY(check_cuda(cudaMemsetAsync(rp.nrm[a], 0, pl, st), "reset records"));
                STY_TRY(check_cuda(cudaMemsetAsync(rp.rad[a], 0, pl, st), "reset records"));
                STY_TRY(check_cuda(cudaMemsetAsync(rp.thr[a], 0, pl, st), "reset records"));
            }
            STY_TRY(check_cuda(cudaMemsetAsync(rp.valid, 0, pl, st), "reset records"));
            if (rp.prim) STY_TRY(check_cuda(cudaMemsetAsync(rp.prim, 0xff, pl, st), "reset records"));
        }
        for (uint32_t d = 0; d < D; d++) {
            k_trace<<<(n + 255) / 256, 256, 0, st>>>(sv, ca, n, d, max_depth, ps, vo[d], vo[d > 0 ? d - 1 : 0], rng,
                                                     dprog, n_programs, vc, split_rough, ro[d],
                                                     ro[d > 0 ? d - 1 : 0]);
            STY_TRY(check_launch("k_trace"));
        }
        return STY_OK;
    }
    float *out(uint32_t d) { return outs + (size_t)d * 3 * n; }
};

}  // namespace

namespace sty {
void render_cache_free(void *cache) { delete static_cast<RenderCache *>(cache); }
}  // namespace sty

namespace {
sty_status check_render_config(const sty_pf_render_config *cfg, const sty_style_program *programs,
                               uint32_t n_programs) {
    STY_ARG_CHECK(cfg->branch >= 1 && cfg->repeats >= 1 && cfg->max_depth <= 30, "bad branch / repeats / max_depth");
    STY_ARG_CHECK(programs || n_programs == 0, "null programs");
    STY_ARG_CHECK(n_programs <= 64, "at most 64 style programs");
    STY_ARG_CHECK(cfg->mode == STY_PF_MODE_REF || cfg->mode == STY_PF_MODE_SCREEN, "unknown render mode %d",
                  cfg->mode);
    if (cfg->mode == STY_PF_MODE_REF) {
        STY_ARG_CHECK(cfg->n_radius_scale >= 1 && cfg->n_radius_scale <= 16 && cfg->n_reuse >= 1 && cfg->n_reuse <= 16,
                      "radius_scale and reuse need 1..16 entries");
    } else {
        const uint32_t b = cfg->branch;
        STY_ARG_CHECK(b == 1 || b == 2 || b == 4 || b == 8 || b == 16, "SCREEN mode: branch must be 1, 2, 4, 8 or 16");
        STY_ARG_CHECK(cfg->screen_style < (int32_t)n_programs, "SCREEN mode: screen_style %d >= %u programs",
                      cfg->screen_style, n_programs);
    }
    return STY_OK;
}
// the SCREEN-mode filter pass over the job's records (deepest depth first) into the job's outputs
sty_status screen_filter_job(TraceJob &job, const sty_pf_render_config *cfg, const sty_style_program *programs,
                             cudaStream_t st) {
    const sty_pf_records r = job.records(cfg->branch);
    const sty_style_program *prog = cfg->screen_style >= 0 ? &programs[cfg->screen_style] : nullptr;
    return sty_pf_screen_filter(&r, &cfg->screen, prog, job.outs, st);
}
}  // namespace

extern "C" sty_status sty_pf_render(sty_scene *scene, const sty_pf_render_config *cfg,
                                    const sty_style_program *programs, uint32_t n_programs, double *film,
                                    uint64_t *vertex_count, void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && cfg && film, "sty_pf_render: null argument");
    STY_TRY(check_render_config(cfg, programs, n_programs));
    cudaStream_t st = as_stream(stream);
    TraceJob job;
    const bool screen = cfg->mode == STY_PF_MODE_SCREEN;
    STY_TRY(job.init(scene, cfg->branch, cfg->max_depth, programs, n_programs, cfg->seed, st, 0,
                     screen ? cfg->branch : 0u));
    const uint32_t n = job.n, D = job.D, npx = job.npx;
    sty_status s = STY_OK;
    if (screen) {
        STY_TRY(job.init_records(nullptr));
        const sty_camera &cam = scene_camera(scene);
        for (uint32_t rep = 0; rep < cfg->repeats && s == STY_OK; rep++) {
            s = job.trace(st);
            if (s == STY_OK) s = screen_filter_job(job, cfg, programs, st);
            if (s == STY_OK)
                s = sty_film_accumulate(job.out(0), (int32_t)cam.width, (int32_t)cam.height, (int32_t)cfg->branch,
                                        1.0 / cfg->repeats, film, st);
        }
    } else {
        RenderCache &rc = *job.cache;
        if (!rc.ctx || rc.ctx_cap < n) {
            if (rc.ctx) sty_pf_ref_destroy(rc.ctx);
            rc.ctx = nullptr;
            rc.ctx_cap = 0;
            STY_TRY(sty_pf_ref_create(n, 1u << 26, &rc.ctx));
            rc.ctx_cap = n;
        }
        sty_pf_ref_ctx *ctx = rc.ctx;
        const auto &mh = scene_materials(scene);
        std::vector<sty_pf_material> pm(mh.size());
        for (size_t i = 0; i < mh.size(); i++) {
            pm[i].kind = mh[i].kind;
            for (int c = 0; c < 3; c++) pm[i].albedo[c] = mh[i].albedo[c];
            pm[i].alpha = mh[i].alpha;
            for (int c = 0; c < 4; c++) pm[i].style[c] = mh[i].style[c];
            pm[i].roughness = mh[i].roughness;
            pm[i].metallic = mh[i].metallic;
            pm[i].ior = mh[i].ior;
            pm[i].transmission = mh[i].transmission;
            pm[i].specular_ior_level = mh[i].specular_ior_level;
            pm[i].coat_weight = mh[i].coat_weight;
            pm[i].coat_roughness = mh[i].coat_roughness;
            pm[i].coat_ior = mh[i].coat_ior;
            for (int c = 0; c < 3; c++) {
                pm[i].specular_tint[c] = mh[i].specular_tint[c];
                pm[i].coat_tint[c] = mh[i].coat_tint[c];
            }
        }
        float bmin[3], bmax[3];
        for (int a = 0; a < 3; a++) {
            bmin[a] = cfg->has_scene_bounds ? cfg->scene_bounds[a] : job.bmin[a];
            bmax[a] = cfg->has_scene_bounds ? cfg->scene_bounds[3 + a] : job.bmax[a];
        }
        const float avg = ((bmax[0] - bmin[0]) + (bmax[1] - bmin[1]) + (bmax[2] - bmin[2])) / 3.0f;
        for (uint32_t rep = 0; rep < cfg->repeats && s == STY_OK; rep++) {
            s = job.trace(st);
            for (int d = (int)D - 1; d >= 0 && s == STY_OK; d--) {
                sty_pf_ref_params prm;
                memset(&prm, 0, sizeof(prm));
                prm.depth = (uint32_t)d;
                const float rs = cfg->radius_scale[std::min<uint32_t>((uint32_t)d, cfg->n_radius_scale - 1)];
                prm.radius = avg * 0.01f * rs;  // lm_path_filtering.rs:1579-1586
                prm.reuse = cfg->reuse[std::min<uint32_t>((uint32_t)d, cfg->n_reuse - 1)];
                prm.smis = cfg->smis;
                prm.cluster = cfg->cluster;
                prm.disable_flag_check = cfg->disable_flag_check;
                prm.no_first_hit_stylization = cfg->no_first_hit_stylization;
                prm.table_size = 1u << 26;
                for (int a = 0; a < 3; a++) {
                    prm.pmin[a] = bmin[a];
                    prm.pmax[a] = bmax[a];
                }
                prm.max_cluster_rounds = 64;
                const float *next = (uint32_t)d + 1 < D ? job.out((uint32_t)d + 1) : nullptr;
                s = sty_pf_ref_filter(ctx, &job.vin[d], next, &prm, pm.data(), (uint32_t)pm.size(), programs,
                                      n_programs, job.rng, job.out((uint32_t)d), nullptr, nullptr, stream);
            }
            if (s == STY_OK) {
                k_splat<<<(npx + 255) / 256, 256, 0, st>>>(npx, cfg->branch, job.out(0), job.vo[0], job.sv.materials,
                                                           job.dprog, n_programs, cfg->no_first_hit_stylization,
                                                           1.0 / cfg->repeats, film);
                s = check_launch("k_splat");
            }
        }
    }
    if (s == STY_OK && vertex_count) {
        unsigned long long h = 0;
        s = check_cuda(cudaMemcpyAsync(&h, job.vc, 8, cudaMemcpyDeviceToHost, st), "read vertex count");
        if (s == STY_OK) s = check_cuda(cudaStreamSynchronize(st), "sync render");
        *vertex_count = h;
    }
    if (s == STY_OK) s = check_cuda(cudaStreamSynchronize(st), "sync render");
    return s;
}

extern "C" sty_status sty_pf_trace_records(sty_scene *scene, const sty_pf_render_config *cfg,
                                           const sty_style_program *programs, uint32_t n_programs,
                                           const sty_pf_records_out *records, uint64_t *vertex_count, void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && cfg && records, "sty_pf_trace_records: null argument");
    STY_TRY(check_render_config(cfg, programs, n_programs));
    STY_ARG_CHECK(cfg->mode == STY_PF_MODE_SCREEN, "sty_pf_trace_records: the config is not a SCREEN-mode render");
    for (int a = 0; a < 3; a++)
        STY_ARG_CHECK(records->pos[a] && records->nrm[a] && records->rad[a] && records->thr[a],
                      "sty_pf_trace_records: null record plane");
    STY_ARG_CHECK(records->valid, "sty_pf_trace_records: null valid plane");
    cudaStream_t st = as_stream(stream);
    TraceJob job;
    STY_TRY(job.init(scene, cfg->branch, cfg->max_depth, programs, n_programs, cfg->seed, st, 0, cfg->branch));
    STY_TRY(job.init_records(records));
    STY_TRY(job.trace(st));
    if (vertex_count) {
        unsigned long long h = 0;
        STY_TRY(check_cuda(cudaMemcpyAsync(&h, job.vc, 8, cudaMemcpyDeviceToHost, st), "read vertex count"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync trace"));
        *vertex_count = h;
    }
    return STY_OK;
}

namespace sty {
namespace {
__global__ void k_camera_rays(CamArgs cam, uint32_t n, StdRngKey key, float *rays) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sty_pcg32 g;  // Pcg32::new_seq_offset(i, seed_i), as k_rng_init
    g.state = 0;
    g.inc = ((uint64_t)i << 1) | 1ull;
    pcg_next(g);
    g.state += std_rng_u64(key.k, i);
    pcg_next(g);
    F3 o, d;
    camera_ray(cam, i % (cam.W * cam.H), g, &o, &d);
    float *r = rays + 8 * (size_t)i;
    r[0] = o.x; r[1] = o.y; r[2] = o.z;
    r[3] = d.x; r[4] = d.y; r[5] = d.z;
    r[6] = 0.0f; r[7] = 1e20f;
}
}  // namespace
}  // namespace sty

extern "C" sty_status sty_scene_camera_rays(sty_scene *scene, uint32_t branch, uint64_t seed, float *rays,
                                            void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && rays, "sty_scene_camera_rays: null argument");
    const sty_camera &cam = scene_camera(scene);
    const uint64_t n = (uint64_t)cam.width * cam.height * branch;
    STY_ARG_CHECK(branch >= 1 && n < (1ull << 31), "sty_scene_camera_rays: bad branch %u", branch);
    k_camera_rays<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(make_camera(cam), (uint32_t)n,
                                                                            std_rng_key_of(seed), rays);
    return check_launch("k_camera_rays");
}

extern "C" sty_status sty_nrc_samples(sty_scene *scene, uint32_t mode, uint32_t layout, uint32_t spp, uint32_t max_depth,
                                      uint64_t seed,
                                      float *inputs, float *targets, uint64_t capacity, uint64_t *count_out,
                                      void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && inputs && targets && count_out, "sty_nrc_samples: null argument");
    STY_ARG_CHECK(mode == STY_NRC_SAMPLES_TRAIN || mode == STY_NRC_SAMPLES_QUERY, "unknown mode");
    STY_ARG_CHECK(layout == STY_NRC_ROWS_REF || layout == STY_NRC_ROWS_SPHERICAL, "unknown row layout");
    STY_ARG_CHECK(spp >= 1 && max_depth <= 30, "bad spp / max_depth");
    cudaStream_t st = as_stream(stream);
    TraceJob job;
    STY_TRY(job.init(scene, spp, mode == STY_NRC_SAMPLES_QUERY ? 0u : max_depth, nullptr, 0, seed, st));
    STY_ARG_CHECK(mode == STY_NRC_SAMPLES_TRAIN || capacity >= job.n,
                  "query mode writes %u rows; capacity %llu is too small", job.n, (unsigned long long)capacity);
    FeatArgs fa;
    for (int a = 0; a < 3; a++) {
        fa.bmin[a] = job.bmin[a];
        fa.bext[a] = std::max(job.bmax[a] - job.bmin[a], 1e-6f);
    }
    fa.max_depth = max_depth;
    fa.layout = layout;
    fa.dims = layout == STY_NRC_ROWS_SPHERICAL ? 11 : 20 + max_depth;
    STY_TRY(job.trace(st));
    const unsigned nb = (job.n + 255) / 256;
    if (mode == STY_NRC_SAMPLES_QUERY) {
        k_nrc_query_rows<<<nb, 256, 0, st>>>(job.sv, fa, job.n, job.vo[0], inputs, targets);
        STY_TRY(check_launch("k_nrc_query_rows"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync samples"));
        *count_out = job.n;
        return STY_OK;
    }
    for (int d = (int)job.D - 1; d >= 0; d--) {
        k_self_radiance<<<nb, 256, 0, st>>>(job.sv, job.n, job.vo[d], (uint32_t)d + 1 < job.D ? job.out(d + 1) : nullptr,
                                            job.out(d));
        STY_TRY(check_launch("k_self_radiance"));
    }
    unsigned long long *cnt = (unsigned long long *)job.alloc(kRowCount, 8, "alloc row counter");
    uint32_t *idx = (uint32_t *)job.alloc(kRowIndex, (size_t)job.n * 4, "alloc row index");
    size_t tmp_bytes = 0;
    STY_TRY(job.s);
    STY_TRY(check_cuda(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, (const uint32_t *)job.vo[0].active, idx,
                                                      (int)job.n, st),
                       "scan size"));
    void *tmp = job.alloc(kScanTmp, tmp_bytes, "alloc scan scratch");
    STY_TRY(job.s);
    STY_TRY(check_cuda(cudaMemsetAsync(cnt, 0, 8, st), "zero rows"));
    for (uint32_t d = 0; d < job.D; d++) {
        const uint32_t *act = (const uint32_t *)job.vo[d].active;  // 0 / 1 flags
        STY_TRY(check_cuda(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, act, idx, (int)job.n, st), "scan rows"));
        k_nrc_train_rows<<<nb, 256, 0, st>>>(job.sv, fa, job.n, d, job.vo[d], job.out(d), idx, cnt, inputs, targets,
                                             capacity);
        STY_TRY(check_launch("k_nrc_train_rows"));
        k_advance_rows<<<1, 1, 0, st>>>(job.n, idx, job.vo[d].active, cnt);
        STY_TRY(check_launch("k_advance_rows"));
    }
    unsigned long long h = 0;
    STY_TRY(check_cuda(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, st), "read rows"));
    STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync samples"));
    *count_out = h < capacity ? h : capacity;
    return STY_OK;
}

namespace {
// The cache's feature rows for this scene (position normalised to its bounds, the cache's layout)
FeatArgs feat_args(sty_scene *scene, uint32_t in_dims, uint32_t max_depth) {
    FeatArgs fa;
    float bmin[3], bmax[3];
    scene_bounds(scene, bmin, bmax);
    for (int a = 0; a < 3; a++) {
        fa.bmin[a] = bmin[a];
        fa.bext[a] = std::max(bmax[a] - bmin[a], 1e-6f);
    }
    fa.max_depth = max_depth;
    fa.layout = in_dims == 11 ? STY_NRC_ROWS_SPHERICAL : STY_NRC_ROWS_REF;
    fa.dims = in_dims;
    return fa;
}

// The NL-NRC training loop (NRCPathTracer::render's training iterations, nrc_pt.rs:1519-1690): per
// iteration `n` paths from pixels drawn from their own Pcg32 streams (:1394), traced to max_depth;
// the cache (training weights) predicts the radiance at every vertex of depth >= 1, styled at that
// depth unless the cache learns styled radiance; each vertex of depth >= the training level gets
// the target Le + NEE + f L_next mis / pdf with L_next that prediction; the rows train the cache.
sty_status nrc_train_loop(sty_scene *scene, sty_nrc *nrc, const sty_nrc_render_config *cfg,
                          const sty_style_program *programs, uint32_t n_programs, const FeatArgs &fa, uint32_t n,
                          cudaStream_t st, void *stream, sty_nrc_render_stats &acc) {
    const uint32_t D = cfg->max_depth;
    const uint32_t npx = scene_camera(scene).width * scene_camera(scene).height;
    for (uint32_t it = 0; it < cfg->training_iters; it++) {
        TraceJob job;
        STY_TRY(job.init(scene, 1, D, programs, n_programs, cfg->seed * 0x9e3779b97f4a7c15ull + it, st, n));
        job.ca.random_px = 1;
        RenderCache &rc = *job.cache;
        const size_t rows = (size_t)D * n;
        float *qin = (float *)job.alloc(kQueryIn, std::max<size_t>(rows, npx) * fa.dims * 4, "alloc query rows");
        float *qpred = (float *)job.alloc(kQueryPred, std::max<size_t>(rows, npx) * 3 * 4, "alloc predictions");
        float *qscr = (float *)job.alloc(kQueryScratch, std::max<size_t>(rows, npx) * 3 * 4, "alloc query scratch");
        float *tgt = (float *)job.alloc(kTargets, (size_t)(D + 1) * 3 * n * 4, "alloc targets");
        float *rin = (float *)job.alloc(kRowsIn, (size_t)(D + 1) * n * fa.dims * 4, "alloc training rows");
        float *rtg = (float *)job.alloc(kRowsTgt, (size_t)(D + 1) * n * 3 * 4, "alloc training targets");
        unsigned long long *cnt = (unsigned long long *)job.alloc(kRowCount, 8, "alloc row counter");
        uint32_t *idx = (uint32_t *)job.alloc(kRowIndex, (size_t)n * 4, "alloc row index");
        STY_TRY(job.s);
        (void)rc;
        STY_TRY(job.trace(st));
        const unsigned nb = (n + 255) / 256;
        // predictions (training weights) at depths 1..D
        for (uint32_t d = 1; d <= D; d++) {
            k_nrc_query_rows<<<nb, 256, 0, st>>>(job.sv, fa, n, job.vo[d], qin + (size_t)(d - 1) * n * fa.dims,
                                                 qscr + (size_t)(d - 1) * n * 3, d);
            STY_TRY(check_launch("k_nrc_query_rows"));
        }
        STY_TRY(sty_nrc_train_inference(nrc, rows, qin, qpred, stream));
        acc.inference_queries += rows;
        for (uint32_t d = 1; d <= D; d++) {
            k_nrc_style_pred<<<nb, 256, 0, st>>>(job.sv, n, job.vo[d], qpred + (size_t)(d - 1) * n * 3, job.dprog,
                                                 n_programs, d, cfg->learn_stylized_radiance ? 0 : 1, job.out(d));
            STY_TRY(check_launch("k_nrc_style_pred"));
        }
        // targets: Le + NEE + continuation with the styled prediction at the next vertex
        for (uint32_t d = 0; d <= D; d++) {
            k_self_radiance<<<nb, 256, 0, st>>>(job.sv, n, job.vo[d], d < D ? job.out(d + 1) : nullptr,
                                                tgt + (size_t)d * 3 * n);
            STY_TRY(check_launch("k_self_radiance"));
        }
        k_finite_targets<<<(unsigned)(((size_t)(D + 1) * 3 * n + 255) / 256), 256, 0, st>>>((size_t)(D + 1) * 3 * n,
                                                                                          tgt);
        STY_TRY(check_launch("k_finite_targets"));
        // rows of the depths >= the training level, depth-major in path order
        const uint32_t level =
            cfg->per_level_training ? (it / cfg->per_level_training >= D ? 0u : D - it / cfg->per_level_training) : 0u;
        size_t tmp_bytes = 0;
        STY_TRY(check_cuda(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, (const uint32_t *)job.vo[0].active, idx,
                                                          (int)n, st),
                           "scan size"));
        void *tmp = job.alloc(kScanTmp, tmp_bytes, "alloc scan scratch");
        STY_TRY(job.s);
        STY_TRY(check_cuda(cudaMemsetAsync(cnt, 0, 8, st), "zero rows"));
        for (uint32_t d = level; d <= D; d++) {
            STY_TRY(check_cuda(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, (const uint32_t *)job.vo[d].active, idx,
                                                              (int)n, st),
                               "scan rows"));
            k_nrc_train_rows<<<nb, 256, 0, st>>>(job.sv, fa, n, d, job.vo[d], tgt + (size_t)d * 3 * n, idx, cnt, rin,
                                                 rtg, (uint64_t)(D + 1) * n);
            STY_TRY(check_launch("k_nrc_train_rows"));
            k_advance_rows<<<1, 1, 0, st>>>(n, idx, job.vo[d].active, cnt);
            STY_TRY(check_launch("k_advance_rows"));
        }
        unsigned long long h = 0;
        STY_TRY(check_cuda(cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, st), "read rows"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync rows"));
        if (h) {
            const bool last = it + 1 == cfg->training_iters;
            STY_TRY(sty_nrc_train(nrc, h, cfg->batches_per_iter, rin, rtg, last ? &acc.last_loss : nullptr, stream));
            acc.training_rows += h;
        }
    }
    return STY_OK;
}
}  // namespace

extern "C" sty_status sty_nrc_render(sty_scene *scene, sty_nrc *nrc, const sty_nrc_render_config *cfg,
                                     const sty_style_program *programs, uint32_t n_programs, double *film,
                                     sty_nrc_render_stats *stats, void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && nrc && cfg && film, "sty_nrc_render: null argument");
    STY_ARG_CHECK(cfg->max_depth >= 1 && cfg->max_depth <= 30 && cfg->repeats >= 1 && cfg->batches_per_iter >= 1,
                  "bad max_depth / repeats / batches_per_iter");
    STY_ARG_CHECK(programs || n_programs == 0, "null programs");
    STY_ARG_CHECK(n_programs <= 64, "at most 64 style programs");
    const uint32_t in_dims = nrc_input_dims(nrc);
    STY_ARG_CHECK(in_dims == 11 || in_dims == 20 + cfg->max_depth,
                  "the cache must take 11-input rows (STY_NRC_ROWS_SPHERICAL) or 20 + max_depth (STY_NRC_ROWS_REF)");
    cudaStream_t st = as_stream(stream);
    const sty_camera &cam = scene_camera(scene);
    const uint32_t npx = cam.width * cam.height, D = cfg->max_depth;
    uint64_t tp = cfg->training_paths;
    if (!tp) tp = (uint64_t)cfg->batches_per_iter * nrc_batch_size(nrc) / (D + 1);
    tp = std::min<uint64_t>(std::max<uint64_t>(tp, 1), npx);
    STY_ARG_CHECK(tp * (D + 1) < (1ull << 31), "too many training rows");
    const uint32_t n = (uint32_t)tp;
    sty_nrc_render_stats acc = {0, 0, 0.0f, 0};

    const FeatArgs fa = feat_args(scene, in_dims, D);
    // ---- training
    STY_TRY(nrc_train_loop(scene, nrc, cfg, programs, n_programs, fa, n, st, stream, acc));
    // ---- rendering
    const int style0 = cfg->no_first_hit_stylization ? 0 : 1;
    const int stylize_pred = cfg->learn_stylized_radiance ? 0 : 1;
    for (uint32_t r = 0; r < cfg->repeats; r++) {
        TraceJob job;
        const uint64_t rseed = cfg->seed * 0x9e3779b97f4a7c15ull + 0x5bd1e995ull + r;
        const uint32_t fg = cfg->final_gather;
        if (fg) job.split_rough = 0.05f;  // denoising roughness above which a path splits (:372)
        STY_TRY(job.init(scene, 1, fg ? D : 0, programs, n_programs, rseed, st));
        float *qin = (float *)job.alloc(kQueryIn, std::max<size_t>((size_t)D * n, npx) * fa.dims * 4, "alloc query rows");
        float *qpred = (float *)job.alloc(kQueryPred, std::max<size_t>((size_t)D * n, npx) * 3 * 4, "alloc predictions");
        float *qscr = (float *)job.alloc(kQueryScratch, std::max<size_t>((size_t)D * n, npx) * 3 * 4, "alloc scratch");
        STY_TRY(job.s);
        STY_TRY(job.trace(st));
        const unsigned nb = (npx + 255) / 256;
        if (!fg) {
            // the cache at each pixel's first hit (kernel_inference_stage_gathering, depth 0)
            k_nrc_query_rows<<<nb, 256, 0, st>>>(job.sv, fa, npx, job.vo[0], qin, qscr);
            STY_TRY(check_launch("k_nrc_query_rows"));
            STY_TRY(sty_nrc_inference(nrc, npx, qin, qpred, stream));
            acc.inference_queries += npx;
            k_nrc_splat_pred<<<nb, 256, 0, st>>>(npx, job.vo[0], qpred, job.sv.materials, job.dprog, n_programs,
                                                 cfg->no_first_hit_stylization, 1.0 / cfg->repeats, film);
            STY_TRY(check_launch("k_nrc_splat_pred"));
            continue;
        }
        // final gathering: per-path planes of the split vertex, accumulators, gather scratch
        constexpr size_t kFgPlanes = 31;  // split vertex 15, accumulators 7, gather scratch 9
        float *fgb = (float *)job.alloc(kFinalGather, kFgPlanes * npx * 4, "alloc final gather");
        STY_TRY(job.s);
        SplitPlanes sp;
        float *acc_direct, *acc_ind, *ngath, *thr, *gmis;
        uint32_t *gmat, *gflags;
        float *gpos;
        {
            int k = 0;
            auto pl = [&]() { return fgb + (size_t)(k++) * npx; };
            for (int a = 0; a < 3; a++) sp.p[a] = pl();
            for (int a = 0; a < 3; a++) sp.wo[a] = pl();
            for (int a = 0; a < 3; a++) sp.ns[a] = pl();
            for (int a = 0; a < 3; a++) sp.ng[a] = pl();
            sp.material = (uint32_t *)pl();
            sp.flags = (uint32_t *)pl();
            sp.prim = (uint32_t *)pl();
            acc_direct = pl();
            pl();
            pl();
            acc_ind = pl();
            pl();
            pl();
            ngath = pl();
            thr = pl();
            pl();
            pl();
            gmis = pl();
            gmat = (uint32_t *)pl();
            gflags = (uint32_t *)pl();
            gpos = pl();
            pl();
            pl();
            if ((size_t)k != kFgPlanes) {
                set_error("final gather planes: %d carved, %zu allocated", k, kFgPlanes);
                return STY_ERR_ARG;
            }
        }
        STY_TRY(check_cuda(cudaMemsetAsync(acc_direct, 0, (size_t)7 * npx * 4, st), "zero gather accumulators"));
        for (uint32_t d = 0; d <= D; d++) {
            k_split_collect<<<nb, 256, 0, st>>>(npx, d, job.vo[d], job.ps.split, job.ps.exclude, sp);
            STY_TRY(check_launch("k_split_collect"));
        }
        for (uint32_t it = 0; it < fg; it++) {
            k_fg_step<<<nb, 256, 0, st>>>(job.sv, fa, npx, job.ps.split, sp, job.rng, job.dprog, n_programs, qin, thr, gmis,
                                          gmat, gflags, gpos, acc_direct);
            STY_TRY(check_launch("k_fg_step"));
            STY_TRY(sty_nrc_inference(nrc, npx, qin, qpred, stream));
            acc.inference_queries += npx;
            k_fg_accumulate<<<nb, 256, 0, st>>>(job.sv, npx, job.ps.split, qpred, thr, gmis, gmat, gflags, gpos,
                                                job.dprog, n_programs, stylize_pred, acc_ind, ngath);
            STY_TRY(check_launch("k_fg_accumulate"));
        }
        for (int d = (int)D; d >= 0; d--) {
            const int sty_d = stylize_pred && (d > 0 || style0);
            k_fg_sweep<<<nb, 256, 0, st>>>(job.sv, npx, (uint32_t)d, job.vo[d], d < (int)D ? job.out(d + 1) : nullptr,
                                           job.ps.split, acc_direct, acc_ind, ngath, job.dprog, n_programs, sty_d,
                                           job.out(d));
            STY_TRY(check_launch("k_fg_sweep"));
        }
        k_fg_splat<<<nb, 256, 0, st>>>(npx, job.vo[0].active, job.out(0), 1.0 / cfg->repeats, film);
        STY_TRY(check_launch("k_fg_splat"));
    }
    STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync nrc render"));
    if (stats) *stats = acc;
    return STY_OK;
}

// NL-PF with the cache at the path ends (sty_pf_nrc_render): the cache trained by the NL-NRC loop,
// then per repeat a SCREEN-mode trace to cache_depth, the cache's EMA prediction at the depth-K
// vertices (styled at K) as out_K, the screen filter on depths K - 1 .. 0 and the splat.
extern "C" sty_status sty_pf_nrc_render(sty_scene *scene, sty_nrc *nrc, const sty_pf_nrc_config *cfg,
                                        const sty_style_program *programs, uint32_t n_programs, double *film,
                                        sty_nrc_render_stats *stats, void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && nrc && cfg && film, "sty_pf_nrc_render: null argument");
    const sty_pf_render_config &pf = cfg->pf;
    const sty_nrc_render_config &nc = cfg->nrc;
    STY_ARG_CHECK(pf.mode == STY_PF_MODE_SCREEN, "sty_pf_nrc_render: pf.mode must be STY_PF_MODE_SCREEN");
    STY_TRY(check_render_config(&pf, programs, n_programs));
    const uint32_t K = cfg->cache_depth, D = nc.max_depth;
    STY_ARG_CHECK(D >= 1 && D <= 30 && nc.batches_per_iter >= 1, "bad nrc.max_depth / batches_per_iter");
    STY_ARG_CHECK(K >= 1 && K <= D, "cache_depth %u must be in [1, nrc.max_depth = %u]", K, D);
    const uint32_t in_dims = nrc_input_dims(nrc);
    STY_ARG_CHECK(in_dims == 11 || in_dims == 20 + D,
                  "the cache must take 11-input rows (STY_NRC_ROWS_SPHERICAL) or 20 + nrc.max_depth (STY_NRC_ROWS_REF)");
    cudaStream_t st = as_stream(stream);
    const sty_camera &cam = scene_camera(scene);
    const uint32_t npx = cam.width * cam.height;
    uint64_t tp = nc.training_paths;
    if (!tp) tp = (uint64_t)nc.batches_per_iter * nrc_batch_size(nrc) / (D + 1);
    tp = std::min<uint64_t>(std::max<uint64_t>(tp, 1), npx);
    STY_ARG_CHECK(tp * (D + 1) < (1ull << 31), "too many training rows");
    sty_nrc_render_stats acc = {0, 0, 0.0f, 0};
    const FeatArgs fa = feat_args(scene, in_dims, D);
    STY_TRY(nrc_train_loop(scene, nrc, &nc, programs, n_programs, fa, (uint32_t)tp, st, stream, acc));
    const sty_style_program *prog = pf.screen_style >= 0 ? &programs[pf.screen_style] : nullptr;
    const int stylize_pred = nc.learn_stylized_radiance ? 0 : 1;
    TraceJob job;
    STY_TRY(job.init(scene, pf.branch, K, programs, n_programs, pf.seed, st, 0, pf.branch));
    STY_TRY(job.init_records(nullptr));
    const uint32_t n = job.n;
    float *qin = (float *)job.alloc(kQueryIn, (size_t)n * fa.dims * 4, "alloc query rows");
    float *qpred = (float *)job.alloc(kQueryPred, (size_t)n * 3 * 4, "alloc predictions");
    float *qscr = (float *)job.alloc(kQueryScratch, (size_t)n * 3 * 4, "alloc query scratch");
    STY_TRY(job.s);
    const sty_pf_records rec = job.records(pf.branch);
    const unsigned nb = (n + 255) / 256;
    for (uint32_t r = 0; r < pf.repeats; r++) {
        STY_TRY(job.trace(st));
        k_nrc_query_rows<<<nb, 256, 0, st>>>(job.sv, fa, n, job.vo[K], qin, qscr, K);
        STY_TRY(check_launch("k_nrc_query_rows"));
        STY_TRY(sty_nrc_inference(nrc, n, qin, qpred, stream));
        acc.inference_queries += n;
        k_nrc_style_pred<<<nb, 256, 0, st>>>(job.sv, n, job.vo[K], qpred, job.dprog, n_programs, K, stylize_pred,
                                             job.out(K));
        STY_TRY(check_launch("k_nrc_style_pred"));
        for (int d = (int)K - 1; d >= 0; d--)
            STY_TRY(sty_pf_screen_filter_depth(&rec, (uint32_t)d, &pf.screen, prog, job.out((uint32_t)d + 1),
                                               job.out((uint32_t)d), nullptr, stream));
        STY_TRY(sty_film_accumulate(job.out(0), (int32_t)cam.width, (int32_t)cam.height, (int32_t)pf.branch,
                                    1.0 / pf.repeats, film, st));
    }
    STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync pf nrc render"));
    if (stats) *stats = acc;
    return STY_OK;
}
