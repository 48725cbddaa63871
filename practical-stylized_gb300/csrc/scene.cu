// scene.cu -- scene object: host-side binned-SAH BVH build, device upload, closest-hit queries.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "bsdf.cuh"
#include "scene.cuh"

using namespace sty;

struct sty_scene {
    uint32_t n_tris = 0, n_materials = 0, n_lights = 0;
    sty_camera camera;
    float bmin[3], bmax[3];
    std::vector<sty_scene_material> materials_h;
    BvhNode *nodes = nullptr;
    TriGeom *tris = nullptr;
    uint32_t *tri_material = nullptr;
    float *tri_normal = nullptr, *tri_area = nullptr, *tri_pos = nullptr;
    sty_scene_material *materials = nullptr;
    uint32_t *light_tris = nullptr;
    float *light_cdf = nullptr;
    void *render_cache = nullptr;  // device buffers of the last render, reused by the next (trace.cu)
};

namespace sty {
SceneView scene_view(const sty_scene *s) {
    SceneView v;
    v.nodes = s->nodes;
    v.tris = s->tris;
    v.tri_material = s->tri_material;
    v.tri_normal = s->tri_normal;
    v.tri_area = s->tri_area;
    v.materials = s->materials;
    v.n_tris = s->n_tris;
    v.n_materials = s->n_materials;
    v.light_tris = s->light_tris;
    v.light_cdf = s->light_cdf;
    v.n_lights = s->n_lights;
    v.tri_pos = s->tri_pos;
    v.ggx_tab = principled_table();
    v.any_closure = 0;
    for (const sty_scene_material &m : s->materials_h) v.any_closure |= bsdf::closure_kind(m.kind) ? 1u : 0u;
    return v;
}
}  // namespace sty

namespace {

struct Box {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float *p) {
        for (int a = 0; a < 3; a++) {
            mn[a] = std::min(mn[a], p[a]);
            mx[a] = std::max(mx[a], p[a]);
        }
    }
    void grow(const Box &b) {
        for (int a = 0; a < 3; a++) {
            mn[a] = std::min(mn[a], b.mn[a]);
            mx[a] = std::max(mx[a], b.mx[a]);
        }
    }
    float area() const {
        float d[3];
        for (int a = 0; a < 3; a++) d[a] = std::max(0.0f, mx[a] - mn[a]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

// Binned SAH (16 bins per axis), leaves of at most 4 triangles.
struct Builder {
    const float *pos;
    std::vector<Box> tbox;
    std::vector<float> cent;  // 3 per triangle
    std::vector<uint32_t> idx;
    std::vector<BvhNode> nodes;

    void build(uint32_t n) {
        tbox.resize(n);
        cent.resize(3 * (size_t)n);
        idx.resize(n);
        for (uint32_t i = 0; i < n; i++) {
            for (int v = 0; v < 3; v++) tbox[i].grow(pos + 9 * (size_t)i + 3 * v);
            for (int a = 0; a < 3; a++) cent[3 * (size_t)i + a] = 0.5f * (tbox[i].mn[a] + tbox[i].mx[a]);
            idx[i] = i;
        }
        nodes.reserve(2 * (size_t)n);
        nodes.push_back(BvhNode());
        subdivide(0, 0, n);
    }
    void set_bounds(BvhNode &nd, uint32_t b, uint32_t e) {
        Box bx;
        for (uint32_t i = b; i < e; i++) bx.grow(tbox[idx[i]]);
        for (int a = 0; a < 3; a++) {
            nd.bmin[a] = bx.mn[a];
            nd.bmax[a] = bx.mx[a];
        }
    }
    void subdivide(uint32_t ni, uint32_t b, uint32_t e) {
        set_bounds(nodes[ni], b, e);
        const uint32_t cnt = e - b;
        if (cnt <= 4) {
            nodes[ni].a = b;
            nodes[ni].count = cnt;
            return;
        }
        Box cb;
        for (uint32_t i = b; i < e; i++) cb.grow(&cent[3 * (size_t)idx[i]]);
        constexpr int NB = 16;
        float best = INFINITY;
        int best_axis = -1, best_bin = 0;
        for (int a = 0; a < 3; a++) {
            const float ext = cb.mx[a] - cb.mn[a];
            if (!(ext > 0.0f)) continue;
            Box bins[NB];
            uint32_t counts[NB] = {0};
            for (uint32_t i = b; i < e; i++) {
                int k = (int)((cent[3 * (size_t)idx[i] + a] - cb.mn[a]) / ext * NB);
                k = std::min(std::max(k, 0), NB - 1);
                bins[k].grow(tbox[idx[i]]);
                counts[k]++;
            }
            float la[NB], ra[NB];
            uint32_t lc[NB], rc[NB];
            Box acc;
            uint32_t c = 0;
            for (int k = 0; k < NB; k++) {
                acc.grow(bins[k]);
                c += counts[k];
                la[k] = acc.area();
                lc[k] = c;
            }
            acc = Box();
            c = 0;
            for (int k = NB - 1; k >= 0; k--) {
                acc.grow(bins[k]);
                c += counts[k];
                ra[k] = acc.area();
                rc[k] = c;
            }
            for (int k = 0; k < NB - 1; k++) {
                if (lc[k] == 0 || rc[k + 1] == 0) continue;
                const float cost = la[k] * lc[k] + ra[k + 1] * rc[k + 1];
                if (cost < best) {
                    best = cost;
                    best_axis = a;
                    best_bin = k;
                }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = b + cnt / 2;  // degenerate centroids: split by index
        } else {
            const float ext = cb.mx[best_axis] - cb.mn[best_axis];
            auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](uint32_t t) {
                int k = (int)((cent[3 * (size_t)t + best_axis] - cb.mn[best_axis]) / ext * NB);
                k = std::min(std::max(k, 0), NB - 1);
                return k <= best_bin;
            });
            mid = (uint32_t)(it - idx.begin());
            if (mid == b || mid == e) mid = b + cnt / 2;
        }
        const uint32_t l = (uint32_t)nodes.size();
        nodes.push_back(BvhNode());
        nodes.push_back(BvhNode());
        nodes[ni].a = l;
        nodes[ni].count = 0;
        subdivide(l, b, mid);
        subdivide(l + 1, mid, e);
    }
};

void free_scene(sty_scene *s) {
    render_cache_free(s->render_cache);
    void *ptrs[] = {s->nodes, s->tris, s->tri_material, s->tri_normal, s->tri_area,
                    s->tri_pos, s->materials, s->light_tris, s->light_cdf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete s;
}

__global__ void k_closest(SceneView s, const float *rays, uint64_t n, uint32_t *prim, float *t, float *bary) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *r = rays + 8 * i;
    const float o[3] = {r[0], r[1], r[2]}, d[3] = {r[3], r[4], r[5]};
    const Hit h = trace_closest(s, o, d, r[6], r[7], 0xffffffffu);
    prim[i] = h.prim;
    if (t) t[i] = h.t;
    if (bary) {
        bary[2 * i] = h.b1;
        bary[2 * i + 1] = h.b2;
    }
}

}  // namespace

extern "C" {

sty_status sty_scene_create(const float *pos, const uint32_t *tmat, uint32_t n, const sty_scene_material *mats,
                            uint32_t nm, const sty_camera *cam, sty_scene **out) {
    clear_error();
    STY_ARG_CHECK(pos && tmat && mats && cam && out, "sty_scene_create: null argument");
    STY_ARG_CHECK(n > 0 && nm > 0, "empty scene");
    STY_ARG_CHECK(cam->width > 0 && cam->height > 0 && cam->fov_y > 0.0f && cam->fov_y < 180.0f, "bad camera");
    STY_ARG_CHECK(cam->filter == STY_FILTER_BOX || cam->filter == STY_FILTER_GAUSSIAN, "unknown pixel filter %d",
                  cam->filter);
    STY_ARG_CHECK(cam->filter_radius >= 0.0f && cam->filter_radius < 1e6f, "bad pixel filter radius");
    for (uint32_t i = 0; i < n; i++) STY_ARG_CHECK(tmat[i] < nm, "triangle %u has material %u >= %u", i, tmat[i], nm);
    for (uint32_t i = 0; i < nm; i++)
        STY_ARG_CHECK(mats[i].kind == STY_MAT_DIFFUSE || mats[i].kind == STY_MAT_GGX ||
                          bsdf::closure_kind(mats[i].kind),
                      "material %u: unknown kind", i);
    for (uint32_t i = 0; i < nm; i++)
        STY_ARG_CHECK(!bsdf::closure_kind(mats[i].kind) ||
                          (mats[i].ior > 0.0f && mats[i].coat_ior > 0.0f && mats[i].roughness >= 0.0f &&
                           mats[i].coat_roughness >= 0.0f),
                      "material %u: principled / glass ior / coat_ior must be > 0 and roughness >= 0", i);
    sty_scene *s = new sty_scene();
    s->n_tris = n;
    s->n_materials = nm;
    s->camera = *cam;
    s->materials_h.assign(mats, mats + nm);
    Builder b;
    b.pos = pos;
    b.build(n);
    Box all;
    for (uint32_t i = 0; i < n; i++) all.grow(b.tbox[i]);
    for (int a = 0; a < 3; a++) {
        s->bmin[a] = all.mn[a];
        s->bmax[a] = all.mx[a];
    }
    std::vector<TriGeom> tg(n);
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t i = b.idx[k];
        const float *p = pos + 9 * (size_t)i;
        uint32_t bits = i;
        float w;
        memcpy(&w, &bits, 4);
        tg[k].v0 = make_float4(p[0], p[1], p[2], w);
        tg[k].v1 = make_float4(p[3], p[4], p[5], 0.0f);
        tg[k].v2 = make_float4(p[6], p[7], p[8], 0.0f);
    }
    std::vector<float> nrm(3 * (size_t)n), area(n);
    std::vector<uint32_t> lt;
    std::vector<double> lw;
    for (uint32_t i = 0; i < n; i++) {
        const float *p = pos + 9 * (size_t)i;
        const double e1[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};
        const double e2[3] = {(double)p[6] - p[0], (double)p[7] - p[1], (double)p[8] - p[2]};
        const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        area[i] = (float)(0.5 * l);
        for (int a = 0; a < 3; a++) nrm[3 * (size_t)i + a] = l > 0 ? (float)(c[a] / l) : 0.0f;
        const float *em = mats[tmat[i]].emission;
        const double lum = 0.2126 * em[0] + 0.7152 * em[1] + 0.0722 * em[2];
        if (lum > 0.0 && area[i] > 0.0f) {
            lt.push_back(i);
            lw.push_back(lum * area[i]);
        }
    }
    std::vector<float> cdf(lt.size() + 1, 0.0f);
    double tot = 0;
    for (double w : lw) tot += w;
    double acc = 0;
    for (size_t k = 0; k < lw.size(); k++) {
        acc += lw[k];
        cdf[k + 1] = (float)(acc / tot);
    }
    if (!lt.empty()) cdf.back() = 1.0f;
    s->n_lights = (uint32_t)lt.size();
    sty_status st = STY_OK;
    auto up = [&](void **dst, const void *src, size_t bytes, const char *what) {
        if (st != STY_OK || bytes == 0) return;
        st = check_cuda(cudaMalloc(dst, bytes), what);
        if (st == STY_OK) st = check_cuda(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), what);
    };
    up((void **)&s->nodes, b.nodes.data(), b.nodes.size() * sizeof(BvhNode), "upload bvh");
    up((void **)&s->tris, tg.data(), tg.size() * sizeof(TriGeom), "upload triangles");
    up((void **)&s->tri_material, tmat, n * 4, "upload materials ids");
    up((void **)&s->tri_normal, nrm.data(), nrm.size() * 4, "upload normals");
    up((void **)&s->tri_area, area.data(), area.size() * 4, "upload areas");
    up((void **)&s->tri_pos, pos, 9 * (size_t)n * 4, "upload positions");
    up((void **)&s->materials, mats, nm * sizeof(sty_scene_material), "upload material table");
    up((void **)&s->light_tris, lt.data(), lt.size() * 4, "upload lights");
    up((void **)&s->light_cdf, cdf.data(), cdf.size() * 4, "upload light cdf");
    if (st != STY_OK) {
        free_scene(s);
        return st;
    }
    *out = s;
    return STY_OK;
}

sty_status sty_scene_destroy(sty_scene *s) {
    clear_error();
    if (s) free_scene(s);
    return STY_OK;
}

sty_status sty_scene_closest_hit(sty_scene *s, const float *rays, uint64_t n, uint32_t *prim, float *t, float *bary,
                                 void *stream) {
    clear_error();
    STY_ARG_CHECK(s && rays && prim, "sty_scene_closest_hit: null argument");
    if (n == 0) return STY_OK;
    k_closest<<<(unsigned)((n + 127) / 128), 128, 0, as_stream(stream)>>>(scene_view(s), rays, n, prim, t, bary);
    return check_launch("k_closest");
}

}  // extern "C"

// accessors used by the render driver
namespace sty {
const sty_camera &scene_camera(const sty_scene *s) { return s->camera; }
void *&scene_render_cache(sty_scene *s) { return s->render_cache; }
void scene_bounds(const sty_scene *s, float mn[3], float mx[3]) {
    for (int a = 0; a < 3; a++) {
        mn[a] = s->bmin[a];
        mx[a] = s->bmax[a];
    }
}
const std::vector<sty_scene_material> &scene_materials(const sty_scene *s) { return s->materials_h; }
}  // namespace sty
