// pf_ref.cu -- reference-mode NL-PF (world-space hash grid, clustering, SMIS) for one depth.
//
// Pipeline per call (all on the caller's stream):
//   1. compact the active path slots in ascending order (cub::DeviceSelect::Flagged, stable);
//   2. bucket key per point = hash(cell) mod table (lm_path_filtering.rs:20-59);
//   3. stable radix sort of (bucket, slot) -> every bucket lists its points in ascending slot
//      order, the fixed replacement of the reference's CAS-built linked lists (:230-255);
//   4. bucket -> [start, end) table;
//   5. (cluster) deterministic clustering rounds (:533-623, :1675-1710): claim / propose / accept;
//   6. filter: one thread per active vertex (evaluate_filtered_radiance, :758-972).
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <cmath>

#include "common.cuh"
#include "style.cuh"

namespace sty {
namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr uint32_t kMaxMaterials = 256;
constexpr uint32_t kMaxPrograms = 64;
constexpr float kPi = 3.14159265358979323846f;

struct Geo {
    float pmin[3], pmax[3];
    uint32_t res[3];
    uint32_t table;
    float r;
};

struct VArgs {  // device views of sty_pf_vertices
    const int32_t *active;
    const float *p[3], *wo[3], *ns[3], *ng[3], *le[3], *mis, *dir_wi[3], *dir_l[3], *dir_pdf, *ind_wi[3], *ind_mis;
    const uint32_t *flags, *material;
    uint64_t n;
};

__device__ __forceinline__ void get_cell(const Geo &g, float px, float py, float pz, int32_t c[3]) {
    const float p[3] = {px, py, pz};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float t = __fdiv_rn(__fsub_rn(p[a], g.pmin[a]), __fsub_rn(g.pmax[a], g.pmin[a]));
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        t = __fmul_rn(t, (float)g.res[a]);
        const uint32_t u = (uint32_t)t;
        c[a] = (int32_t)min(u, g.res[a] - 1u);
    }
}
__device__ __forceinline__ uint32_t bucket_of(const Geo &g, int32_t cx, int32_t cy, int32_t cz) {
    const uint64_t h = ((uint64_t)(uint32_t)cx * 73856093ull) ^ ((uint64_t)(uint32_t)cy * 19349663ull) ^
                       ((uint64_t)(uint32_t)cz * 83492791ull);
    return (uint32_t)(h % (uint64_t)g.table);
}
// (a - b).length() in f32, no contraction
__device__ __forceinline__ float dist_f(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    float s = __fmul_rn(dx, dx);
    s = __fadd_rn(s, __fmul_rn(dy, dy));
    s = __fadd_rn(s, __fmul_rn(dz, dz));
    return __fsqrt_rn(s);
}

// 27-cell walk (:61-123): dz outer, dy, dx inner; f(u) returns false to stop.
template <class F>
__device__ __forceinline__ void walk(const Geo &g, const uint2 *__restrict__ ranges, const uint32_t *__restrict__ sorted,
                                     float qx, float qy, float qz, F &&f) {
    int32_t c[3];
    get_cell(g, qx, qy, qz, c);
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int32_t nx = c[0] + dx, ny = c[1] + dy, nz = c[2] + dz;
                if (nx < 0 || ny < 0 || nz < 0 || nx >= (int32_t)g.res[0] || ny >= (int32_t)g.res[1] ||
                    nz >= (int32_t)g.res[2])
                    continue;
                const uint2 rg = ranges[bucket_of(g, nx, ny, nz)];
                for (uint32_t k = rg.x; k < rg.y; k++)
                    if (!f(sorted[k])) return;
            }
}

__device__ __forceinline__ uint32_t pcg_next(sty_pcg32 &s) {
    const uint64_t old = s.state;
    s.state = old * 0x5851f42d4c957f2dULL + s.inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 ld3(const float *const a[3], uint32_t i) { return {a[0][i], a[1][i], a[2][i]}; }

// SurfaceClosure::check_wo_wi_valid (svm/surface/mod.rs:1699-1712)
__device__ __forceinline__ bool wo_wi_valid(V3 ns, V3 ng, V3 wo, V3 wi) {
    auto sgn = [](float x) { return x > 0.0f ? 1.0f : -1.0f; };
    const float fl = sgn(dot3(ng, ns));
    return sgn(fl * dot3(wo, ns)) * sgn(dot3(wo, ng)) > 0.0f && sgn(fl * dot3(wi, ns)) * sgn(dot3(wi, ng)) > 0.0f;
}
__device__ __forceinline__ float tr_d(float ch, float a) {  // microfacet.rs:44-57, isotropic
    const float c2 = ch * ch, s2 = fmaxf(0.0f, 1.0f - c2);
    const float tan2 = s2 / c2;
    const float e = tan2 / (a * a);
    const float inv_d = kPi * a * a * c2 * c2 * (1.0f + e) * (1.0f + e);
    if (!isfinite(tan2) || !isfinite(inv_d) || inv_d == 0.0f) return 0.0f;
    return 1.0f / inv_d;
}
__device__ __forceinline__ float tr_lambda(float cw, float a) {  // microfacet.rs:58-66
    const float c2 = cw * cw, s2 = fmaxf(0.0f, 1.0f - c2);
    const float at = fabsf(sqrtf(s2) / cw);
    const float l = (-1.0f + sqrtf(1.0f + a * a * at * at)) * 0.5f;
    return isfinite(at) ? l : 0.0f;
}
// Surface::evaluate: f*|cos_i| and pdf (diffuse.rs:17-48; mod.rs:1877-1910 with unit Fresnel)
__device__ void bsdf_eval(const sty_pf_material &m, V3 ns, V3 ng, V3 wo, V3 wi, float f[3], float *pdf) {
    f[0] = f[1] = f[2] = 0.0f;
    *pdf = 0.0f;
    if (!wo_wi_valid(ns, ng, wo, wi)) return;
    const float co = dot3(wo, ns), ci = dot3(wi, ns);
    if (m.kind == STY_MAT_DIFFUSE) {
        if (co * ci >= 0.0f) {
            *pdf = fabsf(ci) / kPi;
#pragma unroll
            for (int c = 0; c < 3; c++) f[c] = m.albedo[c] / kPi * fabsf(ci);
        }
        return;
    }
    const float a = fmaxf(m.alpha, 1e-4f);
    V3 wh = {wo.x + wi.x, wo.y + wi.y, wo.z + wi.z};
    if (dot3(wh, wo) * dot3(wi, wh) < 0.0f || (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) || ci == 0.0f ||
        co == 0.0f || !(co * ci >= 0.0f))
        return;
    const float l = sqrtf(dot3(wh, wh));
    wh = {wh.x / l, wh.y / l, wh.z / l};
    const float d = tr_d(dot3(wh, ns), a);
    const float g = 1.0f / (1.0f + tr_lambda(co, a) + tr_lambda(ci, a));
    const float g1 = 1.0f / (1.0f + tr_lambda(co, a));
    const float k = fabsf(0.25f * d * g / (ci * co)) * fabsf(ci);
#pragma unroll
    for (int c = 0; c < 3; c++) f[c] = m.albedo[c] * k;
    const float owh = fabsf(dot3(wo, wh));
    *pdf = d * g1 * owh / fabsf(co) / (4.0f * owh);
}
__device__ __forceinline__ uint32_t style_index(uint32_t flags) {  // mod.rs:72-84
    uint32_t i = 0;
    if (flags & 2u) i = 1;
    if (flags & 4u) i = 2;
    if (flags & 8u) i = 3;
    return i;
}

// ---- kernels ----------------------------------------------------------------------------------
__global__ void k_keys(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, uint32_t *keys, uint32_t *vals) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    if (i >= *num) {  // padding sorts behind every real bucket
        keys[i] = NONE;
        vals[i] = NONE;
        return;
    }
    const uint32_t s = act[i];
    int32_t c[3];
    get_cell(g, v.p[0][s], v.p[1][s], v.p[2][s], c);
    keys[i] = bucket_of(g, c[0], c[1], c[2]);
    vals[i] = s;
}
__global__ void k_ranges(const uint32_t *keys, const uint32_t *num, uint2 *ranges) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint32_t m = *num;
    if (i >= m) return;
    const uint32_t k = keys[i];
    if (i == 0 || keys[i - 1] != k) ranges[k].x = (uint32_t)i;
    if (i + 1 == m || keys[i + 1] != k) ranges[k].y = (uint32_t)i + 1;
}
// clustering: claim
__global__ void k_cl_claim_reset(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, const uint32_t *cid,
                                 uint32_t *winner) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t s = act[i];
    if (cid[s] != NONE) return;
    int32_t c[3];
    get_cell(g, v.p[0][s], v.p[1][s], v.p[2][s], c);
    winner[bucket_of(g, c[0], c[1], c[2])] = NONE;
}
__global__ void k_cl_claim_min(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, const uint32_t *cid,
                               uint32_t *winner) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t s = act[i];
    if (cid[s] != NONE) return;
    int32_t c[3];
    get_cell(g, v.p[0][s], v.p[1][s], v.p[2][s], c);
    atomicMin(&winner[bucket_of(g, c[0], c[1], c[2])], s);
}
__global__ void k_cl_claim_set(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, uint32_t *cid,
                               uint32_t *csize, const uint32_t *winner) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t s = act[i];
    if (cid[s] != NONE) return;
    int32_t c[3];
    get_cell(g, v.p[0][s], v.p[1][s], v.p[2][s], c);
    if (winner[bucket_of(g, c[0], c[1], c[2])] == s) {
        cid[s] = s;
        csize[s] = 0;
    }
}
__global__ void k_cl_propose(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, const uint2 *ranges,
                             const uint32_t *sorted, const uint32_t *cid, const uint32_t *size0, uint32_t reuse,
                             uint32_t *prop) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t s = act[i];
    if (cid[s] != NONE) return;
    const float px = v.p[0][s], py = v.p[1][s], pz = v.p[2][s];
    uint32_t pick = NONE;
    walk(g, ranges, sorted, px, py, pz, [&](uint32_t u) {
        if (dist_f(v.p[0][u], v.p[1][u], v.p[2][u], px, py, pz) <= g.r && cid[u] == u && size0[u] < reuse) {
            pick = u;
            return false;
        }
        return true;
    });
    prop[s] = pick;
}
__global__ void k_cl_accept(VArgs v, Geo g, const uint32_t *act, const uint32_t *num, const uint2 *ranges,
                            const uint32_t *sorted, uint32_t *cid, uint32_t *csize, const uint32_t *prop,
                            uint32_t reuse) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t c = act[i];
    if (cid[c] != c) return;
    uint32_t sz = csize[c];
    if (sz >= reuse) return;
    walk(g, ranges, sorted, v.p[0][c], v.p[1][c], v.p[2][c], [&](uint32_t u) {
        if (prop[u] == c && cid[u] == NONE) {  // only this thread writes cid[u] (u proposed to c only)
            cid[u] = c;
            sz++;
        }
        return sz < reuse;
    });
    csize[c] = sz;
}
__global__ void k_cl_count(const uint32_t *act, const uint32_t *num, const uint32_t *cid, uint32_t *counter) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    if (cid[act[i]] == NONE) atomicAdd(counter, 1u);
}

template <int MAXK>
__global__ void __launch_bounds__(128) k_ref_filter(VArgs v, Geo g, const uint32_t *act, const uint32_t *num,
                                                    const uint2 *ranges, const uint32_t *sorted, const uint32_t *cid,
                                                    const float *in_next, sty_pf_ref_params prm,
                                                    const sty_pf_material *mats, uint32_t n_mats,
                                                    const sty_style_program *progs, uint32_t n_progs, sty_pcg32 *rng,
                                                    float *out, uint32_t *neighbours) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= *num) return;
    const uint32_t vi = act[i];
    const uint64_t n = v.n;
    const uint32_t qs = prm.cluster ? cid[vi] : vi;
    const float qx = v.p[0][qs], qy = v.p[1][qs], qz = v.p[2][qs];
    const uint32_t my_cluster = prm.cluster ? cid[vi] : NONE;
    const uint32_t my_flags = v.flags[vi] & 15u;
    const uint32_t reuse = prm.reuse;
    uint32_t list[MAXK];
    uint32_t cnt = 0;
    sty_pcg32 st = rng[vi];
    walk(g, ranges, sorted, qx, qy, qz, [&](uint32_t u) {
        if (!(dist_f(v.p[0][u], v.p[1][u], v.p[2][u], qx, qy, qz) <= g.r)) return true;
        if (prm.cluster && cid[u] != my_cluster) return true;
        if (!prm.disable_flag_check && (v.flags[u] & 15u) != my_flags) return true;
        if (cnt < reuse) {
            list[cnt] = u;
        } else {
            const uint32_t j = pcg_next(st) % (cnt + 1);
            if (j < reuse) list[j] = u;
        }
        cnt++;
        return true;
    });
    rng[vi] = st;
    if (neighbours) neighbours[vi] = cnt;
    const uint32_t k = min(cnt, reuse);
    const sty_pf_material mv = mats[min(v.material[vi], n_mats - 1)];
    const V3 wo = ld3(v.wo, vi), ns = ld3(v.ns, vi), ng = ld3(v.ng, vi);
    float direct[3] = {0.f, 0.f, 0.f}, indirect[3] = {0.f, 0.f, 0.f};
    const float invk = 1.0f / (float)k;
    for (uint32_t t = 0; t < k; t++) {
        const uint32_t u = list[t];
        const float dpdf = v.dir_pdf[u];
        if (dpdf > 0.0f) {  // :839-863
            float f[3], pdf;
            bsdf_eval(mv, ns, ng, wo, ld3(v.dir_wi, u), f, &pdf);
            const float w = dpdf / (dpdf + pdf);
#pragma unroll
            for (int c = 0; c < 3; c++) direct[c] += f[c] * v.dir_l[c][u] * w / dpdf * invk;
        }
        const V3 wi = ld3(v.ind_wi, u);
        if (dot3(wi, wi) == 0.0f) continue;
        float f[3], pdf;
        bsdf_eval(mv, ns, ng, wo, wi, f, &pdf);
        const float mis = v.ind_mis[u];
        float reused[3];
#pragma unroll
        for (int c = 0; c < 3; c++) reused[c] = f[c] * (in_next ? in_next[c * n + u] : 0.0f) * mis;
        if (prm.smis) {  // :886-939
            float sum_pdf = 0.0f;
            for (uint32_t jj = 0; jj < k; jj++) {
                const uint32_t a = list[jj];
                const sty_pf_material ma = mats[min(v.material[a], n_mats - 1)];
                float fa[3], pa;
                bsdf_eval(ma, ld3(v.ns, a), ld3(v.ng, a), ld3(v.wo, a), wi, fa, &pa);
                sum_pdf += pa;
            }
            if (sum_pdf > 0.0f)
#pragma unroll
                for (int c = 0; c < 3; c++) indirect[c] += reused[c] / sum_pdf;
        } else if (pdf > 0.0f) {
#pragma unroll
            for (int c = 0; c < 3; c++) indirect[c] += reused[c] / pdf * invk;
        }
    }
    f3 rad = {v.le[0][vi] + direct[0] + indirect[0], v.le[1][vi] + direct[1] + indirect[1],
              v.le[2][vi] + direct[2] + indirect[2]};
    const uint32_t fl = v.flags[vi];
    if ((prm.depth > 0 || !prm.no_first_hit_stylization) && !(fl & 1u)) {
        const int32_t pi = mv.style[style_index(fl)];
        if (pi >= 0 && (uint32_t)pi < n_progs) rad = style_apply(progs[pi], prm.depth, rad);
    }
    out[vi] = rad.x;
    out[n + vi] = rad.y;
    out[2 * n + vi] = rad.z;
}

}  // namespace
}  // namespace sty

struct sty_pf_ref_ctx {
    uint64_t cap = 0;
    uint32_t table = 0;
    uint32_t *act = nullptr, *num = nullptr, *keys = nullptr, *vals = nullptr, *keys_s = nullptr, *vals_s = nullptr;
    uint2 *ranges = nullptr;
    uint32_t *cid = nullptr, *csize = nullptr, *size0 = nullptr, *prop = nullptr, *winner = nullptr;
    uint32_t *counter = nullptr;
    sty_pf_material *mats = nullptr;      // device copies of the host tables
    sty_style_program *progs = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int device = -1;
};

using namespace sty;

namespace {
void free_ctx(sty_pf_ref_ctx *c) {
    void *ptrs[] = {c->act,   c->num,    c->keys,  c->vals,    c->keys_s,  c->vals_s, c->ranges, c->cid,
                    c->csize, c->size0,  c->prop,  c->winner,  c->counter, c->mats,   c->progs,  c->tmp};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete c;
}
VArgs make_vargs(const sty_pf_vertices *v) {
    VArgs a;
    a.active = v->active;
    for (int k = 0; k < 3; k++) {
        a.p[k] = v->p[k];
        a.wo[k] = v->wo[k];
        a.ns[k] = v->ns[k];
        a.ng[k] = v->ng[k];
        a.le[k] = v->le[k];
        a.dir_wi[k] = v->dir_wi[k];
        a.dir_l[k] = v->dir_l[k];
        a.ind_wi[k] = v->ind_wi[k];
    }
    a.mis = v->mis;
    a.dir_pdf = v->dir_pdf;
    a.ind_mis = v->ind_mis;
    a.flags = v->flags;
    a.material = v->material;
    a.n = v->n;
    return a;
}
bool vertices_complete(const sty_pf_vertices *v) {
    if (!v->active || !v->mis || !v->dir_pdf || !v->ind_mis || !v->flags || !v->material) return false;
    for (int k = 0; k < 3; k++)
        if (!v->p[k] || !v->wo[k] || !v->ns[k] || !v->ng[k] || !v->le[k] || !v->dir_wi[k] || !v->dir_l[k] ||
            !v->ind_wi[k])
            return false;
    return true;
}
}  // namespace

extern "C" {

sty_status sty_pf_ref_create(uint64_t max_vertices, uint32_t table_size, sty_pf_ref_ctx **out) {
    clear_error();
    STY_ARG_CHECK(out, "sty_pf_ref_create: null out");
    STY_ARG_CHECK(max_vertices > 0 && max_vertices < (1ull << 31), "max_vertices must be in [1, 2^31)");
    STY_ARG_CHECK(table_size > 0 && table_size < 0xffffffffu, "table_size must be in [1, 2^32-1)");
    sty_pf_ref_ctx *c = new sty_pf_ref_ctx();
    c->cap = max_vertices;
    c->table = table_size;
    cudaGetDevice(&c->device);
    const size_t n = max_vertices;
    sty_status st = STY_OK;
    auto alloc = [&](void **p, size_t bytes, const char *what) {
        if (st == STY_OK) st = check_cuda(cudaMalloc(p, bytes), what);
    };
    alloc((void **)&c->act, n * 4, "alloc act");
    alloc((void **)&c->num, 4, "alloc num");
    alloc((void **)&c->keys, n * 4, "alloc keys");
    alloc((void **)&c->vals, n * 4, "alloc vals");
    alloc((void **)&c->keys_s, n * 4, "alloc keys_s");
    alloc((void **)&c->vals_s, n * 4, "alloc vals_s");
    alloc((void **)&c->ranges, (size_t)table_size * sizeof(uint2), "alloc ranges");
    alloc((void **)&c->cid, n * 4, "alloc cid");
    alloc((void **)&c->csize, n * 4, "alloc csize");
    alloc((void **)&c->size0, n * 4, "alloc size0");
    alloc((void **)&c->prop, n * 4, "alloc prop");
    alloc((void **)&c->winner, (size_t)table_size * 4, "alloc winner");
    alloc((void **)&c->counter, 4, "alloc counter");
    alloc((void **)&c->mats, kMaxMaterials * sizeof(sty_pf_material), "alloc materials");
    alloc((void **)&c->progs, kMaxPrograms * sizeof(sty_style_program), "alloc programs");
    if (st == STY_OK) {
        size_t b1 = 0, b2 = 0;
        thrust::counting_iterator<uint32_t> it(0);
        st = check_cuda(cub::DeviceSelect::Flagged(nullptr, b1, it, (const int32_t *)nullptr, c->act, c->num, (int)n),
                        "cub select size");
        if (st == STY_OK)
            st = check_cuda(cub::DeviceRadixSort::SortPairs(nullptr, b2, c->keys, c->keys_s, c->vals, c->vals_s, (int)n),
                            "cub sort size");
        c->tmp_bytes = b1 > b2 ? b1 : b2;
        alloc(&c->tmp, c->tmp_bytes, "alloc cub temp");
    }
    if (st != STY_OK) {
        free_ctx(c);
        return st;
    }
    *out = c;
    return STY_OK;
}

sty_status sty_pf_ref_destroy(sty_pf_ref_ctx *ctx) {
    clear_error();
    if (!ctx) return STY_OK;
    free_ctx(ctx);
    return STY_OK;
}

sty_status sty_pf_ref_filter(sty_pf_ref_ctx *ctx, const sty_pf_vertices *v, const float *in_next,
                             const sty_pf_ref_params *prm, const sty_pf_material *materials, uint32_t n_materials,
                             const sty_style_program *programs, uint32_t n_programs, sty_pcg32 *rng, float *out,
                             uint32_t *neighbours, uint32_t *cluster_id, void *stream) {
    clear_error();
    STY_ARG_CHECK(ctx && v && prm && materials && rng && out, "sty_pf_ref_filter: null argument");
    STY_ARG_CHECK(vertices_complete(v), "sty_pf_ref_filter: a vertex field is null");
    STY_ARG_CHECK(v->n > 0 && v->n <= ctx->cap, "vertex count %llu exceeds the context capacity %llu",
                  (unsigned long long)v->n, (unsigned long long)ctx->cap);
    STY_ARG_CHECK(prm->table_size == ctx->table, "table_size differs from the context's");
    STY_ARG_CHECK(prm->radius > 0.0f && std::isfinite(prm->radius), "radius must be > 0");
    STY_ARG_CHECK(prm->reuse >= 1 && prm->reuse <= 1024, "reuse must be in [1, 1024]");
    STY_ARG_CHECK(n_materials >= 1 && n_materials <= kMaxMaterials, "n_materials must be in [1, %u]", kMaxMaterials);
    STY_ARG_CHECK(n_programs <= kMaxPrograms, "n_programs must be <= %u", kMaxPrograms);
    STY_ARG_CHECK(programs || n_programs == 0, "null programs");
    for (uint32_t i = 0; i < n_programs; i++)
        STY_ARG_CHECK(style_program_valid(&programs[i]), "invalid style program %u", i);
    for (int a = 0; a < 3; a++) STY_ARG_CHECK(prm->pmax[a] > prm->pmin[a], "empty grid bounds");
    cudaStream_t st = as_stream(stream);
    const uint64_t n = v->n;
    VArgs va = make_vargs(v);
    Geo g;
    for (int a = 0; a < 3; a++) {
        g.pmin[a] = prm->pmin[a];
        g.pmax[a] = prm->pmax[a];
        const float ext = prm->pmax[a] - prm->pmin[a];
        const float rr = floorf(ext / prm->radius);  // (aabb_extent / radius).floor() (:1587)
        STY_ARG_CHECK(rr < 4.0e9f, "grid resolution overflows");
        g.res[a] = rr < 1.0f ? 1u : (uint32_t)rr;
    }
    g.table = prm->table_size;
    g.r = prm->radius;
    const int bs = 256;
    const unsigned nb = (unsigned)((n + bs - 1) / bs);
    STY_TRY(check_cuda(cudaMemcpyAsync(ctx->mats, materials, n_materials * sizeof(sty_pf_material),
                                       cudaMemcpyHostToDevice, st), "upload materials"));
    if (n_programs)
        STY_TRY(check_cuda(cudaMemcpyAsync(ctx->progs, programs, n_programs * sizeof(sty_style_program),
                                           cudaMemcpyHostToDevice, st), "upload programs"));

    // 1. compact active slots (stable)
    thrust::counting_iterator<uint32_t> it(0);
    size_t tb = ctx->tmp_bytes;
    STY_TRY(check_cuda(cub::DeviceSelect::Flagged(ctx->tmp, tb, it, v->active, ctx->act, ctx->num, (int)n, st),
                       "compact active"));
    count_launch();
    // 2-4. keys, stable sort, bucket ranges
    k_keys<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->keys, ctx->vals);
    STY_TRY(check_launch("k_keys"));
    tb = ctx->tmp_bytes;
    STY_TRY(check_cuda(cub::DeviceRadixSort::SortPairs(ctx->tmp, tb, ctx->keys, ctx->keys_s, ctx->vals, ctx->vals_s,
                                                       (int)n, 0, 32, st),
                       "sort buckets"));
    count_launch();
    STY_TRY(check_cuda(cudaMemsetAsync(ctx->ranges, 0, (size_t)ctx->table * sizeof(uint2), st), "reset ranges"));
    k_ranges<<<nb, bs, 0, st>>>(ctx->keys_s, ctx->num, ctx->ranges);
    STY_TRY(check_launch("k_ranges"));

    // 5. clustering
    STY_TRY(check_cuda(cudaMemsetAsync(ctx->cid, 0xff, n * 4, st), "reset cid"));
    if (prm->cluster) {
        STY_TRY(check_cuda(cudaMemsetAsync(ctx->csize, 0, n * 4, st), "reset csize"));
        STY_TRY(check_cuda(cudaMemsetAsync(ctx->prop, 0xff, n * 4, st), "reset prop"));
        bool done = false;
        for (uint32_t round = 0; round <= prm->max_cluster_rounds; round++) {
            STY_TRY(check_cuda(cudaMemsetAsync(ctx->counter, 0, 4, st), "reset counter"));
            k_cl_count<<<nb, bs, 0, st>>>(ctx->act, ctx->num, ctx->cid, ctx->counter);
            STY_TRY(check_launch("k_cl_count"));
            uint32_t remaining = 0;  // host read-back per round, like the reference (:1699)
            STY_TRY(check_cuda(cudaMemcpyAsync(&remaining, ctx->counter, 4, cudaMemcpyDeviceToHost, st), "read counter"));
            STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync counter"));
            if (remaining == 0) {
                done = true;
                break;
            }
            if (round == prm->max_cluster_rounds) break;
            k_cl_claim_reset<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->cid, ctx->winner);
            STY_TRY(check_launch("k_cl_claim_reset"));
            k_cl_claim_min<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->cid, ctx->winner);
            STY_TRY(check_launch("k_cl_claim_min"));
            k_cl_claim_set<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->cid, ctx->csize, ctx->winner);
            STY_TRY(check_launch("k_cl_claim_set"));
            STY_TRY(check_cuda(cudaMemcpyAsync(ctx->size0, ctx->csize, n * 4, cudaMemcpyDeviceToDevice, st), "snapshot"));
            k_cl_propose<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->ranges, ctx->vals_s, ctx->cid, ctx->size0,
                                            prm->reuse, ctx->prop);
            STY_TRY(check_launch("k_cl_propose"));
            k_cl_accept<<<nb, bs, 0, st>>>(va, g, ctx->act, ctx->num, ctx->ranges, ctx->vals_s, ctx->cid, ctx->csize,
                                           ctx->prop, prm->reuse);
            STY_TRY(check_launch("k_cl_accept"));
        }
        if (!done) {
            set_error("clustering did not converge within %u rounds", prm->max_cluster_rounds);
            return STY_ERR_ITER_LIMIT;
        }
    }
    // 6. filter
    STY_TRY(check_cuda(cudaMemsetAsync(out, 0, 3 * n * sizeof(float), st), "reset out"));
    if (neighbours) STY_TRY(check_cuda(cudaMemsetAsync(neighbours, 0, n * 4, st), "reset neighbours"));
    const unsigned nbf = (unsigned)((n + 127) / 128);
    if (prm->reuse <= 128)
        k_ref_filter<128><<<nbf, 128, 0, st>>>(va, g, ctx->act, ctx->num, ctx->ranges, ctx->vals_s, ctx->cid, in_next,
                                               *prm, ctx->mats, n_materials, ctx->progs, n_programs, rng, out, neighbours);
    else
        k_ref_filter<1024><<<nbf, 128, 0, st>>>(va, g, ctx->act, ctx->num, ctx->ranges, ctx->vals_s, ctx->cid, in_next,
                                                *prm, ctx->mats, n_materials, ctx->progs, n_programs, rng, out,
                                                neighbours);
    STY_TRY(check_launch("k_ref_filter"));
    if (cluster_id)
        STY_TRY(check_cuda(cudaMemcpyAsync(cluster_id, ctx->cid, n * 4, cudaMemcpyDeviceToDevice, st), "copy cid"));
    return STY_OK;
}

}  // extern "C"
