// pf_ref.cu -- reference-mode NL-PF (world-space hash grid, clustering, SMIS) for one depth.
//
// Pipeline per call (all on the caller's stream):
//   1. compact the active path slots in ascending order (cub::DeviceSelect::Flagged, stable);
//   2. bucket key per point = hash(cell) mod table (lm_path_filtering.rs:20-59);
//   3. stable radix sort of (bucket, slot) -> every bucket lists its points in ascending slot
//      order, the fixed replacement of the reference's CAS-built linked lists (:230-255);
//   4. bucket -> [start, end) table;
//   5. (cluster) deterministic clustering rounds (:533-623, :1675-1710): claim / propose / accept;
//   6. filter: one warp per active vertex (evaluate_filtered_radiance, :758-972).
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cmath>

#include <vector>

#include "bsdf.cuh"
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
    float r2max;  // largest f32 s with sqrt_rn(s) <= r: dist_f(..) <= r  <=>  dist2_f(..) <= r2max
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

// the radicand of dist_f, rounded the same way
__device__ __forceinline__ float dist2_f(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    float s = __fmul_rn(dx, dx);
    s = __fadd_rn(s, __fmul_rn(dy, dy));
    return __fadd_rn(s, __fmul_rn(dz, dz));
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
__device__ __forceinline__ bsdf::B3 tob(V3 v) { return bsdf::b3(v.x, v.y, v.z); }
// the principled closure (inlined: an out-of-line call costs the filter more spills than it saves)
__device__ __forceinline__ float princ_eval(const bsdf::PClosure *pc, const float *tab, V3 ns, V3 ng, V3 wo, V3 wi,
                                         float *f) {
    return bsdf::eval_world(*pc, tab, tob(ns), tob(ng), tob(wo), tob(wi), f);
}
// Surface::evaluate: f*|cos_i| and pdf (diffuse.rs:17-48; mod.rs:1877-1910 with unit Fresnel; the
// principled closure pc with the albedo table tab, bsdf.cuh)
// the fields of a material the diffuse / GGX evaluation and the style lookup read (the principled
// path reads its precomputed closure instead)
struct MatCore {
    int32_t kind;
    float albedo[3];
    float alpha;
    int32_t style[4];
};
__device__ __forceinline__ MatCore mat_core(const sty_pf_material &m) {
    MatCore c;
    c.kind = m.kind;
    c.albedo[0] = m.albedo[0];
    c.albedo[1] = m.albedo[1];
    c.albedo[2] = m.albedo[2];
    c.alpha = m.alpha;
    for (int i = 0; i < 4; i++) c.style[i] = m.style[i];
    return c;
}
template <bool PRINC>
__device__ __forceinline__ void bsdf_eval(const MatCore &m, V3 ns, V3 ng, V3 wo, V3 wi, float f[3], float *pdf,
                          const bsdf::PClosure *pc, const float *tab) {
    if constexpr (PRINC) {
        if (bsdf::closure_kind(m.kind)) {
            *pdf = princ_eval(pc, tab, ns, ng, wo, wi, f);
            return;
        }
    }
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
// bucket-ordered copies of what the walk reads per candidate: position + flags (16 B), cluster id
__global__ void k_sorted_view(VArgs v, const uint32_t *num, const uint32_t *sorted, const uint32_t *cid, int cluster,
                              float4 *spos, uint32_t *scid) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *num) return;
    const uint32_t u = sorted[k];
    spos[k] = make_float4(v.p[0][u], v.p[1][u], v.p[2][u], __uint_as_float(v.flags[u] & 15u));
    if (cluster) scid[k] = cid[u];
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

__device__ __forceinline__ uint32_t pcg_output(uint64_t old) {
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}

// Per-warp shared scratch for a reservoir of R neighbours: 64-bit (candidate index, vertex) keys,
// the neighbour list, and each neighbour's BSDF frame with its wo-side terms precomputed for the
// SMIS pdf sums.
struct __align__(16) NbFrame {  // 64 bytes: four 16-byte shared-memory reads
    float ns[3], ng[3], wo[3];
    float fl;      // sign(ng . ns)
    float co;      // wo . ns
    float alpha;   // GGX: max(alpha, 1e-4)
    float g1;      // GGX: 1 / (1 + Lambda(co))
    uint32_t bits; // bit 0: the wo half of check_wo_wi_valid holds; bit 1: GGX; bit 2: principled
    uint32_t mat;  // material index (the principled closure)
    uint32_t pad;
};
// rounded up to 16 bytes so that every warp's scratch starts 16-byte aligned for any R
__host__ __device__ constexpr size_t warp_scratch_bytes(uint32_t R) {
    return ((size_t)R * (sizeof(unsigned long long) + sizeof(uint32_t) + sizeof(NbFrame)) + 15u) & ~(size_t)15u;
}
__device__ __forceinline__ NbFrame make_frame(const sty_pf_material &m, uint32_t mi, V3 ns, V3 ng, V3 wo) {
    auto sgn = [](float x) { return x > 0.0f ? 1.0f : -1.0f; };
    NbFrame f;
    f.ns[0] = ns.x, f.ns[1] = ns.y, f.ns[2] = ns.z;
    f.ng[0] = ng.x, f.ng[1] = ng.y, f.ng[2] = ng.z;
    f.wo[0] = wo.x, f.wo[1] = wo.y, f.wo[2] = wo.z;
    f.fl = sgn(dot3(ng, ns));
    f.co = dot3(wo, ns);
    const bool ok = sgn(f.fl * f.co) * sgn(dot3(wo, ng)) > 0.0f;
    const bool ggx = m.kind != STY_MAT_DIFFUSE;
    f.alpha = fmaxf(m.alpha, 1e-4f);
    f.g1 = ggx ? 1.0f / (1.0f + tr_lambda(f.co, f.alpha)) : 0.0f;
    f.bits = (ok ? 1u : 0u) | (ggx ? 2u : 0u) | (bsdf::closure_kind(m.kind) ? 4u : 0u);
    f.mat = mi;
    f.pad = 0;
    return f;
}
// the pdf of bsdf_eval for a precomputed frame (same arithmetic; the lane-dependent validity tests
// become selects, only the frame's lobe -- the same on every lane -- branches)
template <bool PRINC>
__device__ __forceinline__ float frame_pdf(const NbFrame &f, V3 wi, const bsdf::PClosure *cls, const float *tab) {
    auto sgn = [](float x) { return x > 0.0f ? 1.0f : -1.0f; };
    const V3 ns = {f.ns[0], f.ns[1], f.ns[2]}, ng = {f.ng[0], f.ng[1], f.ng[2]};
    if constexpr (PRINC) {
        if (f.bits & 4u) {  // principled: the closure's pdf (no precomputed terms)
            float fv[3];
            return princ_eval(cls + f.mat, tab, ns, ng, V3{f.wo[0], f.wo[1], f.wo[2]}, wi, fv);
        }
    }
    const float ci = dot3(wi, ns), co = f.co;
    const bool ok = (f.bits & 1u) && sgn(f.fl * ci) * sgn(dot3(wi, ng)) > 0.0f && co * ci >= 0.0f;
    if (!(f.bits & 2u)) return ok ? fabsf(ci) / kPi : 0.0f;
    const V3 wo = {f.wo[0], f.wo[1], f.wo[2]};
    V3 wh = {wo.x + wi.x, wo.y + wi.y, wo.z + wi.z};
    const bool ok2 = ok && !(dot3(wh, wo) * dot3(wi, wh) < 0.0f) && !(wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) &&
                     ci != 0.0f && co != 0.0f;
    if (!ok2) wh = {0.0f, 0.0f, 1.0f};  // any unit vector: the result is discarded
    const float l = sqrtf(dot3(wh, wh));
    wh = {wh.x / l, wh.y / l, wh.z / l};
    const float d = tr_d(dot3(wh, ns), f.alpha);
    const float owh = fabsf(dot3(wo, wh));
    const float p = d * f.g1 * owh / fabsf(co) / (4.0f * owh);
    return ok2 ? p : 0.0f;
}

// One warp per active vertex (evaluate_filtered_radiance, :758-972); persistent warps take the
// vertices in bucket order from a work counter, so that warps running together walk the same cells.
// Gather: the 27-cell walk in the sequential order (cells dz, dy, dx; bucket entries ascending),
// 32 candidates at a time from the bucket-ordered positions; a passing candidate's index c in that
// order comes from a ballot prefix count. The reservoir (:806-829) keeps the first R candidates and
// lets candidate c >= R replace slot j = pcg32() % (c + 1) when j < R, the draw being the
// (c - R)-th of the vertex's stream. The replacing candidates of one chunk take consecutive draws,
// so lane r's state is A^r s + inc * (1 + A + ... + A^(r-1)) from the chunk's starting state s,
// with (A^r, sum) held by lane r; slot j keeps the largest replacing c (64-bit atomicMax of
// (c, vertex)), which is what the sequential loop leaves there. Neighbour counts, lists and the
// final RNG state are therefore bit-identical to the sequential walk.
// Evaluate: lanes take neighbours t = lane, lane + 32, ...; the SMIS pdf sums (:886-939) read the
// reservoir's frames from shared memory (warp-wide broadcasts); lane sums are combined by a
// shuffle tree, then lane 0 applies the style node and writes the vertex's radiance.
__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
    const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)x, src), hi = __shfl_sync(0xffffffffu, (uint32_t)(x >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}
// PRINC: some material is STY_MAT_PRINCIPLED or STY_MAT_GLASS (the variant without it keeps the diffuse / GGX path's
// registers and stack as they were)
template <bool PRINC>
__global__ void __launch_bounds__(256, 4) k_ref_filter(VArgs v, Geo g, const uint32_t *num, uint32_t *next,
                                                    const uint2 *ranges,
                                                    const uint32_t *sorted, const float4 *spos, const uint32_t *scid,
                                                    const uint32_t *cid, const float *in_next, sty_pf_ref_params prm,
                                                    const sty_pf_material *mats, uint32_t n_mats,
                                                    const bsdf::PClosure *cls, const float *tab,
                                                    const sty_style_program *progs, uint32_t n_progs, sty_pcg32 *rng,
                                                    float *out, uint32_t *neighbours) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    static_assert(sizeof(NbFrame) == 64 && alignof(NbFrame) == 16, "frame layout");
    const uint32_t R = prm.reuse;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint8_t *ws = smem_raw + (size_t)wib * warp_scratch_bytes(R);
    // frames first (16-byte aligned), then the 8-byte keys, then the list
    NbFrame *frames = reinterpret_cast<NbFrame *>(ws);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + (size_t)R * sizeof(NbFrame));
    uint32_t *list = reinterpret_cast<uint32_t *>(ws + (size_t)R * (sizeof(NbFrame) + sizeof(unsigned long long)));
    const unsigned lt_mask = (1u << lane) - 1u;
    // lane r: A^r and 1 + A + ... + A^(r-1) (mod 2^64), for the reservoir draws
    uint64_t a_pow = 1u, a_sum = 0u;
    for (int r = 0; r < lane; r++) {
        a_sum += a_pow;
        a_pow *= 0x5851f42d4c957f2dULL;
    }
    const uint32_t nact = *num;
    for (;;) {
    // next vertex in bucket order from the launch's work counter (dynamic balance: vertices in
    // dense regions cost far more than others)
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(next, 1u);
    i = __shfl_sync(0xffffffffu, i, 0);
    if (i >= nact) break;
    const uint32_t vi = sorted[i];
    const uint64_t n = v.n;
    const uint32_t qs = prm.cluster ? cid[vi] : vi;
    const float qx = v.p[0][qs], qy = v.p[1][qs], qz = v.p[2][qs];
    const uint32_t my_cluster = prm.cluster ? cid[vi] : NONE;
    const uint32_t my_flags = v.flags[vi] & 15u;
    const sty_pcg32 st0 = rng[vi];
    uint64_t s_cur = st0.state;  // state before the next draw (warp-uniform)
    // lane l < 27 looks up cell l of the walk order (dz outer, dy, dx inner)
    uint2 my_rg = make_uint2(0u, 0u);
    {
        int32_t c0[3];
        get_cell(g, qx, qy, qz, c0);
        if (lane < 27) {
            const int32_t nx = c0[0] + lane % 3 - 1, ny = c0[1] + (lane / 3) % 3 - 1, nz = c0[2] + lane / 9 - 1;
            if (nx >= 0 && ny >= 0 && nz >= 0 && nx < (int32_t)g.res[0] && ny < (int32_t)g.res[1] &&
                nz < (int32_t)g.res[2])
                my_rg = ranges[bucket_of(g, nx, ny, nz)];
        }
    }
    // ---- gather
    uint32_t cnt = 0;  // warp-uniform
    for (int cell = 0; cell < 27; cell++) {
                const uint2 rg = make_uint2(__shfl_sync(0xffffffffu, my_rg.x, cell), __shfl_sync(0xffffffffu, my_rg.y, cell));
                // four chunks of 32 candidates per step: their loads are issued together
                for (uint32_t base = rg.x; base < rg.y; base += 128) {
                    float4 e[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const uint32_t kk = base + q * 32 + lane;
                        e[q] = kk < rg.y ? spos[kk] : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        if (base + q * 32 >= rg.y) break;  // warp-uniform
                        const uint32_t kk = base + q * 32 + lane;
                        bool pass = false;
                        if (kk < rg.y) {
                            pass = dist2_f(e[q].x, e[q].y, e[q].z, qx, qy, qz) <= g.r2max;
                            if (pass && prm.cluster && scid[kk] != my_cluster) pass = false;
                            if (pass && !prm.disable_flag_check && __float_as_uint(e[q].w) != my_flags) pass = false;
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, pass);
                        if (bal == 0u) continue;
                        const uint32_t c = cnt + __popc(bal & lt_mask);
                        const uint32_t u = pass ? sorted[kk] : 0u;
                        if (pass && c < R) keys[c] = ((unsigned long long)c << 32) | u;
                        __syncwarp();
                        const bool rep = pass && c >= R;
                        const unsigned balr = __ballot_sync(0xffffffffu, rep);
                        if (balr) {
                            const int r = __popc(balr & lt_mask);
                            const uint64_t ap = shfl64(a_pow, r), as = shfl64(a_sum, r);
                            const uint64_t s_m = ap * s_cur + st0.inc * as;
                            if (rep) {
                                const uint32_t j = pcg_output(s_m) % (c + 1u);
                                if (j < R) atomicMax(&keys[j], ((unsigned long long)c << 32) | u);
                            }
                            const int last = 31 - __clz((int)balr);
                            s_cur = shfl64(s_m * 0x5851f42d4c957f2dULL + st0.inc, last);
                        }
                        __syncwarp();
                        cnt += __popc(bal);
                    }
                }
            }
    if (lane == 0) {
        sty_pcg32 st = st0;
        st.state = s_cur;
        rng[vi] = st;
        if (neighbours) neighbours[vi] = cnt;
    }
    const uint32_t k = min(cnt, R);
    for (uint32_t t = lane; t < k; t += 32) {
        const uint32_t u = (uint32_t)keys[t];
        list[t] = u;
        const uint32_t mu = min(v.material[u], n_mats - 1);
        frames[t] = make_frame(mats[mu], mu, ld3(v.ns, u), ld3(v.ng, u), ld3(v.wo, u));
    }
    __syncwarp();

    // ---- evaluate
    const uint32_t mvi = min(v.material[vi], n_mats - 1);
    const MatCore mv = mat_core(mats[mvi]);
    const bsdf::PClosure *pcv = cls + mvi;
    const V3 wo = ld3(v.wo, vi), ns = ld3(v.ns, vi), ng = ld3(v.ng, vi);
    float direct[3] = {0.f, 0.f, 0.f}, indirect[3] = {0.f, 0.f, 0.f};
    const float invk = k ? 1.0f / (float)k : 0.0f;
    const uint32_t rounds = (k + 31u) / 32u;  // every lane runs the SMIS loop the same number of times
    for (uint32_t r = 0; r < rounds; r++) {
        const uint32_t t = r * 32u + lane;
        const bool have = t < k;
        const uint32_t u = have ? list[t] : 0u;
        V3 wi = {0.f, 0.f, 0.f};
        float reused[3] = {0.f, 0.f, 0.f}, pdf_v = 0.0f;
        bool ind = false;
        if (have) {
            const float dpdf = v.dir_pdf[u];
            if (dpdf > 0.0f) {  // :839-863
                float f[3], pdf;
                bsdf_eval<PRINC>(mv, ns, ng, wo, ld3(v.dir_wi, u), f, &pdf, pcv, tab);
                const float w = dpdf / (dpdf + pdf);
#pragma unroll
                for (int c = 0; c < 3; c++) direct[c] += f[c] * v.dir_l[c][u] * w / dpdf * invk;
            }
            wi = ld3(v.ind_wi, u);
            if (dot3(wi, wi) != 0.0f) {
                ind = true;
                float f[3];
                bsdf_eval<PRINC>(mv, ns, ng, wo, wi, f, &pdf_v, pcv, tab);
                const float mis = v.ind_mis[u];
#pragma unroll
                for (int c = 0; c < 3; c++) reused[c] = f[c] * (in_next ? in_next[c * n + u] : 0.0f) * mis;
            }
        }
        if (prm.smis) {
            float sum_pdf = 0.0f;
            uint32_t a = 0;
            for (; a + 4 <= k; a += 4) {
                const float p0 = frame_pdf<PRINC>(frames[a], wi, cls, tab);
                const float p1 = frame_pdf<PRINC>(frames[a + 1], wi, cls, tab);
                const float p2 = frame_pdf<PRINC>(frames[a + 2], wi, cls, tab);
                const float p3 = frame_pdf<PRINC>(frames[a + 3], wi, cls, tab);
                sum_pdf += p0;  // in list order, as the sequential sum
                sum_pdf += p1;
                sum_pdf += p2;
                sum_pdf += p3;
            }
            for (; a < k; a++) sum_pdf += frame_pdf<PRINC>(frames[a], wi, cls, tab);
            if (ind && sum_pdf > 0.0f)
#pragma unroll
                for (int c = 0; c < 3; c++) indirect[c] += reused[c] / sum_pdf;
        } else if (ind && pdf_v > 0.0f) {
#pragma unroll
            for (int c = 0; c < 3; c++) indirect[c] += reused[c] / pdf_v * invk;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            direct[c] += __shfl_xor_sync(0xffffffffu, direct[c], o);
            indirect[c] += __shfl_xor_sync(0xffffffffu, indirect[c], o);
        }
    if (lane == 0) {
        f3 rad = {v.le[0][vi] + direct[0] + indirect[0], v.le[1][vi] + direct[1] + indirect[1],
                  v.le[2][vi] + direct[2] + indirect[2]};
        const uint32_t fl = v.flags[vi];
        if ((prm.depth > 0 || !prm.no_first_hit_stylization) && !(fl & 1u)) {
            const int32_t pi = mv.style[style_index(fl)];
            if (pi >= 0 && (uint32_t)pi < n_progs) {
                const V3 pp = ld3(v.p, vi);
                rad = style_apply(progs[pi], prm.depth, rad, f3{pp.x, pp.y, pp.z});
            }
        }
        out[vi] = rad.x;
        out[n + vi] = rad.y;
        out[2 * n + vi] = rad.z;
    }
    __syncwarp();  // the next vertex reuses the warp's scratch
    }
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
    float4 *spos = nullptr;  // bucket-ordered position + flags
    uint32_t *scid = nullptr;  // bucket-ordered cluster id
    sty_pf_material *mats = nullptr;      // device copies of the host tables
    sty::bsdf::PClosure *cls = nullptr;   // principled closures of the materials (host-built)
    std::vector<sty::bsdf::PClosure> hcls;  // their host copy (the async upload's source)
    sty_style_program *progs = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int device = -1;
};

using namespace sty;

namespace {
void free_ctx(sty_pf_ref_ctx *c) {
    void *ptrs[] = {c->act,   c->num,    c->keys,  c->vals,    c->keys_s,  c->vals_s, c->ranges, c->cid,
                    c->csize, c->size0,  c->prop,  c->winner,  c->counter, c->mats,   c->progs,  c->tmp,
                    c->spos,  c->scid,   c->cls};
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
    alloc((void **)&c->spos, n * sizeof(float4), "alloc sorted positions");
    alloc((void **)&c->scid, n * 4, "alloc sorted cluster ids");
    alloc((void **)&c->mats, kMaxMaterials * sizeof(sty_pf_material), "alloc materials");
    alloc((void **)&c->cls, kMaxMaterials * sizeof(bsdf::PClosure), "alloc closures");
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
    {
        // f32 sqrt is correctly rounded on host and device: find the largest s with sqrt(s) <= r
        float t = prm->radius * prm->radius;
        while (std::sqrt(t) > prm->radius) t = std::nextafter(t, 0.0f);
        for (;;) {
            const float nx = std::nextafter(t, INFINITY);
            if (!(std::sqrt(nx) <= prm->radius)) break;
            t = nx;
        }
        g.r2max = t;
    }
    const int bs = 256;
    const unsigned nb = (unsigned)((n + bs - 1) / bs);
    STY_TRY(check_cuda(cudaMemcpyAsync(ctx->mats, materials, n_materials * sizeof(sty_pf_material),
                                       cudaMemcpyHostToDevice, st), "upload materials"));
    ctx->hcls.resize(n_materials);
    for (uint32_t i = 0; i < n_materials; i++) ctx->hcls[i] = bsdf::make_closure(materials[i]);
    STY_TRY(check_cuda(cudaMemcpyAsync(ctx->cls, ctx->hcls.data(), n_materials * sizeof(bsdf::PClosure),
                                       cudaMemcpyHostToDevice, st), "upload closures"));
    const float *ggx_tab = principled_table();
    if (!ggx_tab) {
        set_error("principled albedo table unavailable");
        return STY_ERR_CUDA;
    }
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
    // one warp per active vertex; warps per block as the reservoir's shared scratch allows
    const size_t wsb = warp_scratch_bytes(prm->reuse);
    uint32_t wpb = (uint32_t)std::min<size_t>(8, (96u * 1024u) / wsb);
    if (wpb < 1) wpb = 1;
    const size_t smem = wpb * wsb;
    bool any_princ = false;
    for (uint32_t i = 0; i < n_materials; i++) any_princ = any_princ || bsdf::closure_kind(materials[i].kind);
    auto kern = any_princ ? k_ref_filter<true> : k_ref_filter<false>;
    if (smem > 48u * 1024u)
        STY_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "attr k_ref_filter"));
    // persistent warps: as many blocks as stay resident, each warp looping over vertices
    int per_sm = 0, dev = 0, sms = 0;
    STY_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * wpb, smem),
                       "occupancy k_ref_filter"));
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (n + wpb - 1) / wpb, cap_blocks = (uint64_t)std::max(per_sm, 1) * (uint64_t)std::max(sms, 1);
    const unsigned nbf = (unsigned)std::min(want, cap_blocks);
    k_sorted_view<<<nb, bs, 0, st>>>(va, ctx->num, ctx->vals_s, ctx->cid, prm->cluster, ctx->spos, ctx->scid);
    STY_TRY(check_launch("k_sorted_view"));
    STY_TRY(check_cuda(cudaMemsetAsync(ctx->counter, 0, 4, st), "reset work counter"));
    kern<<<nbf, 32 * wpb, smem, st>>>(va, g, ctx->num, ctx->counter, ctx->ranges, ctx->vals_s, ctx->spos,
                                              ctx->scid, ctx->cid,
                                              in_next, *prm, ctx->mats, n_materials, ctx->cls, ggx_tab, ctx->progs,
                                              n_programs, rng, out, neighbours);
    STY_TRY(check_launch("k_ref_filter"));
    if (cluster_id)
        STY_TRY(check_cuda(cudaMemcpyAsync(cluster_id, ctx->cid, n * 4, cudaMemcpyDeviceToDevice, st), "copy cid"));
    return STY_OK;
}

}  // extern "C"
