// brpt.cu -- the branching path tracer (crates/akari_integrator/src/branching_pt.rs): the paper's
// BrPT baseline and, with inner_samples = [1], the plain stylized path tracer of
// configs/teaser/pt.json.
//
// Per pixel a tree of vertices. A vertex whose surface is rough (average roughness > 0.01) and is
// the k-th rough vertex of its path takes inner_samples[k] branches (1 beyond the list, 1 at smooth
// vertices, none at max_depth); each branch is one light sample (NEE, the light's style at depth + 1
// with the vertex's updated flags) and one BSDF sample whose continuation ray makes the child vertex
// (kernel_advance :543-726). Bottom-up, a vertex's radiance is
//   style_depth(Le + (1/n) sum_branches (direct_s + throughput_s * L_child_s * mis_child_s))
// with the style picked by the flags the vertex inherited (kernel_propagate :240-500, the
// non-debiased estimator; mis_child is the child's emission weight, :568-575); the depth-0 vertex's
// radiance is the pixel sample.
//
// GB300 layout: one breadth-first wavefront per depth over SoA slot planes. A vertex's children are
// one contiguous block (exclusive scan of the branch counts), so the tree needs no linked lists or
// atomics, a child finds its parent by binary search over the scan, and the bottom-up sums run in a
// fixed order (deterministic). Pixels go through in passes sized so the worst-case tree fits the
// `vram_mb` budget (the reference's pixels_per_pass rule, :806-846).
// Sampling: hierarchical 64-bit keys -- the camera slot of pixel px in repeat r keys on
// (seed, r, px), a child on (its parent's key, branch index) -- each seeding one PCG32 stream
// (2 draws for the camera; per branch 3 for the light, then 3 for the BSDF), so an image does not
// depend on how pixels are grouped into passes. The reference draws from a per-slot PCG32 buffer
// whose slots are handed out by atomics; that assignment is not reproducible, so no stream of it is
// matched here.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "scene.cuh"
#include "style.cuh"
#include "tracer.cuh"

namespace sty {
const sty_camera &scene_camera(const sty_scene *s);
bool style_program_valid(const sty_style_program *p);
}  // namespace sty

namespace sty {
namespace {

constexpr uint32_t kBrSlotBytes = 100;  // 22 four-byte planes + one 8-byte key per slot

struct BrSlots {
    float *p[3], *ng[3], *wo[3], *rad[3], *thr[3], *dir[3], *mis;
    uint32_t *prim, *flags, *ab, *nchild, *cbase;
    uint64_t *key;
};
struct BrInner {
    uint32_t n;
    uint32_t v[STY_BRPT_MAX_LEVELS];
};

__device__ __forceinline__ sty_pcg32 key_stream(uint64_t key) {
    sty_pcg32 g;
    g.state = 0;
    g.inc = (key << 1) | 1ull;
    pcg_next(g);
    g.state += splitmix64(key);
    pcg_next(g);
    return g;
}
__device__ __forceinline__ uint64_t child_key(uint64_t parent, uint32_t s) {
    return splitmix64(parent ^ (0x9e3779b97f4a7c15ull * (uint64_t)(s + 1u)));
}
__device__ __forceinline__ F3 hit_point(const SceneView &sc, const Hit &h) {
    const float *tp = sc.tri_pos + 9 * (size_t)h.prim;
    const float b0 = 1.0f - h.b1 - h.b2;
    return f3m(b0 * tp[0] + h.b1 * tp[3] + h.b2 * tp[6], b0 * tp[1] + h.b1 * tp[4] + h.b2 * tp[7],
               b0 * tp[2] + h.b1 * tp[5] + h.b2 * tp[8]);
}
__device__ __forceinline__ F3 tri_ng(const SceneView &sc, uint32_t prim) {
    return f3m(sc.tri_normal[3 * prim], sc.tri_normal[3 * prim + 1], sc.tri_normal[3 * prim + 2]);
}
__device__ __forceinline__ void put3(float *const (&pl)[3], size_t i, F3 v) {
    pl[0][i] = v.x;
    pl[1][i] = v.y;
    pl[2][i] = v.z;
}
__device__ __forceinline__ F3 get3(float *const (&pl)[3], size_t i) { return f3m(pl[0][i], pl[1][i], pl[2][i]); }

// key of repeat r: every pixel sample of that repeat keys on it
__host__ __device__ __forceinline__ uint64_t repeat_key(uint64_t seed, uint64_t r) {
    return splitmix64(splitmix64(seed ^ 0x4252505400000000ull) + r);
}
// depth 0: the camera slots of samples q0 .. q0 + n, sample q = repeat * npx + pixel (kernel_init
// :501-541)
__global__ void k_br_camera(SceneView sc, CamArgs cam, uint32_t n, uint64_t q0, uint32_t npx, uint64_t seed,
                            uint64_t first_repeat, BrSlots s, unsigned long long *hits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t q = q0 + i;
    const uint32_t px = (uint32_t)(q % npx);
    const uint64_t key = splitmix64(repeat_key(seed, first_repeat + q / npx) + px);
    sty_pcg32 st = key_stream(key);
    F3 ro, rd;
    camera_ray(cam, px, st, &ro, &rd);
    s.key[i] = key;
    s.flags[i] = 0;
    s.ab[i] = 0;
    s.mis[i] = 1.0f;
    put3(s.thr, i, f3m(1.0f, 1.0f, 1.0f));
    const float o3[3] = {ro.x, ro.y, ro.z}, d3[3] = {rd.x, rd.y, rd.z};
    const Hit h = trace_closest(sc, o3, d3, 0.0f, 1e20f, NONE);
    s.prim[i] = h.prim;
    if (h.prim == NONE) {
        put3(s.rad, i, f3m(0.0f, 0.0f, 0.0f));
        return;
    }
    atomicAdd(hits, 1ull);
    const F3 p = hit_point(sc, h), ng = tri_ng(sc, h.prim);
    const sty_scene_material m = sc.materials[sc.tri_material[h.prim]];
    F3 le;
    float mis;
    emitter_le(sc, m, h.prim, p, ng, rd, 0, ro, 0.0f, &le, &mis);
    put3(s.p, i, p);
    put3(s.ng, i, ng);
    put3(s.wo, i, -rd);
    put3(s.rad, i, le);
}

// branch count of each slot of one depth (kernel_advance :598-620)
template <bool PRINC>
__global__ void k_br_count(SceneView sc, uint32_t n, uint32_t base, uint32_t depth, uint32_t max_depth, BrInner inner,
                           BrSlots s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t g = base + i;
    uint32_t c = 0;
    const uint32_t prim = s.prim[g];
    if (prim != NONE && depth + 1 <= max_depth) {
        const sty_scene_material m = sc.materials[sc.tri_material[prim]];
        const uint32_t ab = s.ab[g];
        const F3 ng = get3(s.ng, g), wo = get3(s.wo, g);
        c = lobe_roughness<PRINC>(m, sc.ggx_tab, ng, wo) > 0.01f ? (ab < inner.n ? inner.v[ab] : 1u) : 1u;
    }
    s.nchild[g] = c;
}

// one thread per branch of the parents of one depth: NEE + BSDF sample + continuation ray -> the
// child slot (kernel_advance :622-712)
// 3 blocks of 256 per SM (80 registers): the BVH walk is latency-bound, and the compiler would
// otherwise take 95 registers for the closure-free variant and drop to 2 blocks
template <bool PRINC>
__global__ void __launch_bounds__(256, 3) k_br_branch(SceneView sc, uint32_t n_child, uint32_t pbase, uint32_t n_par, uint32_t cbase0,
                            uint32_t depth, const sty_style_program *progs, uint32_t n_progs, BrSlots s,
                            unsigned long long *hits) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_child) return;
    uint32_t lo = 0, hi = n_par - 1;  // the last parent whose block starts at or before j
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (s.cbase[pbase + mid] <= j) lo = mid;
        else hi = mid - 1u;
    }
    const uint32_t pg = pbase + lo, sidx = j - s.cbase[pg], cg = cbase0 + j;
    const uint32_t prim = s.prim[pg];
    const F3 p = get3(s.p, pg), ng = get3(s.ng, pg), wo = get3(s.wo, pg);
    const sty_scene_material m = sc.materials[sc.tri_material[prim]];
    const uint32_t new_flags = update_flags(m, s.flags[pg]);
    const uint32_t ab = s.ab[pg] + (lobe_roughness<PRINC>(m, sc.ggx_tab, ng, wo) > 0.01f ? 1u : 0u);
    const uint64_t key = child_key(s.key[pg], sidx);
    sty_pcg32 st = key_stream(key);
    // NEE (sample_light :727-783, shaded with balance MIS in sample_surface_and_shade_direct :170-197)
    F3 direct = f3m(0.0f, 0.0f, 0.0f);
    {
        F3 lwi;
        f3 li;
        float lpdf;
        if (nee_sample(sc, p, ng, prim, new_flags, depth, progs, n_progs, st, &lwi, &li, &lpdf)) {
            F3 f;
            const float bp = bsdf_eval<PRINC>(m, ng, ng, wo, lwi, &f, sc.ggx_tab);
            const float w = lpdf / (lpdf + bp) / lpdf;
            direct = f3m(li.x * f.x, li.y * f.y, li.z * f.z) * w;
        }
    }
    put3(s.dir, cg, direct);
    s.key[cg] = key;
    s.flags[cg] = new_flags;
    s.ab[cg] = ab;
    s.prim[cg] = NONE;
    s.mis[cg] = 1.0f;
    put3(s.rad, cg, f3m(0.0f, 0.0f, 0.0f));
    put3(s.thr, cg, f3m(0.0f, 0.0f, 0.0f));
    const float usel = next_1d(st), u0 = next_1d(st), u1 = next_1d(st);
    float pdf = 0.0f;
    const F3 wi = bsdf_sample<PRINC>(m, ng, ng, wo, usel, u0, u1, &pdf, sc.ggx_tab);
    if (!(pdf > 0.0f)) return;
    F3 f;
    bsdf_eval<PRINC>(m, ng, ng, wo, wi, &f, sc.ggx_tab);
    const F3 ro = offset_ray_origin(p, face_forward(ng, wi));
    const float o3[3] = {ro.x, ro.y, ro.z}, d3[3] = {wi.x, wi.y, wi.z};
    const Hit h = trace_closest(sc, o3, d3, 0.0f, 1e20f, prim);
    if (h.prim == NONE) return;
    atomicAdd(hits, 1ull);
    const F3 q = hit_point(sc, h), qn = tri_ng(sc, h.prim);
    const sty_scene_material mq = sc.materials[sc.tri_material[h.prim]];
    F3 le;
    float mis;
    emitter_le(sc, mq, h.prim, q, qn, wi, depth + 1, p, pdf, &le, &mis);
    s.prim[cg] = h.prim;
    put3(s.p, cg, q);
    put3(s.ng, cg, qn);
    put3(s.wo, cg, -wi);
    put3(s.rad, cg, le);
    put3(s.thr, cg, f * (1.0f / pdf));
    s.mis[cg] = mis;
}

// bottom-up radiance of one depth (kernel_propagate); depth 0 leaves the pixel samples in `rad`
__global__ void __launch_bounds__(256, 5) k_br_propagate(SceneView sc, uint32_t n, uint32_t base, uint32_t cbase0, uint32_t depth,
                               const sty_style_program *progs, uint32_t n_progs, BrSlots s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t g = base + i;
    f3 out = {0.0f, 0.0f, 0.0f};
    const uint32_t prim = s.prim[g];
    if (prim != NONE) {
        F3 li = get3(s.rad, g);
        const uint32_t nc = s.nchild[g];
        if (nc) {
            F3 dsum = f3m(0.0f, 0.0f, 0.0f), isum = f3m(0.0f, 0.0f, 0.0f);
            const uint32_t c0 = cbase0 + s.cbase[g];
            for (uint32_t k = 0; k < nc; k++) {
                const uint32_t c = c0 + k;
                dsum = dsum + get3(s.dir, c);
                if (s.prim[c] != NONE) {
                    const F3 t = get3(s.thr, c), r = get3(s.rad, c);
                    isum = isum + f3m(t.x * r.x, t.y * r.y, t.z * r.z) * s.mis[c];
                }
            }
            li = li + (dsum + isum) * (1.0f / (float)nc);
        }
        out = {li.x, li.y, li.z};
        const uint32_t fl = s.flags[g];
        if (!(fl & 1u)) {
            const int32_t pi = sc.materials[sc.tri_material[prim]].style[style_index(fl)];
            if (pi >= 0 && (uint32_t)pi < n_progs) {
                const F3 p = get3(s.p, g);
                out = style_apply(progs[pi], depth, out, f3{p.x, p.y, p.z});
            }
        }
        put3(s.rad, g, f3m(out.x, out.y, out.z));
    } else if (depth == 0) {
        put3(s.rad, g, f3m(0.0f, 0.0f, 0.0f));
    }
}
// film += weight * sample for every sample of the pass, per pixel in repeat order (film.add_sample):
// the sequence of FP64 additions does not depend on how samples are grouped into passes
__global__ void k_br_film(uint32_t npx, uint64_t q0, uint32_t n, BrSlots s, double weight, double *film) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npx) return;
    uint64_t q = q0 + (px + npx - (uint32_t)(q0 % npx)) % npx;  // the pass's first sample of px
    double *fp = film + 3 * (size_t)px;
    for (; q < q0 + n; q += npx) {
        const size_t i = (size_t)(q - q0);
        fp[0] += weight * s.rad[0][i];
        fp[1] += weight * s.rad[1][i];
        fp[2] += weight * s.rad[2][i];
    }
}

}  // namespace
}  // namespace sty

using namespace sty;

sty_status sty_brpt_render(sty_scene *scene, const sty_brpt_config *cfg, const sty_style_program *programs,
                           uint32_t n_programs, double *film, sty_brpt_stats *stats, void *stream) {
    clear_error();
    STY_ARG_CHECK(scene && cfg && film, "sty_brpt_render: null argument");
    STY_ARG_CHECK(cfg->max_depth <= 64, "max_depth must be <= 64");
    STY_ARG_CHECK(cfg->n_levels >= 1 && cfg->n_levels <= STY_BRPT_MAX_LEVELS, "n_levels must be in [1, %d]",
                  STY_BRPT_MAX_LEVELS);
    for (uint32_t k = 0; k < cfg->n_levels; k++)
        STY_ARG_CHECK(cfg->inner_samples[k] >= 1 && cfg->inner_samples[k] <= 65536, "inner_samples[%u] must be in [1, 65536]",
                      k);
    STY_ARG_CHECK(cfg->repeats >= 1 && cfg->vram_mb >= 1, "repeats and vram_mb must be >= 1");
    STY_ARG_CHECK((uint64_t)cfg->first_repeat + cfg->repeats <= 0xFFFFFFFFull, "first_repeat + repeats overflows");
    STY_ARG_CHECK(n_programs <= 64 && (n_programs == 0 || programs), "bad style programs");
    for (uint32_t k = 0; k < n_programs; k++)
        STY_ARG_CHECK(style_program_valid(&programs[k]), "style program %u is invalid", k);
    const cudaStream_t st = as_stream(stream);
    const sty_camera &cam = scene_camera(scene);
    const uint32_t npx = cam.width * cam.height;
    // worst-case tree per pixel: every vertex rough and every ray hitting
    double worst = 0.0, level = 1.0;
    for (uint32_t d = 0; d <= cfg->max_depth; d++) {
        worst += level;
        level *= d < cfg->n_levels ? cfg->inner_samples[d] : 1.0;
    }
    const double budget = (double)cfg->vram_mb * 1048576.0 / kBrSlotBytes;
    uint64_t ppp = (uint64_t)(budget / worst);
    if (ppp == 0) {
        set_error("vram_mb (%u) is below one pixel's worst-case vertex tree (%.0f vertices)", cfg->vram_mb, worst);
        return STY_ERR_ARG;
    }
    ppp = std::min<uint64_t>(ppp, (uint64_t)npx * cfg->repeats);
    ppp = std::min<uint64_t>(ppp, (uint64_t)(2147483647.0 / worst));
    STY_ARG_CHECK(ppp >= 1, "vertex tree of one pixel exceeds 2^31 slots");
    const uint64_t cap = (uint64_t)((double)ppp * worst) + 1;

    // slot planes
    std::vector<void *> allocs;
    auto cleanup = [&]() {
        for (void *q : allocs) cudaFree(q);
    };
    sty_status s = STY_OK;
    auto mk = [&](size_t bytes, const char *what) -> void * {
        void *q = nullptr;
        if (s == STY_OK) s = check_cuda(cudaMalloc(&q, std::max<size_t>(bytes, 16)), what);
        if (q) allocs.push_back(q);
        return q;
    };
    BrSlots sl;
    float *fpl = (float *)mk(cap * 4 * 19, "alloc brpt float planes");
    uint32_t *upl = (uint32_t *)mk(cap * 4 * 5, "alloc brpt index planes");
    sl.key = (uint64_t *)mk(cap * 8, "alloc brpt keys");
    sty_style_program *dprog = (sty_style_program *)mk(std::max<uint32_t>(n_programs, 1) * sizeof(sty_style_program),
                                                       "alloc programs");
    unsigned long long *dhits = (unsigned long long *)mk(8, "alloc counter");
    uint32_t *dtail = (uint32_t *)mk(8, "alloc tail");
    size_t scan_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)cap);
    void *dscan = mk(scan_bytes, "alloc scan scratch");
    if (s != STY_OK) {
        cleanup();
        return s;
    }
    {
        int k = 0;
        auto fp = [&]() { return fpl + (size_t)(k++) * cap; };
        for (int a = 0; a < 3; a++) sl.p[a] = fp();
        for (int a = 0; a < 3; a++) sl.ng[a] = fp();
        for (int a = 0; a < 3; a++) sl.wo[a] = fp();
        for (int a = 0; a < 3; a++) sl.rad[a] = fp();
        for (int a = 0; a < 3; a++) sl.thr[a] = fp();
        for (int a = 0; a < 3; a++) sl.dir[a] = fp();
        sl.mis = fp();
        sl.prim = upl;
        sl.flags = upl + cap;
        sl.ab = upl + 2 * cap;
        sl.nchild = upl + 3 * cap;
        sl.cbase = upl + 4 * cap;
    }
    BrInner inner;
    inner.n = cfg->n_levels;
    for (uint32_t k = 0; k < STY_BRPT_MAX_LEVELS; k++) inner.v[k] = k < cfg->n_levels ? cfg->inner_samples[k] : 1u;
    const SceneView sv = scene_view(scene);
    const CamArgs ca = make_camera(cam);
    auto run = [&]() -> sty_status {
        if (n_programs)
            STY_TRY(check_cuda(cudaMemcpyAsync(dprog, programs, n_programs * sizeof(sty_style_program),
                                               cudaMemcpyHostToDevice, st), "upload programs"));
        STY_TRY(check_cuda(cudaMemsetAsync(dhits, 0, 8, st), "zero counter"));
        uint64_t slots = 0, passes = 0, max_pass = 0;
        const double weight = 1.0 / cfg->repeats;
        std::vector<uint32_t> cnt, off;
        const uint64_t total = (uint64_t)npx * cfg->repeats;
        {
            for (uint64_t q0 = 0; q0 < total; q0 += ppp) {
                const uint32_t P = (uint32_t)std::min<uint64_t>(ppp, total - q0);
                cnt.assign(1, P);
                off.assign(1, 0);
                k_br_camera<<<(P + 255) / 256, 256, 0, st>>>(sv, ca, P, q0, npx, cfg->seed, cfg->first_repeat, sl,
                                                             dhits);
                STY_TRY(check_launch("k_br_camera"));
                for (uint32_t d = 0; d <= cfg->max_depth; d++) {
                    const uint32_t n = cnt[d], base = off[d];
                    (sv.any_closure ? k_br_count<true> : k_br_count<false>)<<<(n + 255) / 256, 256, 0, st>>>(
                        sv, n, base, d, cfg->max_depth, inner, sl);
                    STY_TRY(check_launch("k_br_count"));
                    size_t tb = scan_bytes;
                    STY_TRY(check_cuda(cub::DeviceScan::ExclusiveSum(dscan, tb, sl.nchild + base, sl.cbase + base,
                                                                     (int)n, st),
                                       "scan branch counts"));
                    count_launch();
                    STY_TRY(check_cuda(cudaMemcpyAsync(dtail, sl.cbase + base + n - 1, 4, cudaMemcpyDeviceToDevice, st),
                                       "tail"));
                    STY_TRY(check_cuda(cudaMemcpyAsync(dtail + 1, sl.nchild + base + n - 1, 4,
                                                       cudaMemcpyDeviceToDevice, st),
                                       "tail"));
                    uint32_t tail[2];
                    STY_TRY(check_cuda(cudaMemcpyAsync(tail, dtail, 8, cudaMemcpyDeviceToHost, st), "read tail"));
                    STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync"));
                    const uint64_t next = (uint64_t)tail[0] + tail[1];
                    if (next == 0) break;
                    if ((uint64_t)base + n + next > cap) {
                        set_error("vertex tree overflow (%llu slots, capacity %llu)",
                                  (unsigned long long)(base + n + next), (unsigned long long)cap);
                        return STY_ERR_ITER_LIMIT;
                    }
                    off.push_back(base + n);
                    cnt.push_back((uint32_t)next);
                    (sv.any_closure ? k_br_branch<true> : k_br_branch<false>)<<<(unsigned)((next + 255) / 256), 256, 0, st>>>(sv, (uint32_t)next, base, n, base + n,
                                                                                d, dprog, n_programs, sl, dhits);
                    STY_TRY(check_launch("k_br_branch"));
                }
                for (int d = (int)cnt.size() - 1; d >= 0; d--) {
                    const uint32_t cb = (size_t)d + 1 < off.size() ? off[d + 1] : 0u;
                    k_br_propagate<<<(cnt[d] + 255) / 256, 256, 0, st>>>(sv, cnt[d], off[d], cb, (uint32_t)d, dprog,
                                                                         n_programs, sl);
                    STY_TRY(check_launch("k_br_propagate"));
                }
                k_br_film<<<(npx + 255) / 256, 256, 0, st>>>(npx, q0, P, sl, weight, film);
                STY_TRY(check_launch("k_br_film"));
                uint64_t pass_slots = 0;
                for (uint32_t c : cnt) pass_slots += c;
                slots += pass_slots;
                max_pass = std::max(max_pass, pass_slots);
                passes++;
            }
        }
        if (stats) {
            unsigned long long h = 0;
            STY_TRY(check_cuda(cudaMemcpyAsync(&h, dhits, 8, cudaMemcpyDeviceToHost, st), "read counter"));
            STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync"));
            stats->vertices = h;
            stats->slots = slots;
            stats->passes = passes;
            stats->pixels_per_pass = ppp;
            stats->max_pass_slots = max_pass;
        }
        return check_cuda(cudaStreamSynchronize(st), "sty_brpt_render");
    };
    s = run();
    cudaStreamSynchronize(st);
    cleanup();
    return s;
}
