// sty_oracle_ref.cpp -- CPU restatement of the reference-mode NL-PF pass (test infrastructure).
//
// Follows crates/akari_integrator/src/lm_path_filtering.rs (paths relative to the reference
// project) with the fixed evaluation order documented in include/sty_gb300.h: buckets list their
// points in ascending path index, clustering claims / joins are resolved deterministically.
// Geometry tests (cell, distance) are done in float exactly as the reference's f32 code; radiance
// arithmetic is double.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "sty_oracle.h"

namespace {

constexpr uint32_t NONE = 0xffffffffu;

struct Grid {
    float pmin[3], pmax[3];
    uint32_t res[3];
    uint32_t table;
    std::unordered_map<uint32_t, std::vector<uint32_t>> buckets;
};

// HashGridVar::get_cell (:47-54)
inline void get_cell(const Grid &g, const float p[3], int32_t c[3]) {
    for (int a = 0; a < 3; a++) {
        float t = (p[a] - g.pmin[a]) / (g.pmax[a] - g.pmin[a]);
        t = std::min(std::max(t, 0.0f), 1.0f);
        t = t * (float)g.res[a];
        uint32_t u = (uint32_t)t;
        c[a] = (int32_t)std::min(u, g.res[a] - 1u);
    }
}
// hash + cell_pos_to_index (:21-23, :56-59)
inline uint32_t bucket_of(const Grid &g, const int32_t c[3]) {
    uint64_t h = ((uint64_t)(uint32_t)c[0] * 73856093ULL) ^ ((uint64_t)(uint32_t)c[1] * 19349663ULL) ^
                 ((uint64_t)(uint32_t)c[2] * 83492791ULL);
    return (uint32_t)(h % (uint64_t)g.table);
}
// (a - b).length() in f32 without contraction
inline float dist_f(const float a[3], const float b[3]) {
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return std::sqrt(s);
}

// for_each_neighbor (:61-123): dz outer, dy, dx inner; skip cells outside [0, res)
template <class F>
void walk(const Grid &g, const float q[3], F &&f) {
    int32_t c[3];
    get_cell(g, q, c);
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int32_t n[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                if (n[0] < 0 || n[1] < 0 || n[2] < 0 || n[0] >= (int32_t)g.res[0] || n[1] >= (int32_t)g.res[1] ||
                    n[2] >= (int32_t)g.res[2])
                    continue;
                auto it = g.buckets.find(bucket_of(g, n));
                if (it == g.buckets.end()) continue;
                for (uint32_t u : it->second) f(u);
            }
}

inline uint32_t pcg_next(sty_pcg32 &s) {
    uint64_t old = s.state;
    s.state = old * 0x5851f42d4c957f2dULL + s.inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}

struct D3 {
    double x, y, z;
};
inline double dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ---- BSDFs ------------------------------------------------------------------------------------
// SurfaceClosure::check_wo_wi_valid (svm/surface/mod.rs:1699-1712)
inline bool wo_wi_valid(D3 ns, D3 ng, D3 wo, D3 wi) {
    auto sgn = [](double x) { return x > 0 ? 1.0 : -1.0; };
    double flipped = sgn(dot3(ng, ns));
    return sgn(flipped * dot3(wo, ns)) * sgn(dot3(wo, ng)) > 0 && sgn(flipped * dot3(wi, ns)) * sgn(dot3(wi, ng)) > 0;
}
// Trowbridge-Reitz D / Lambda, isotropic alpha (microfacet.rs:44-66)
inline double tr_d(double cos_h, double a) {
    double c2 = cos_h * cos_h, s2 = std::max(0.0, 1.0 - c2);
    double tan2 = s2 / c2;
    double e = tan2 / (a * a);
    double inv_d = M_PI * a * a * c2 * c2 * (1.0 + e) * (1.0 + e);
    if (!std::isfinite(tan2) || !std::isfinite(inv_d) || inv_d == 0.0) return 0.0;
    return 1.0 / inv_d;
}
inline double tr_lambda(double cos_w, double a) {
    double c2 = cos_w * cos_w, s2 = std::max(0.0, 1.0 - c2);
    double abs_tan = std::fabs(std::sqrt(s2) / cos_w);
    double l = (-1.0 + std::sqrt(1.0 + a * a * abs_tan * abs_tan)) * 0.5;
    return std::isfinite(abs_tan) ? l : 0.0;
}
// evaluate(): returns f*|cos| (rgb) and pdf. diffuse.rs:17-48, mod.rs:1877-1910.
void bsdf_eval(const sty_pf_material &m, D3 ns, D3 ng, D3 wo, D3 wi, double f[3], double *pdf) {
    f[0] = f[1] = f[2] = 0.0;
    *pdf = 0.0;
    if (!wo_wi_valid(ns, ng, wo, wi)) return;
    const double co = dot3(wo, ns), ci = dot3(wi, ns);
    if (m.kind == STY_MAT_DIFFUSE) {
        if (co * ci >= 0.0) {
            *pdf = std::fabs(ci) / M_PI;
            for (int c = 0; c < 3; c++) f[c] = (double)m.albedo[c] / M_PI * std::fabs(ci);
        }
        return;
    }
    // microfacet reflection
    const double a = std::max((double)m.alpha, 1e-4);
    D3 wh = {wo.x + wi.x, wo.y + wi.y, wo.z + wi.z};
    if (dot3(wh, wo) * dot3(wi, wh) < 0.0 || (wh.x == 0 && wh.y == 0 && wh.z == 0) || ci == 0.0 || co == 0.0 ||
        !(co * ci >= 0.0))
        return;
    const double l = std::sqrt(dot3(wh, wh));
    wh = {wh.x / l, wh.y / l, wh.z / l};
    const double ch = dot3(wh, ns);
    const double d = tr_d(ch, a);
    const double g = 1.0 / (1.0 + tr_lambda(co, a) + tr_lambda(ci, a));
    const double g1 = 1.0 / (1.0 + tr_lambda(co, a));
    const double k = std::fabs(0.25 * d * g / (ci * co)) * std::fabs(ci);
    for (int c = 0; c < 3; c++) f[c] = (double)m.albedo[c] * k;
    const double owh = std::fabs(dot3(wo, wh));
    *pdf = d * g1 * owh / std::fabs(co) / (4.0 * owh);
}

struct View {
    const sty_pf_vertices *v;
    D3 get(const float *const a[3], uint32_t i) const { return {a[0][i], a[1][i], a[2][i]}; }
    void pf(uint32_t i, float out[3]) const {
        out[0] = v->p[0][i];
        out[1] = v->p[1][i];
        out[2] = v->p[2][i];
    }
};

inline uint32_t style_index(uint32_t flags) {  // StylizationFlagsExpr::get_style_index (mod.rs:72-84)
    uint32_t i = 0;
    if (flags & 2u) i = 1;
    if (flags & 4u) i = 2;
    if (flags & 8u) i = 3;
    return i;
}

}  // namespace

extern "C" {

// select (nullable): filter only the active vertices with select[i] != 0 (the grid and clusters are
// still built from every active vertex); the others keep out = 0 and their RNG state. For checks at
// full vertex counts.
int32_t orc_pf_ref_filter_select(const sty_pf_vertices *v, const float *in_next,
                                 const sty_pf_ref_params *prm, const sty_pf_material *mats, uint32_t n_mats,
                                 const sty_style_program *progs, uint32_t n_progs, sty_pcg32 *rng, double *out,
                                 uint32_t *neighbours, uint32_t *cluster_id, const uint8_t *select) {
    const uint64_t n = v->n;
    View V{v};
    Grid g;
    for (int a = 0; a < 3; a++) {
        g.pmin[a] = prm->pmin[a];
        g.pmax[a] = prm->pmax[a];
        float ext = prm->pmax[a] - prm->pmin[a];
        float r = std::floor(ext / prm->radius);  // (aabb_extent / radius).floor().as_uvec3() (:1587)
        g.res[a] = r < 1.0f ? 1u : (uint32_t)r;
    }
    g.table = prm->table_size;
    std::vector<uint32_t> act;
    for (uint64_t i = 0; i < n; i++)
        if (v->active[i]) act.push_back((uint32_t)i);
    for (uint32_t i : act) {  // build: buckets list points in ascending index
        float p[3];
        int32_t c[3];
        V.pf(i, p);
        get_cell(g, p, c);
        g.buckets[bucket_of(g, c)].push_back(i);
    }
    const float r = prm->radius;
    std::vector<uint32_t> cid(n, NONE), csize(n, 0);

    if (prm->cluster) {
        uint32_t round = 0;
        for (;; round++) {
            std::vector<uint32_t> un;
            for (uint32_t i : act)
                if (cid[i] == NONE) un.push_back(i);
            if (un.empty()) break;
            if (round >= prm->max_cluster_rounds) return STY_ERR_ITER_LIMIT;
            // claim: lowest unclustered index per bucket becomes a centre (kernel_init_cluster)
            std::unordered_map<uint32_t, uint32_t> winner;
            for (uint32_t i : un) {
                float p[3];
                int32_t c[3];
                V.pf(i, p);
                get_cell(g, p, c);
                uint32_t b = bucket_of(g, c);
                auto it = winner.find(b);
                if (it == winner.end() || i < it->second) winner[b] = i;
            }
            for (auto &kv : winner) {
                cid[kv.second] = kv.second;
                csize[kv.second] = 0;
            }
            // propose (kernel_cluster): first centre in walk order within r with room
            std::vector<uint32_t> size0 = csize;
            std::vector<uint32_t> prop(n, NONE);
            for (uint32_t i : un) {
                if (cid[i] != NONE) continue;
                float p[3];
                V.pf(i, p);
                bool done = false;
                walk(g, p, [&](uint32_t u) {
                    if (done) return;
                    float q[3];
                    V.pf(u, q);
                    if (dist_f(q, p) <= r && cid[u] == u && size0[u] < prm->reuse) {
                        prop[i] = u;
                        done = true;
                    }
                });
            }
            // accept: each centre, walk order, while it has room
            for (uint32_t c : act) {
                if (cid[c] != c) continue;
                float p[3];
                V.pf(c, p);
                walk(g, p, [&](uint32_t u) {
                    if (prop[u] == c && cid[u] == NONE && csize[c] < prm->reuse) {
                        cid[u] = c;
                        csize[c]++;
                    }
                });
            }
        }
    }

    const uint32_t reuse = prm->reuse;
    std::vector<uint32_t> list(reuse);
    for (uint64_t i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) out[c * n + i] = 0.0;
        if (neighbours) neighbours[i] = 0;
        if (cluster_id) cluster_id[i] = prm->cluster ? cid[i] : NONE;
    }
    for (uint32_t vi : act) {
        if (select && !select[vi]) continue;
        float q[3];
        V.pf(prm->cluster ? cid[vi] : vi, q);
        const uint32_t my_cluster = cid[vi];
        const uint32_t my_flags = v->flags[vi] & 15u;
        uint32_t cnt = 0;
        walk(g, q, [&](uint32_t u) {
            float pu[3];
            V.pf(u, pu);
            if (!(dist_f(pu, q) <= r)) return;
            if (prm->cluster && cid[u] != my_cluster) return;
            if (!prm->disable_flag_check && (v->flags[u] & 15u) != my_flags) return;
            if (cnt < reuse) {
                list[cnt] = u;
            } else {
                uint32_t j = pcg_next(rng[vi]) % (cnt + 1);
                if (j < reuse) list[j] = u;
            }
            cnt++;
        });
        if (neighbours) neighbours[vi] = cnt;
        const uint32_t k = std::min(cnt, reuse);
        const sty_pf_material &mv = mats[std::min(v->material[vi], n_mats - 1)];
        const D3 wo = V.get(v->wo, vi), ns = V.get(v->ns, vi), ng = V.get(v->ng, vi);
        double direct[3] = {0, 0, 0}, indirect[3] = {0, 0, 0};
        for (uint32_t t = 0; t < k; t++) {
            const uint32_t u = list[t];
            const double dpdf = v->dir_pdf[u];
            if (dpdf > 0.0) {  // :839-863
                double f[3], pdf;
                bsdf_eval(mv, ns, ng, wo, V.get(v->dir_wi, u), f, &pdf);
                const double w = dpdf / (dpdf + pdf);
                for (int c = 0; c < 3; c++) direct[c] += f[c] * (double)v->dir_l[c][u] * 1.0 * w / dpdf / (double)k;
            }
            const D3 wi = V.get(v->ind_wi, u);
            if (dot3(wi, wi) == 0.0) continue;  // :864-868
            double f[3], pdf;
            bsdf_eval(mv, ns, ng, wo, wi, f, &pdf);
            double reused[3];
            for (int c = 0; c < 3; c++)
                reused[c] = f[c] * (in_next ? (double)in_next[c * n + u] : 0.0) * (double)v->ind_mis[u];
            if (prm->smis) {  // :886-939
                double sum_pdf = 0.0;
                for (uint32_t jj = 0; jj < k; jj++) {
                    const uint32_t a = list[jj];
                    const sty_pf_material &ma = mats[std::min(v->material[a], n_mats - 1)];
                    double fa[3], pa;
                    bsdf_eval(ma, V.get(v->ns, a), V.get(v->ng, a), V.get(v->wo, a), wi, fa, &pa);
                    sum_pdf += pa;
                }
                if (sum_pdf > 0.0)
                    for (int c = 0; c < 3; c++) indirect[c] += reused[c] / sum_pdf;
            } else if (pdf > 0.0) {  // :940-944
                for (int c = 0; c < 3; c++) indirect[c] += reused[c] / pdf / (double)k;
            }
        }
        double rad[3];
        for (int c = 0; c < 3; c++) rad[c] = (double)v->le[c][vi] + direct[c] + indirect[c];
        const bool stylize = (prm->depth > 0 || !prm->no_first_hit_stylization) && !(v->flags[vi] & 1u);
        if (stylize) {
            const int32_t pi = mv.style[style_index(v->flags[vi])];
            if (pi >= 0 && (uint32_t)pi < n_progs) {
                const double pp[3] = {(double)v->p[0][vi], (double)v->p[1][vi], (double)v->p[2][vi]};
                orc_style_apply_at_f64(&progs[pi], prm->depth, rad, pp, rad, 1);
            }
        }
        for (int c = 0; c < 3; c++) out[c * n + vi] = rad[c];
    }
    return STY_OK;
}

int32_t orc_pf_ref_filter(const sty_pf_vertices *v, const float *in_next,
                          const sty_pf_ref_params *prm, const sty_pf_material *mats, uint32_t n_mats,
                          const sty_style_program *progs, uint32_t n_progs, sty_pcg32 *rng, double *out,
                          uint32_t *neighbours, uint32_t *cluster_id) {
    return orc_pf_ref_filter_select(v, in_next, prm, mats, n_mats, progs, n_progs, rng, out, neighbours, cluster_id,
                                    nullptr);
}

}  // extern "C"
