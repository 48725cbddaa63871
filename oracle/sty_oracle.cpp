// sty_oracle.cpp -- CPU restatement of the reference arithmetic (test infrastructure only;
// see sty_oracle.h). Reference paths are relative to the reference project root.
#include "sty_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T>
struct V3 {
    T x, y, z;
};
template <class T>
inline V3<T> v3(T x, T y, T z) {
    return {x, y, z};
}

// ---- colour helpers: crates/akari_render/src/color.rs:328-361, 536-600 ----------------------
template <class T>
inline T lum709(V3<T> c) {  // Color::lum, color.rs:356-361
    return c.x * T(0.2126) + c.y * T(0.7152) + c.z * T(0.0722);
}
template <class T>
inline T linear_to_srgb1(T v) {  // color.rs:545-549
    return v <= T(0.0031308) ? v * T(12.92) : std::pow(v, T(1) / T(2.4)) * T(1.055) - T(0.055);
}
template <class T>
inline T srgb_to_linear1(T v) {  // color.rs:540-544
    return v <= T(0.04045) ? v / T(12.92) : std::pow((v + T(0.055)) / T(1.055), T(2.4));
}
template <class T>
inline V3<T> linear_to_srgb(V3<T> c) {
    return {linear_to_srgb1(c.x), linear_to_srgb1(c.y), linear_to_srgb1(c.z)};
}
template <class T>
inline V3<T> srgb_to_linear(V3<T> c) {
    return {srgb_to_linear1(c.x), srgb_to_linear1(c.y), srgb_to_linear1(c.z)};
}
template <class T>
inline T clampv(T v, T lo, T hi) {
    return std::min(std::max(v, lo), hi);
}
template <class T>
inline T rem_euclid(T a, T b) {
    T r = std::fmod(a, b);
    return r < T(0) ? r + std::fabs(b) : r;
}
template <class T>
V3<T> rgb_to_hsv(V3<T> c) {  // color.rs:551-575
    T mx = std::max(c.x, std::max(c.y, c.z));
    T mn = std::min(c.x, std::min(c.y, c.z));
    T diff = mx - mn;
    T h;
    if (mx == mn)
        h = 0;
    else if (mx == c.x)
        h = rem_euclid((c.y - c.z) / diff, T(6));
    else if (mx == c.y)
        h = (c.z - c.x) / diff + T(2);
    else
        h = (c.x - c.y) / diff + T(4);
    h = h / T(6);
    T s = mx == T(0) ? T(0) : diff / mx;
    return {h, s, mx};
}
template <class T>
V3<T> hsv_to_rgb(V3<T> hsv) {  // color.rs:577-590
    auto f = [&](int n) {
        T k = rem_euclid(T(n) + hsv.x * T(6), T(6));
        T m = std::max(std::min(std::min(k, T(4) - k), T(1)), T(0));
        return hsv.z - hsv.z * hsv.y * m;
    };
    return {f(5), f(3), f(1)};
}
template <class T>
inline T round_half_away(T v) {
    return std::round(v);
}

// ---- style nodes: crates/akari_render/src/svm/surface/mod.rs ---------------------------------
template <class T>
V3<T> style_node(const sty_style_node &nd, uint32_t depth, V3<T> li, V3<T> pos) {
    switch (nd.kind) {
        case STY_STYLE_HALF_TONE: {  // HalfToneSurface::apply_stylization, mod.rs:1180-1232
            if ((double)depth > (double)nd.p[4]) return li;
            const T lum = (li.x + li.y + li.z) / T(3);
            if (lum == T(0)) return li;
            T r = depth == 0 ? lum / T(nd.p[1]) : round_half_away(lum / T(nd.p[0])) / T(nd.p[1]);
            r = T(1) - clampv(r, T(0), T(1));
            const T d = T(nd.p[3]);
            r = r * d * T(0.5) * T(nd.p[2]);
            const float *A = nd.p + 12;
            const T tp[3] = {T(A[0]) * pos.x + T(A[1]) * pos.y + T(A[2]) * pos.z + T(A[3]),
                             T(A[4]) * pos.x + T(A[5]) * pos.y + T(A[6]) * pos.z + T(A[7]),
                             T(A[8]) * pos.x + T(A[9]) * pos.y + T(A[10]) * pos.z + T(A[11])};
            const T ip[3] = {std::floor(tp[0] / d) * d, std::floor(tp[1] / d) * d, std::floor(tp[2] / d) * d};
            T mind = T(1e16);
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++)
                    for (int k = 0; k < 2; k++) {
                        const T qx = ip[0] + T(i) * d - pos.x, qy = ip[1] + T(j) * d - pos.y, qz = ip[2] + T(k) * d - pos.z;
                        mind = std::min(mind, (T)std::sqrt(qx * qx + qy * qy + qz * qz));
                    }
            const float *tone = mind < r ? nd.p + 6 : nd.p + 9;
            const T b = T(nd.p[5]);
            return {li.x + (T(tone[0]) * li.x - li.x) * b, li.y + (T(tone[1]) * li.y - li.y) * b,
                    li.z + (T(tone[2]) * li.z - li.z) * b};
        }
        case STY_STYLE_TOON: {  // ToonSurface::apply_stylization, mod.rs:573-610
            T w = T(nd.p[0]);
            V3<T> c = {clampv(li.x, T(0), T(1e5)), clampv(li.y, T(0), T(1e5)),
                       clampv(li.z, T(0), T(1e5))};
            T lum = lum709(c);
            if (lum <= T(0)) return c;
            V3<T> hue = {c.x / lum, c.y / lum, c.z / lum};
            T nl;
            if (lum > T(1)) {
                nl = std::floor(lum / w) * w;
            } else {
                T a = linear_to_srgb1(lum);
                nl = srgb_to_linear1(std::floor(a / w) * w);
            }
            return {hue.x * nl, hue.y * nl, hue.z * nl};
        }
        case STY_STYLE_PALETTE: {  // ColorPaletteSurface::apply_stylization, mod.rs:697-735
            T indirect_scale = T(nd.p[0]), gamma = T(nd.p[1]);
            V3<T> c = li;
            T lum = (c.x + c.y + c.z) / T(3);
            if (depth != 0) c = {c.x / indirect_scale, c.y / indirect_scale, c.z / indirect_scale};
            c = {clampv(c.x, T(0), T(1)), clampv(c.y, T(0), T(1)), clampv(c.z, T(0), T(1))};
            c = {std::pow(c.x, gamma), std::pow(c.y, gamma), std::pow(c.z, gamma)};
            T min_dist = T(1e16);
            V3<T> best = {0, 0, 0};
            for (int k = 0; k < nd.n; k++) {
                V3<T> q = {T(nd.p[2 + 3 * k]), T(nd.p[3 + 3 * k]), T(nd.p[4 + 3 * k])};
                T dx = q.x - c.x, dy = q.y - c.y, dz = q.z - c.z;
                T dist = dx * dx + dy * dy + dz * dz;
                if (dist < min_dist) {
                    min_dist = dist;
                    best = q;
                }
            }
            T ig = T(1) / gamma;
            c = {std::pow(best.x, ig), std::pow(best.y, ig), std::pow(best.z, ig)};
            if (depth != 0) {
                T nl = (c.x + c.y + c.z) / T(3);
                if (nl != T(0)) {
                    T s = lum / nl;
                    c = {c.x * s, c.y * s, c.z * s};
                }
            }
            return c;
        }
        case STY_STYLE_SAT_ADJUST: {  // SaturationAdjustSurface, mod.rs:821-851
            T power = T(nd.p[0]), indirect_scale = T(nd.p[1]);
            T lum = std::max(li.x, std::max(li.y, li.z));
            if (lum == T(0)) return li;
            V3<T> c = li;
            if (depth != 0) c = {c.x / indirect_scale, c.y / indirect_scale, c.z / indirect_scale};
            c = {clampv(c.x, T(0), T(1)), clampv(c.y, T(0), T(1)), clampv(c.z, T(0), T(1))};
            c = linear_to_srgb(c);
            V3<T> hsv = rgb_to_hsv(c);
            hsv.y = std::pow(hsv.y, power);
            c = srgb_to_linear(hsv_to_rgb(hsv));
            if (depth != 0) c = {c.x * indirect_scale, c.y * indirect_scale, c.z * indirect_scale};
            return c;
        }
        case STY_STYLE_SAT_REX: {  // SaturationAdjustRexSurface, mod.rs:1060-1089
            T blend = T(nd.p[0]);
            T lum = (li.x + li.y + li.z) / T(3);
            T cmin = std::min(li.x, std::min(li.y, li.z));
            if (lum <= T(0) || cmin < T(0)) return li;
            T cmax = std::max(li.x, std::max(li.y, li.z));
            V3<T> imax = {(li.x - cmin) / cmax, (li.y - cmin) / cmax, (li.z - cmin) / cmax};
            T u = (imax.x + imax.y + imax.z) / T(3);
            if (u != T(0)) {
                T k = (T(1) - blend);
                return {blend * lum + k * imax.x * lum / u, blend * lum + k * imax.y * lum / u,
                        blend * lum + k * imax.z * lum / u};
            }
            T v = blend * lum + (T(1) - blend) * lum;
            return {v, v, v};
        }
        case STY_STYLE_EIGHT_BIT: {  // EightBitSurface, mod.rs:1316-1345
            T indirect_scale = T(nd.p[0]);
            auto map8 = [&](V3<T> c) {
                V3<T> s = linear_to_srgb(c);
                V3<T> q = {round_half_away(s.x * T(8)) / T(8), round_half_away(s.y * T(8)) / T(8),
                           round_half_away(s.z * T(4)) / T(4)};
                return srgb_to_linear(q);
            };
            T lum = std::max(li.x, std::max(li.y, li.z));
            if (lum == T(0)) return li;
            if (depth > 0) {
                V3<T> m = map8({li.x / indirect_scale, li.y / indirect_scale, li.z / indirect_scale});
                return {m.x * indirect_scale, m.y * indirect_scale, m.z * indirect_scale};
            }
            T nl = std::min(lum, T(1));
            return map8({li.x / lum * nl, li.y / lum * nl, li.z / lum * nl});
        }
        case STY_STYLE_TOON_STEPS: {  // threshold toon (no reference counterpart)
            V3<T> c = {clampv(li.x, T(0), T(1e5)), clampv(li.y, T(0), T(1e5)),
                       clampv(li.z, T(0), T(1e5))};
            T lum = lum709(c);
            if (lum <= T(0)) return c;
            int k = 0;
            for (int t = 0; t < nd.n; t++) k += (T(nd.p[t]) <= lum) ? 1 : 0;
            T level = T(nd.p[8 + k]);
            return {c.x / lum * level, c.y / lum * level, c.z / lum * level};
        }
        case STY_STYLE_RAMP_SMOOTH: {  // smoothed colour ramp (no reference counterpart)
            V3<T> c = {clampv(li.x, T(0), T(1e5)), clampv(li.y, T(0), T(1e5)),
                       clampv(li.z, T(0), T(1e5))};
            T lum = lum709(c);
            T s = T(nd.p[0]);
            V3<T> o = {0, 0, 0};
            V3<T> prev = {0, 0, 0};
            for (int k = 0; k < nd.n; k++) {
                V3<T> ck = {T(nd.p[9 + 3 * k]), T(nd.p[10 + 3 * k]), T(nd.p[11 + 3 * k])};
                T sg = T(1) / (T(1) + std::exp(-s * (lum - T(nd.p[1 + k]))));
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
template <class T>
V3<T> style_apply(const sty_style_program *prog, uint32_t depth, V3<T> li, V3<T> pos) {
    if (!prog) return li;
    uint32_t bit = depth > 31 ? 31 : depth;
    for (int i = 0; i < prog->n_nodes && i < STY_STYLE_MAX_NODES; i++) {
        const sty_style_node &nd = prog->nodes[i];
        if (!((nd.depth_mask >> bit) & 1u)) continue;
        li = style_node<T>(nd, depth, li, pos);
    }
    return li;
}
template <class T>
V3<T> style_apply(const sty_style_program *prog, uint32_t depth, V3<T> li) {
    return style_apply<T>(prog, depth, li, V3<T>{T(0), T(0), T(0)});
}

inline size_t rec_index(const sty_pf_records *r, int d, int y, int x, int s) {
    return (((size_t)d * r->height + y) * r->width + x) * r->spp + s;
}

}  // namespace

extern "C" {

int32_t orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_num_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_style_apply_f64(const sty_style_program *prog, uint32_t depth, const double *in,
                         double *out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        V3<double> c = style_apply<double>(prog, depth, v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        out[3 * i] = c.x;
        out[3 * i + 1] = c.y;
        out[3 * i + 2] = c.z;
    }
}
void orc_style_apply_at_f64(const sty_style_program *prog, uint32_t depth, const double *in, const double *pos,
                            double *out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        V3<double> c = style_apply<double>(prog, depth, v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]),
                                           v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
        out[3 * i] = c.x;
        out[3 * i + 1] = c.y;
        out[3 * i + 2] = c.z;
    }
}

// Screen-space NL-PF restated in FP64. The neighbour set, weights and recursion are the ones
// documented in include/sty_gb300.h; the per-depth backward order and the propagation of the
// styled result into the parent's "indirect" term follow lm_path_filtering.rs:1673-1764 and
// :974-998, the style call follows :947-971.
void orc_pf_screen_filter_depth_f64(const sty_pf_records *r, uint32_t depth,
                                    const sty_pf_screen_params *prm,
                                    const sty_style_program *style, const double *out_next,
                                    double *out, double *filtered) {
    const int W = r->width, H = r->height, S = r->spp, R = prm->radius;
    const size_t N = (size_t)W * H * S;
    const int d = (int)depth;
    const double inv2s2 = prm->sigma_pixel > 0 ? 1.0 / (2.0 * (double)prm->sigma_pixel * prm->sigma_pixel) : 0.0;
    const double inv2p2 = 1.0 / (2.0 * (double)prm->sigma_pos * prm->sigma_pos);
    const double invn2 = 1.0 / ((double)prm->sigma_nrm * prm->sigma_nrm);
    // in_d(j) = rad + thr * out_{d+1}
    std::vector<double> in(3 * N);
    for (size_t j = 0; j < N; j++) {
        size_t gj = (size_t)d * N + j;
        for (int c = 0; c < 3; c++) {
            double v = r->rad[c][gj];
            if (out_next) v += (double)r->thr[c][gj] * out_next[c * N + j];
            in[3 * j + c] = v;
        }
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; y++) {
        for (int x = 0; x < W; x++) {
            for (int s = 0; s < S; s++) {
                size_t qi = ((size_t)y * W + x) * S + s;
                size_t gq = (size_t)d * N + qi;
                if (!r->valid[gq]) {
                    for (int c = 0; c < 3; c++) {
                        out[c * N + qi] = 0.0;
                        if (filtered) filtered[c * N + qi] = 0.0;
                    }
                    continue;
                }
                double px = r->pos[0][gq], py = r->pos[1][gq], pz = r->pos[2][gq];
                double nx = r->nrm[0][gq], ny = r->nrm[1][gq], nz = r->nrm[2][gq];
                double sw = 0, sr = 0, sg = 0, sb = 0;
                for (int yy = std::max(0, y - R); yy <= std::min(H - 1, y + R); yy++) {
                    for (int xx = std::max(0, x - R); xx <= std::min(W - 1, x + R); xx++) {
                        double dd2 = (double)(xx - x) * (xx - x) + (double)(yy - y) * (yy - y);
                        for (int t = 0; t < S; t++) {
                            size_t j = ((size_t)yy * W + xx) * S + t;
                            size_t gj = (size_t)d * N + j;
                            if (!r->valid[gj]) continue;
                            double dx = px - r->pos[0][gj], dy = py - r->pos[1][gj], dz = pz - r->pos[2][gj];
                            double nd = nx * r->nrm[0][gj] + ny * r->nrm[1][gj] + nz * r->nrm[2][gj];
                            double arg = -dd2 * inv2s2 - (dx * dx + dy * dy + dz * dz) * inv2p2 - (1.0 - nd) * invn2;
                            double w = std::exp(arg);
                            sw += w;
                            sr += w * in[3 * j];
                            sg += w * in[3 * j + 1];
                            sb += w * in[3 * j + 2];
                        }
                    }
                }
                V3<double> f = {sr / sw, sg / sw, sb / sw};
                V3<double> o = style_apply<double>(style, depth, f);
                out[qi] = o.x;
                out[N + qi] = o.y;
                out[2 * N + qi] = o.z;
                if (filtered) {
                    filtered[qi] = f.x;
                    filtered[N + qi] = f.y;
                    filtered[2 * N + qi] = f.z;
                }
            }
        }
    }
}

// The FP64 filter above at the listed records only (idx: record indices within the depth), for
// checks at full image sizes: out / filtered are [3][n_idx].
void orc_pf_screen_filter_records_f64(const sty_pf_records *r, uint32_t depth, const sty_pf_screen_params *prm,
                                      const sty_style_program *style, const double *out_next, const uint64_t *idx,
                                      uint64_t n_idx, double *out, double *filtered) {
    const int W = r->width, H = r->height, S = r->spp, R = prm->radius;
    const size_t N = (size_t)W * H * S;
    const size_t dbase = (size_t)depth * N;
    const double inv2s2 = prm->sigma_pixel > 0 ? 1.0 / (2.0 * (double)prm->sigma_pixel * prm->sigma_pixel) : 0.0;
    const double inv2p2 = 1.0 / (2.0 * (double)prm->sigma_pos * prm->sigma_pos);
    const double invn2 = 1.0 / ((double)prm->sigma_nrm * prm->sigma_nrm);
    auto in_of = [&](size_t j, int c) {
        double v = r->rad[c][dbase + j];
        if (out_next) v += (double)r->thr[c][dbase + j] * out_next[c * N + j];
        return v;
    };
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t k = 0; k < (int64_t)n_idx; k++) {
        const size_t qi = idx[k];
        const size_t gq = dbase + qi;
        const int x = (int)((qi / S) % W), y = (int)(qi / S / W);
        double o3[3] = {0, 0, 0}, f3v[3] = {0, 0, 0};
        if (qi < N && r->valid[gq]) {
            const double px = r->pos[0][gq], py = r->pos[1][gq], pz = r->pos[2][gq];
            const double nx = r->nrm[0][gq], ny = r->nrm[1][gq], nz = r->nrm[2][gq];
            double sw = 0, sr = 0, sg = 0, sb = 0;
            for (int yy = std::max(0, y - R); yy <= std::min(H - 1, y + R); yy++)
                for (int xx = std::max(0, x - R); xx <= std::min(W - 1, x + R); xx++) {
                    const double dd2 = (double)(xx - x) * (xx - x) + (double)(yy - y) * (yy - y);
                    for (int t = 0; t < S; t++) {
                        const size_t j = ((size_t)yy * W + xx) * S + t;
                        const size_t gj = dbase + j;
                        if (!r->valid[gj]) continue;
                        const double dx = px - r->pos[0][gj], dy = py - r->pos[1][gj], dz = pz - r->pos[2][gj];
                        const double nd = nx * r->nrm[0][gj] + ny * r->nrm[1][gj] + nz * r->nrm[2][gj];
                        const double w = std::exp(-dd2 * inv2s2 - (dx * dx + dy * dy + dz * dz) * inv2p2 -
                                                  (1.0 - nd) * invn2);
                        sw += w;
                        sr += w * in_of(j, 0);
                        sg += w * in_of(j, 1);
                        sb += w * in_of(j, 2);
                    }
                }
            const V3<double> f = {sr / sw, sg / sw, sb / sw};
            const V3<double> o = style_apply<double>(style, depth, f);
            f3v[0] = f.x, f3v[1] = f.y, f3v[2] = f.z;
            o3[0] = o.x, o3[1] = o.y, o3[2] = o.z;
        }
        for (int c = 0; c < 3; c++) {
            out[c * n_idx + k] = o3[c];
            if (filtered) filtered[c * n_idx + k] = f3v[c];
        }
    }
}

// FP32 restatement (CPU baseline). Per candidate pixel row the partial sums are plain FP32 and
// are folded into Kahan-compensated totals (CompensatedSum, crates/akari_render/src/util/mod.rs:
// 337-356).
void orc_pf_screen_filter_depth_f32(const sty_pf_records *r, uint32_t depth,
                                    const sty_pf_screen_params *prm,
                                    const sty_style_program *style, const float *out_next,
                                    float *out, float *filtered, int32_t y0, int32_t y1) {
    const int W = r->width, H = r->height, S = r->spp, R = prm->radius;
    const size_t N = (size_t)W * H * S;
    const int d = (int)depth;
    const float inv2s2 = prm->sigma_pixel > 0 ? 1.0f / (2.0f * prm->sigma_pixel * prm->sigma_pixel) : 0.0f;
    const float inv2p2 = 1.0f / (2.0f * prm->sigma_pos * prm->sigma_pos);
    const float invn2 = 1.0f / (prm->sigma_nrm * prm->sigma_nrm);
    y0 = std::max(0, y0);
    y1 = std::min(H, y1);
    if (y1 <= y0) return;
    // candidate rows needed: [y0-R, y1+R)
    const int cy0 = std::max(0, y0 - R), cy1 = std::min(H, y1 + R);
    const size_t c0 = (size_t)cy0 * W * S, cn = (size_t)(cy1 - cy0) * W * S;
    std::vector<float> in(3 * cn);
    for (size_t k = 0; k < cn; k++) {
        size_t j = c0 + k, gj = (size_t)d * N + j;
        for (int c = 0; c < 3; c++) {
            float v = r->rad[c][gj];
            if (out_next) v += r->thr[c][gj] * out_next[c * N + j];
            in[3 * k + c] = v;
        }
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; y++) {
        for (int x = 0; x < W; x++) {
            for (int s = 0; s < S; s++) {
                size_t qi = ((size_t)y * W + x) * S + s;
                size_t gq = (size_t)d * N + qi;
                if (!r->valid[gq]) {
                    for (int c = 0; c < 3; c++) {
                        out[c * N + qi] = 0.0f;
                        if (filtered) filtered[c * N + qi] = 0.0f;
                    }
                    continue;
                }
                float px = r->pos[0][gq], py = r->pos[1][gq], pz = r->pos[2][gq];
                float nx = r->nrm[0][gq], ny = r->nrm[1][gq], nz = r->nrm[2][gq];
                float tot[4] = {0, 0, 0, 0}, cmp[4] = {0, 0, 0, 0};
                for (int yy = std::max(0, y - R); yy <= std::min(H - 1, y + R); yy++) {
                    float part[4] = {0, 0, 0, 0};
                    for (int xx = std::max(0, x - R); xx <= std::min(W - 1, x + R); xx++) {
                        float dd2 = (float)((xx - x) * (xx - x) + (yy - y) * (yy - y));
                        for (int t = 0; t < S; t++) {
                            size_t j = ((size_t)yy * W + xx) * S + t;
                            size_t gj = (size_t)d * N + j;
                            if (!r->valid[gj]) continue;
                            float dx = px - r->pos[0][gj], dy = py - r->pos[1][gj], dz = pz - r->pos[2][gj];
                            float nd = nx * r->nrm[0][gj] + ny * r->nrm[1][gj] + nz * r->nrm[2][gj];
                            float arg = -dd2 * inv2s2 - (dx * dx + dy * dy + dz * dz) * inv2p2 - (1.0f - nd) * invn2;
                            float w = std::exp(arg);
                            size_t k = j - c0;
                            part[0] += w;
                            part[1] += w * in[3 * k];
                            part[2] += w * in[3 * k + 1];
                            part[3] += w * in[3 * k + 2];
                        }
                    }
                    for (int c = 0; c < 4; c++) {  // Kahan update
                        float yv = part[c] - cmp[c];
                        float t = tot[c] + yv;
                        cmp[c] = (t - tot[c]) - yv;
                        tot[c] = t;
                    }
                }
                V3<float> f = {tot[1] / tot[0], tot[2] / tot[0], tot[3] / tot[0]};
                V3<float> o = style_apply<float>(style, depth, f);
                out[qi] = o.x;
                out[N + qi] = o.y;
                out[2 * N + qi] = o.z;
                if (filtered) {
                    filtered[qi] = f.x;
                    filtered[N + qi] = f.y;
                    filtered[2 * N + qi] = f.z;
                }
            }
        }
    }
}

// Pcg32 restated from crates/akari_render/src/sampler/mod.rs:82-123.
static inline uint32_t pcg_next(sty_pcg32 &g) {
    uint64_t old = g.state;
    g.state = old * 0x5851f42d4c957f2dULL + g.inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}

void orc_pcg32_streams(const uint64_t *seeds, uint64_t first_seq, uint64_t n, uint32_t draws,
                       uint32_t *out, sty_pcg32 *states) {
    for (uint64_t i = 0; i < n; i++) {
        sty_pcg32 g;
        g.state = 0;
        g.inc = ((first_seq + i) << 1) | 1u;  // set_seq_offset, mod.rs:94-100
        pcg_next(g);
        g.state += seeds[i];
        pcg_next(g);
        for (uint32_t k = 0; k < draws; k++) out[i * draws + k] = pcg_next(g);
        if (states) states[i] = g;
    }
}

// HashGridVar::get_cell / cell_pos_to_index, lm_path_filtering.rs:20-59 (float arithmetic).
void orc_hash_cells(const float *pts, uint64_t n, const float pmin[3], const float pmax[3],
                    const uint32_t res[3], uint32_t table_size, uint32_t *cell_xyz,
                    uint32_t *cell_index) {
    for (uint64_t i = 0; i < n; i++) {
        uint32_t c[3];
        for (int a = 0; a < 3; a++) {
            float p = (pts[3 * i + a] - pmin[a]) / (pmax[a] - pmin[a]);
            p = std::min(std::max(p, 0.0f), 1.0f);
            p = p * (float)res[a];
            uint32_t u = (uint32_t)p;
            c[a] = std::min(u, res[a] - 1u);
            if (cell_xyz) cell_xyz[3 * i + a] = c[a];
        }
        uint64_t h = ((uint64_t)c[0] * 73856093ULL) ^ ((uint64_t)c[1] * 19349663ULL) ^
                     ((uint64_t)c[2] * 83492791ULL);
        if (cell_index) cell_index[i] = (uint32_t)(h % (uint64_t)table_size);
    }
}

}  // extern "C"

// ---- adjoint of the screen filter + smoothed ramp (FP64) -------------------------------------
// Loss and gradient of the 36 parameters exactly as documented for sty_pf_adjoint in
// include/sty_gb300.h, evaluated in double: the forward restates the screen filter above with a
// single ramp node, the backward the chain rule written out in the CUDA file's header comment.
namespace {
struct AdjFwd {
    std::vector<double> f, D;  // f: 3 per query record; D: weight sum
    std::vector<double> img;   // 3 per pixel
};
double adj_forward(const sty_pf_records *r, uint32_t depth, int R, const double *prm, int nsteps,
                   const double *in_next, const double *target, AdjFwd *keep) {
    const int W = r->width, H = r->height, S = r->spp;
    const size_t N = (size_t)W * H * S;
    const int d = (int)depth;
    const double sx = prm[33], sp = prm[34], sn = prm[35];
    std::vector<double> in(3 * N);
    for (size_t j = 0; j < N; j++)
        for (int c = 0; c < 3; c++) {
            size_t g = (size_t)d * N + j;
            double v = r->rad[c][g];
            if (in_next) v += (double)r->thr[c][g] * in_next[c * N + j];
            in[3 * j + c] = v;
        }
    std::vector<double> f(3 * N, 0.0), D(N, 0.0), out(3 * N, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int s = 0; s < S; s++) {
                size_t qi = ((size_t)y * W + x) * S + s, gq = (size_t)d * N + qi;
                if (!r->valid[gq]) continue;
                double sw = 0, a[3] = {0, 0, 0};
                for (int yy = std::max(0, y - R); yy <= std::min(H - 1, y + R); yy++)
                    for (int xx = std::max(0, x - R); xx <= std::min(W - 1, x + R); xx++)
                        for (int t = 0; t < S; t++) {
                            size_t j = ((size_t)yy * W + xx) * S + t, gj = (size_t)d * N + j;
                            if (!r->valid[gj]) continue;
                            double rho = (double)(xx - x) * (xx - x) + (double)(yy - y) * (yy - y);
                            double d2 = 0, nn = 0;
                            for (int k = 0; k < 3; k++) {
                                double e = (double)r->pos[k][gq] - r->pos[k][gj];
                                d2 += e * e;
                                nn += (double)r->nrm[k][gq] * r->nrm[k][gj];
                            }
                            double w = std::exp(-rho / (2 * sx * sx) - d2 / (2 * sp * sp) - (1 - nn) / (sn * sn));
                            sw += w;
                            for (int c = 0; c < 3; c++) a[c] += w * in[3 * j + c];
                        }
                D[qi] = sw;
                double cl[3];
                for (int c = 0; c < 3; c++) {
                    f[3 * qi + c] = a[c] / sw;
                    cl[c] = std::min(std::max(f[3 * qi + c], 0.0), 1e5);
                }
                double lum = cl[0] * 0.2126 + cl[1] * 0.7152 + cl[2] * 0.0722;
                double prev[3] = {0, 0, 0};
                for (int k = 0; k < nsteps; k++) {
                    double sg = 1.0 / (1.0 + std::exp(-prm[0] * (lum - prm[1 + k])));
                    for (int c = 0; c < 3; c++) {
                        out[3 * qi + c] += sg * (prm[9 + 3 * k + c] - prev[c]);
                        prev[c] = prm[9 + 3 * k + c];
                    }
                }
            }
    std::vector<double> img(3 * (size_t)W * H, 0.0);
    double loss = 0;
    for (size_t p = 0; p < (size_t)W * H; p++)
        for (int c = 0; c < 3; c++) {
            double m = 0;
            for (int s = 0; s < S; s++) m += out[3 * (p * S + s) + c];
            m /= S;
            img[3 * p + c] = m;
            double e = m - target[3 * p + c];
            loss += e * e;
        }
    if (keep) {
        keep->f = std::move(f);
        keep->D = std::move(D);
        keep->img = std::move(img);
    }
    return loss;
}
}  // namespace

extern "C" {

double orc_pf_adjoint_loss_f64(const sty_pf_records *r, uint32_t depth, int32_t radius, const double *prm,
                               uint32_t n_steps, const double *in_next, const double *target) {
    return adj_forward(r, depth, radius, prm, (int)n_steps, in_next, target, nullptr);
}

double orc_pf_adjoint_f64(const sty_pf_records *r, uint32_t depth, int32_t R, const double *prm, uint32_t n_steps,
                          const double *in_next, const double *target, double *grad) {
    AdjFwd fw;
    const double loss = adj_forward(r, depth, R, prm, (int)n_steps, in_next, target, &fw);
    const int W = r->width, H = r->height, S = r->spp, d = (int)depth;
    const size_t N = (size_t)W * H * S;
    const double sx = prm[33], sp = prm[34], sn = prm[35], s = prm[0];
    std::vector<double> in(3 * N);
    for (size_t j = 0; j < N; j++)
        for (int c = 0; c < 3; c++) {
            size_t g = (size_t)d * N + j;
            double v = r->rad[c][g];
            if (in_next) v += (double)r->thr[c][g] * in_next[c * N + j];
            in[3 * j + c] = v;
        }
    std::vector<double> acc((size_t)H * 36, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; y++) {
        double *gs = &acc[(size_t)y * 36];
        for (int x = 0; x < W; x++)
            for (int q = 0; q < S; q++) {
                size_t qi = ((size_t)y * W + x) * S + q, gq = (size_t)d * N + qi;
                if (!r->valid[gq]) continue;
                const size_t p = (size_t)y * W + x;
                double g[3];
                for (int c = 0; c < 3; c++) g[c] = 2.0 * (fw.img[3 * p + c] - target[3 * p + c]) / S;
                const double *f = &fw.f[3 * qi];
                double cl[3];
                for (int c = 0; c < 3; c++) cl[c] = std::min(std::max(f[c], 0.0), 1e5);
                double lum = cl[0] * 0.2126 + cl[1] * 0.7152 + cl[2] * 0.0722;
                double dlum = 0, prev[3] = {0, 0, 0};
                std::vector<double> sgv(n_steps + 1, 0.0);
                for (uint32_t k = 0; k < n_steps; k++) {
                    double sg = 1.0 / (1.0 + std::exp(-s * (lum - prm[1 + k])));
                    sgv[k] = sg;
                    double dsg = sg * (1 - sg);
                    double gdc = 0;
                    for (int c = 0; c < 3; c++) {
                        gdc += g[c] * (prm[9 + 3 * k + c] - prev[c]);
                        prev[c] = prm[9 + 3 * k + c];
                    }
                    dlum += s * dsg * gdc;
                    gs[0] += dsg * (lum - prm[1 + k]) * gdc;
                    gs[1 + k] += -s * dsg * gdc;
                }
                for (uint32_t k = 0; k < n_steps; k++)
                    for (int c = 0; c < 3; c++) gs[9 + 3 * k + c] += g[c] * (sgv[k] - sgv[k + 1]);
                const double Yw[3] = {0.2126, 0.7152, 0.0722};
                double h[3];
                for (int c = 0; c < 3; c++) h[c] = (f[c] > 0 && f[c] < 1e5) ? dlum * Yw[c] : 0.0;
                const double hf = h[0] * f[0] + h[1] * f[1] + h[2] * f[2];
                double e0 = 0, e1 = 0, e2 = 0;
                for (int yy = std::max(0, y - R); yy <= std::min(H - 1, y + R); yy++)
                    for (int xx = std::max(0, x - R); xx <= std::min(W - 1, x + R); xx++)
                        for (int t = 0; t < S; t++) {
                            size_t j = ((size_t)yy * W + xx) * S + t, gj = (size_t)d * N + j;
                            if (!r->valid[gj]) continue;
                            double rho = (double)(xx - x) * (xx - x) + (double)(yy - y) * (yy - y);
                            double d2 = 0, nn = 0;
                            for (int k = 0; k < 3; k++) {
                                double ee = (double)r->pos[k][gq] - r->pos[k][gj];
                                d2 += ee * ee;
                                nn += (double)r->nrm[k][gq] * r->nrm[k][gj];
                            }
                            double w = std::exp(-rho / (2 * sx * sx) - d2 / (2 * sp * sp) - (1 - nn) / (sn * sn));
                            double tt = w * (h[0] * in[3 * j] + h[1] * in[3 * j + 1] + h[2] * in[3 * j + 2] - hf);
                            e0 += tt * rho;
                            e1 += tt * d2;
                            e2 += tt * (1 - nn);
                        }
                const double iD = 1.0 / fw.D[qi];
                gs[33] += e0 * iD / (sx * sx * sx);
                gs[34] += e1 * iD / (sp * sp * sp);
                gs[35] += 2.0 * e2 * iD / (sn * sn * sn);
            }
    }
    for (int k = 0; k < 36; k++) {
        double t = 0;
        for (int y = 0; y < H; y++) t += acc[(size_t)y * 36 + k];
        grad[k] = t;
    }
    return loss;
}

}  // extern "C"

extern "C" double orc_pf_adjoint_image_f64(const sty_pf_records *r, uint32_t depth, int32_t radius, const double *prm,
                                           uint32_t n_steps, const double *in_next, double *img) {
    AdjFwd fw;
    std::vector<double> zero(3 * (size_t)r->width * r->height, 0.0);
    double l = adj_forward(r, depth, radius, prm, (int)n_steps, in_next, zero.data(), &fw);
    std::copy(fw.img.begin(), fw.img.end(), img);
    return l;
}

// ---- closest hit by brute force (watertight ray/triangle test of Woop, Benthin and Wald 2013, the
// published algorithm, in f32 with the double fallback on exact zeros); ties -> lowest id ----------
extern "C" void orc_closest_hit(const float *pos, uint32_t n_tris, const float *rays, uint64_t n, uint32_t *prim,
                                float *tout, float *bary) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const float *r = rays + 8 * i;
        const float o[3] = {r[0], r[1], r[2]}, d[3] = {r[3], r[4], r[5]};
        const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
        int kz = 0;
        if (ay > ax) kz = 1;
        if (az > (kz == 0 ? ax : ay)) kz = 2;
        int kx = kz + 1 == 3 ? 0 : kz + 1, ky = kx + 1 == 3 ? 0 : kx + 1;
        if (d[kz] < 0.0f) std::swap(kx, ky);
        const float Sx = d[kx] / d[kz], Sy = d[ky] / d[kz], Sz = 1.0f / d[kz];
        float best = r[7], bb1 = 0, bb2 = 0;
        uint32_t bp = 0xffffffffu;
        for (uint32_t t = 0; t < n_tris; t++) {
            const float *p = pos + 9 * (size_t)t;
            float A[3], B[3], C[3];
            for (int a = 0; a < 3; a++) {
                A[a] = p[a] - o[a];
                B[a] = p[3 + a] - o[a];
                C[a] = p[6 + a] - o[a];
            }
            const float Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
            const float Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
            const float Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
            float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
            if (U == 0.0f || V == 0.0f || W == 0.0f) {
                U = (float)((double)Cx * By - (double)Cy * Bx);
                V = (float)((double)Ax * Cy - (double)Ay * Cx);
                W = (float)((double)Bx * Ay - (double)By * Ax);
            }
            if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) continue;
            const float det = (U + V) + W;
            if (det == 0.0f) continue;
            const float Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
            const float T = ((U * Az) + (V * Bz)) + (W * Cz);
            const float tt = T / det;
            if (!(tt > r[6])) continue;
            if (tt > best || (tt == best && t >= bp)) continue;
            best = tt;
            bb1 = V / det;
            bb2 = W / det;
            bp = t;
        }
        prim[i] = bp;
        if (tout) tout[i] = best;
        if (bary) {
            bary[2 * i] = bb1;
            bary[2 * i + 1] = bb2;
        }
    }
}

// ---- independent CPU path tracer (FP64 radiance, brute-force f32 watertight hits) ---------------
// The textbook estimator with next-event estimation and balance-heuristic MIS, restated from the
// reference's per-vertex terms (handle_surface_light lm_path_filtering.rs:388-426, sample_light
// :1261-1316, the BSDF sample :1180-1211) for diffuse surfaces. With black emitters it is the
// expectation the NL-PF estimator converges to when every vertex only reuses itself.
namespace {
struct PtScene {
    const float *pos;
    const uint32_t *mat;
    uint32_t n;
    const float *albedo;    // 3 per material
    const float *emission;  // 3 per material
    std::vector<uint32_t> lights;
    std::vector<double> cdf;
    std::vector<double> area;
    std::vector<std::array<double, 3>> nrm;
};
inline uint32_t pcg_u32(sty_pcg32 &g) { return pcg_next(g); }
inline double u01(sty_pcg32 &g) { return (double)((float)pcg_u32(g) * 2.3283064e-10f); }
inline uint32_t hit_bf(const PtScene &s, const double o[3], const double d[3], double tmax, uint32_t ex0,
                       uint32_t ex1, double *tout, double *b1o, double *b2o) {
    // double-precision Moller-Trumbore (the oracle only needs unbiased shading, not bit parity)
    uint32_t best = 0xffffffffu;
    double bt = tmax;
    for (uint32_t t = 0; t < s.n; t++) {
        if (t == ex0 || t == ex1) continue;
        const float *p = s.pos + 9 * (size_t)t;
        double e1[3], e2[3], pv[3], tv[3], qv[3];
        for (int a = 0; a < 3; a++) {
            e1[a] = (double)p[3 + a] - p[a];
            e2[a] = (double)p[6 + a] - p[a];
        }
        pv[0] = d[1] * e2[2] - d[2] * e2[1];
        pv[1] = d[2] * e2[0] - d[0] * e2[2];
        pv[2] = d[0] * e2[1] - d[1] * e2[0];
        const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
        if (std::fabs(det) < 1e-14) continue;
        const double inv = 1.0 / det;
        for (int a = 0; a < 3; a++) tv[a] = o[a] - p[a];
        const double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
        if (u < 0 || u > 1) continue;
        qv[0] = tv[1] * e1[2] - tv[2] * e1[1];
        qv[1] = tv[2] * e1[0] - tv[0] * e1[2];
        qv[2] = tv[0] * e1[1] - tv[1] * e1[0];
        const double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
        if (v < 0 || u + v > 1) continue;
        const double tt = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
        if (tt > 1e-7 && tt < bt) {
            bt = tt;
            best = t;
            *b1o = u;
            *b2o = v;
        }
    }
    *tout = bt;
    return best;
}
}  // namespace

extern "C" void orc_path_trace(const float *pos, const uint32_t *mat, uint32_t n_tris, const float *albedo,
                               const float *emission, const float *cam /* eye3 target3 up3 fov W H radius */,
                               uint32_t spp, uint32_t max_depth, uint64_t seed, double *img) {
    PtScene s;
    s.pos = pos;
    s.mat = mat;
    s.n = n_tris;
    s.albedo = albedo;
    s.emission = emission;
    s.area.resize(n_tris);
    s.nrm.resize(n_tris);
    double tot = 0;
    std::vector<double> w;
    for (uint32_t t = 0; t < n_tris; t++) {
        const float *p = pos + 9 * (size_t)t;
        double e1[3], e2[3];
        for (int a = 0; a < 3; a++) {
            e1[a] = (double)p[3 + a] - p[a];
            e2[a] = (double)p[6 + a] - p[a];
        }
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        s.area[t] = 0.5 * l;
        s.nrm[t] = {c[0] / l, c[1] / l, c[2] / l};
        const float *em = emission + 3 * (size_t)mat[t];
        double lum = 0.2126 * em[0] + 0.7152 * em[1] + 0.0722 * em[2];
        if (lum > 0) {
            s.lights.push_back(t);
            w.push_back(lum * s.area[t]);
            tot += lum * s.area[t];
        }
    }
    s.cdf.assign(w.size() + 1, 0.0);
    for (size_t k = 0; k < w.size(); k++) s.cdf[k + 1] = s.cdf[k] + w[k] / tot;
    const uint32_t W = (uint32_t)cam[10], H = (uint32_t)cam[11];
    double f[3], r[3], u[3];
    for (int a = 0; a < 3; a++) f[a] = cam[3 + a] - cam[a];
    double l = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (int a = 0; a < 3; a++) f[a] /= l;
    r[0] = f[1] * cam[8] - f[2] * cam[7];
    r[1] = f[2] * cam[6] - f[0] * cam[8];
    r[2] = f[0] * cam[7] - f[1] * cam[6];
    l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int a = 0; a < 3; a++) r[a] /= l;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    const double th = std::tan(cam[9] * 0.5 * M_PI / 180.0), asp = (double)W / H, rad = cam[12];
#pragma omp parallel for schedule(dynamic, 1)
    for (int py = 0; py < (int)H; py++)
        for (uint32_t px = 0; px < W; px++) {
            double acc[3] = {0, 0, 0};
            for (uint32_t sp = 0; sp < spp; sp++) {
                sty_pcg32 g;
                const uint64_t idx = ((uint64_t)py * W + px) * spp + sp;
                g.state = 0;
                g.inc = (idx << 1) | 1u;
                pcg_next(g);
                g.state += seed * 0x9E3779B97F4A7C15ULL + idx * 0xD1B54A32D192ED03ULL;
                pcg_next(g);
                const double fx = px + 0.5 + (u01(g) - 0.5) * rad, fy = py + 0.5 + (u01(g) - 0.5) * rad;
                const double sx = (2 * fx / W - 1) * th * asp, sy = (1 - 2 * fy / H) * th;
                double o[3] = {cam[0], cam[1], cam[2]}, d[3];
                for (int a = 0; a < 3; a++) d[a] = f[a] + r[a] * sx + u[a] * sy;
                l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (int a = 0; a < 3; a++) d[a] /= l;
                double thr[3] = {1, 1, 1}, prev_pdf = 0, prev_p[3] = {o[0], o[1], o[2]};
                uint32_t ex = 0xffffffffu;
                for (uint32_t depth = 0; depth <= max_depth; depth++) {
                    double t, b1, b2;
                    const uint32_t hit = hit_bf(s, o, d, 1e30, ex, ex, &t, &b1, &b2);
                    if (hit == 0xffffffffu) break;
                    double p[3];
                    for (int a = 0; a < 3; a++) p[a] = o[a] + t * d[a];
                    const auto &n = s.nrm[hit];
                    const float *em = emission + 3 * (size_t)mat[hit];
                    const float *alb = albedo + 3 * (size_t)mat[hit];
                    const double ndd = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
                    if (em[0] > 0 || em[1] > 0 || em[2] > 0) {
                        double mis = 1.0;
                        if (depth > 0) {
                            double sel = 0;
                            for (size_t k = 0; k < s.lights.size(); k++)
                                if (s.lights[k] == hit) sel = s.cdf[k + 1] - s.cdf[k];
                            double wv[3] = {p[0] - prev_p[0], p[1] - prev_p[1], p[2] - prev_p[2]};
                            double d2 = wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2];
                            double lp = sel / s.area[hit] * d2 / std::max(std::fabs(ndd), 1e-6);
                            mis = prev_pdf / (prev_pdf + lp);
                        }
                        if (ndd < 0)
                            for (int c = 0; c < 3; c++) acc[c] += thr[c] * em[c] * mis;
                    }
                    if (depth == max_depth) break;
                    // shading frame: flat, normal facing the incoming direction side as in the GPU path
                    double ns[3] = {n[0], n[1], n[2]};
                    const double wo[3] = {-d[0], -d[1], -d[2]};
                    const double co = ns[0] * wo[0] + ns[1] * wo[1] + ns[2] * wo[2];
                    // NEE
                    {
                        const double ux = u01(g), uy = u01(g), uz = u01(g);
                        size_t k = 0;
                        while (k + 1 < s.lights.size() && !(s.cdf[k + 1] > ux)) k++;
                        if (!s.lights.empty()) {
                            const uint32_t lt = s.lights[k];
                            const double sel = s.cdf[k + 1] - s.cdf[k];
                            double bx, by;
                            if (uy < uz) {
                                bx = uy / 2;
                                by = uz - bx;
                            } else {
                                by = uz / 2;
                                bx = uy - by;
                            }
                            const float *lp = pos + 9 * (size_t)lt;
                            double q[3];
                            for (int a = 0; a < 3; a++) q[a] = (1 - bx - by) * lp[a] + bx * lp[3 + a] + by * lp[6 + a];
                            double wi[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
                            const double d2 = wi[0] * wi[0] + wi[1] * wi[1] + wi[2] * wi[2];
                            const double dist = std::sqrt(d2);
                            for (int a = 0; a < 3; a++) wi[a] /= dist;
                            const auto &ln = s.nrm[lt];
                            const double lnw = ln[0] * wi[0] + ln[1] * wi[1] + ln[2] * wi[2];
                            const double ci = ns[0] * wi[0] + ns[1] * wi[1] + ns[2] * wi[2];
                            const double lpdf = sel / s.area[lt] * d2 / std::fabs(lnw);
                            if (lnw < 0 && co * ci > 0 && std::isfinite(lpdf)) {
                                double tt, c1, c2;
                                const uint32_t blk = hit_bf(s, p, wi, dist * (1 - 1e-3), hit, lt, &tt, &c1, &c2);
                                if (blk == 0xffffffffu) {
                                    const double bp = std::fabs(ci) / M_PI;
                                    const double wmis = lpdf / (lpdf + bp);
                                    const float *lem = emission + 3 * (size_t)mat[lt];
                                    for (int c = 0; c < 3; c++)
                                        acc[c] += thr[c] * alb[c] / M_PI * std::fabs(ci) * lem[c] * wmis / lpdf;
                                }
                            }
                        }
                    }
                    // BSDF sample (cosine hemisphere around the normal on wo's side)
                    const double usel = u01(g), u0 = u01(g), u1 = u01(g);
                    (void)usel;
                    const double rr = std::sqrt(u0), ph = 2 * M_PI * u1;
                    double lx = rr * std::cos(ph), ly = rr * std::sin(ph), lz = std::sqrt(std::max(0.0, 1 - lx * lx - ly * ly));
                    double tx[3];
                    if (std::fabs(ns[0]) > std::fabs(ns[1])) {
                        double il = 1.0 / std::sqrt(ns[0] * ns[0] + ns[2] * ns[2]);
                        tx[0] = -ns[2] * il; tx[1] = 0; tx[2] = ns[0] * il;
                    } else {
                        double il = 1.0 / std::sqrt(ns[1] * ns[1] + ns[2] * ns[2]);
                        tx[0] = 0; tx[1] = ns[2] * il; tx[2] = -ns[1] * il;
                    }
                    double sx3[3] = {ns[1] * tx[2] - ns[2] * tx[1], ns[2] * tx[0] - ns[0] * tx[2], ns[0] * tx[1] - ns[1] * tx[0]};
                    if (co < 0) lz = -lz;
                    double wi[3];
                    for (int a = 0; a < 3; a++) wi[a] = tx[a] * lx + sx3[a] * ly + ns[a] * lz;
                    const double pdf = std::fabs(lz) / M_PI;
                    if (!(pdf > 0)) break;
                    for (int c = 0; c < 3; c++) thr[c] *= alb[c];  // f cos / pdf = albedo
                    prev_pdf = pdf;
                    for (int a = 0; a < 3; a++) {
                        prev_p[a] = p[a];
                        o[a] = p[a];
                        d[a] = wi[a];
                    }
                    ex = hit;
                }
            }
            for (int c = 0; c < 3; c++) img[3 * ((size_t)py * W + px) + c] = acc[c] / spp;
        }
}

// ---- branching path tracer (branching_pt.rs), recursive FP64 restatement -------------------------
// Test infrastructure for sty_brpt_render: the same tree (inner_samples at the k-th rough vertex,
// 1 at smooth vertices, none at max_depth), the same estimator (style(Le + mean over branches of
// (direct + throughput * child radiance * child emission MIS))), the same sampling keys (camera on
// (seed, repeat, pixel), children on (parent key, branch)) and draws (2 camera; per branch 3 light
// + 3 BSDF, float u = u32 * 2^-32 as IndependentSampler::next_1d), the same light CDF (FP32
// luminance x area) and sampling maps (uniform_sample_triangle, polar disk -> cosine hemisphere in
// the frame of frame_from_n). Diffuse surfaces only; FP64 geometry and brute-force FP64 hits, so a
// ray grazing an edge can hit differently than the GPU's FP32 BVH.
namespace {
inline uint64_t smix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
inline sty_pcg32 key_stream(uint64_t key) {
    sty_pcg32 g;
    g.state = 0;
    g.inc = (key << 1) | 1ull;
    pcg_next(g);
    g.state += smix64(key);
    pcg_next(g);
    return g;
}
inline uint32_t style_idx(uint32_t f) { return (f & 8u) ? 3u : (f & 4u) ? 2u : (f & 2u) ? 1u : 0u; }
inline uint32_t flags_after(const sty_scene_material &m, uint32_t f) {
    if (m.set_style < 0) return f;
    return (f & 1u) | (m.set_style == 1 ? 2u : m.set_style == 2 ? 4u : m.set_style == 3 ? 8u : 0u);
}
struct BrScene {
    PtScene pt;
    const sty_scene_material *mats;
    std::vector<float> cdf;  // FP32 like the GPU scene's
    const sty_style_program *progs;
    uint32_t n_progs, max_depth, n_levels;
    const uint32_t *inner;
};
typedef std::array<double, 3> D3;
inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// emitted radiance at a hit of triangle `prim` by direction d and its balance weight against the
// light pdf seen from prev_p (handle_surface_light)
inline bool br_emitter(const BrScene &s, uint32_t prim, const double *q, const double *d, uint32_t depth,
                       const double *prev_p, double prev_pdf, D3 &le, double &mis) {
    const sty_scene_material &m = s.mats[s.pt.mat[prim]];
    le = {0, 0, 0};
    mis = 1.0;
    if (!(m.emission[0] > 0 || m.emission[1] > 0 || m.emission[2] > 0)) return false;
    const auto &n = s.pt.nrm[prim];
    if (n[0] * d[0] + n[1] * d[1] + n[2] * d[2] < 0) le = {m.emission[0], m.emission[1], m.emission[2]};
    if (depth > 0) {
        double sel = 0;
        for (size_t k = 0; k < s.pt.lights.size(); k++)
            if (s.pt.lights[k] == prim) sel = (double)s.cdf[k + 1] - (double)s.cdf[k];
        const double w[3] = {q[0] - prev_p[0], q[1] - prev_p[1], q[2] - prev_p[2]};
        const double d2 = dot3(w, w), dl = std::sqrt(d2);
        const double cw = std::fabs((n[0] * w[0] + n[1] * w[1] + n[2] * w[2]) / dl);
        const double lp = sel / s.pt.area[prim] * d2 / std::max(cw, 1e-6);
        mis = prev_pdf / (prev_pdf + lp);
    }
    return true;
}

D3 br_radiance(const BrScene &s, uint32_t depth, const double *p, uint32_t prim, const double *wo, uint32_t flags,
               uint32_t ab, uint64_t key, D3 le) {
    const sty_scene_material &m = s.mats[s.pt.mat[prim]];
    const auto &ngv = s.pt.nrm[prim];
    const double ng[3] = {ngv[0], ngv[1], ngv[2]};
    D3 li = le;
    if (depth + 1 <= s.max_depth) {
        const bool rough = (m.kind == STY_MAT_DIFFUSE ? 1.0f : m.alpha) > 0.01f;
        const uint32_t n = rough ? (ab < s.n_levels ? s.inner[ab] : 1u) : 1u;
        const uint32_t nf = flags_after(m, flags), ab2 = ab + (rough ? 1u : 0u);
        const double co = dot3(wo, ng);
        D3 sum = {0, 0, 0};
        for (uint32_t b = 0; b < n; b++) {
            const uint64_t ck = smix64(key ^ (0x9e3779b97f4a7c15ull * (uint64_t)(b + 1u)));
            sty_pcg32 g = key_stream(ck);
            // NEE
            const float ux = (float)pcg_next(g) * 2.3283064e-10f, uy = (float)pcg_next(g) * 2.3283064e-10f,
                        uz = (float)pcg_next(g) * 2.3283064e-10f;
            if (!s.pt.lights.empty()) {
                uint32_t lo = 0, hi = (uint32_t)s.pt.lights.size() - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (s.cdf[mid + 1] > ux) hi = mid;
                    else lo = mid + 1;
                }
                const uint32_t lt = s.pt.lights[lo];
                const double sel = (double)s.cdf[lo + 1] - (double)s.cdf[lo];
                double bx, by;
                if (uy < uz) {
                    bx = uy / 2.0;
                    by = uz - bx;
                } else {
                    by = uz / 2.0;
                    bx = uy - by;
                }
                const float *lp = s.pt.pos + 9 * (size_t)lt;
                double q[3], wi[3];
                for (int a = 0; a < 3; a++) q[a] = (1 - bx - by) * lp[a] + bx * lp[3 + a] + by * lp[6 + a];
                for (int a = 0; a < 3; a++) wi[a] = q[a] - p[a];
                const double d2 = dot3(wi, wi);
                if (d2 > 0) {
                    const double dist = std::sqrt(d2);
                    for (int a = 0; a < 3; a++) wi[a] /= dist;
                    const auto &ln = s.pt.nrm[lt];
                    const double lnw = ln[0] * wi[0] + ln[1] * wi[1] + ln[2] * wi[2];
                    const double lpdf = sel / s.pt.area[lt] * d2 / std::fabs(lnw);
                    const sty_scene_material &lm = s.mats[s.pt.mat[lt]];
                    V3<double> lli = {0, 0, 0};
                    if (lnw < 0) lli = {lm.emission[0], lm.emission[1], lm.emission[2]};
                    if (std::isfinite(lpdf) && lpdf > 0) {
                        if (!(nf & 1u)) {
                            const int32_t pi = lm.style[style_idx(nf)];
                            if (pi >= 0 && (uint32_t)pi < s.n_progs)
                                lli = style_apply<double>(&s.progs[pi], depth + 1, lli, v3(q[0], q[1], q[2]));
                        }
                        double tt, c1, c2;
                        const uint32_t blk = hit_bf(s.pt, p, wi, dist * (1 - 1e-3), prim, lt, &tt, &c1, &c2);
                        const double ci = dot3(wi, ng);
                        if (blk == 0xffffffffu && co * ci >= 0) {
                            const double bp = std::fabs(ci) / M_PI, w = lpdf / (lpdf + bp) / lpdf;
                            const double lv[3] = {lli.x, lli.y, lli.z};
                            for (int c = 0; c < 3; c++) sum[c] += lv[c] * m.albedo[c] * bp * w;
                        }
                    }
                }
            }
            // BSDF sample: cosine hemisphere (polar disk) in frame_from_n(ng), flipped to wo's side
            const float usel = (float)pcg_next(g) * 2.3283064e-10f, u0 = (float)pcg_next(g) * 2.3283064e-10f,
                        u1 = (float)pcg_next(g) * 2.3283064e-10f;
            (void)usel;
            const double r = std::sqrt((double)u0), ph = (double)u1 * 2.0 * M_PI;
            const double lx = r * std::cos(ph), ly = r * std::sin(ph);
            double lz = std::sqrt(std::max(0.0, 1 - lx * lx - ly * ly));
            double t[3];
            if (std::fabs(ng[0]) > std::fabs(ng[1])) {
                const double il = 1.0 / std::sqrt(ng[0] * ng[0] + ng[2] * ng[2]);
                t[0] = -ng[2] * il; t[1] = 0; t[2] = ng[0] * il;
            } else {
                const double il = 1.0 / std::sqrt(ng[1] * ng[1] + ng[2] * ng[2]);
                t[0] = 0; t[1] = ng[2] * il; t[2] = -ng[1] * il;
            }
            const double sv[3] = {ng[1] * t[2] - ng[2] * t[1], ng[2] * t[0] - ng[0] * t[2], ng[0] * t[1] - ng[1] * t[0]};
            if (!(co * lz >= 0)) lz = -lz;
            double wi[3];
            for (int a = 0; a < 3; a++) wi[a] = t[a] * lx + sv[a] * ly + ng[a] * lz;
            const double pdf = std::fabs(lz) / M_PI;
            if (!(pdf > 0)) continue;
            double tt, b1, b2;
            const uint32_t h = hit_bf(s.pt, p, wi, 1e30, prim, prim, &tt, &b1, &b2);
            if (h == 0xffffffffu) continue;
            double q[3];
            for (int a = 0; a < 3; a++) q[a] = p[a] + tt * wi[a];
            D3 cle;
            double cmis;
            br_emitter(s, h, q, wi, depth + 1, p, pdf, cle, cmis);
            const double cwo[3] = {-wi[0], -wi[1], -wi[2]};
            const D3 cl = br_radiance(s, depth + 1, q, h, cwo, nf, ab2, ck, cle);
            for (int c = 0; c < 3; c++) sum[c] += m.albedo[c] * cl[c] * cmis;  // f cos / pdf = albedo
        }
        for (int c = 0; c < 3; c++) li[c] += sum[c] / n;
    }
    if (!(flags & 1u)) {
        const int32_t pi = m.style[style_idx(flags)];
        if (pi >= 0 && (uint32_t)pi < s.n_progs) {
            const V3<double> o = style_apply<double>(&s.progs[pi], depth, v3(li[0], li[1], li[2]), v3(p[0], p[1], p[2]));
            li = {o.x, o.y, o.z};
        }
    }
    return li;
}
}  // namespace

extern "C" void orc_brpt(const float *pos, const uint32_t *mat, uint32_t n_tris, const sty_scene_material *mats,
                         const float *cam /* eye3 target3 up3 fov W H radius */, const sty_style_program *progs,
                         uint32_t n_progs, uint32_t max_depth, const uint32_t *inner, uint32_t n_levels,
                         uint32_t repeats, uint32_t first_repeat, uint64_t seed, double *img) {
    BrScene s;
    s.pt.pos = pos;
    s.pt.mat = mat;
    s.pt.n = n_tris;
    s.pt.area.resize(n_tris);
    s.pt.nrm.resize(n_tris);
    s.mats = mats;
    s.progs = progs;
    s.n_progs = n_progs;
    s.max_depth = max_depth;
    s.n_levels = n_levels;
    s.inner = inner;
    std::vector<double> lw;
    for (uint32_t t = 0; t < n_tris; t++) {
        const float *p = pos + 9 * (size_t)t;
        double e1[3], e2[3];
        for (int a = 0; a < 3; a++) {
            e1[a] = (double)p[3 + a] - p[a];
            e2[a] = (double)p[6 + a] - p[a];
        }
        const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        s.pt.area[t] = (double)(float)(0.5 * l);
        s.pt.nrm[t] = {c[0] / l, c[1] / l, c[2] / l};
        const float *em = mats[mat[t]].emission;
        const double lum = 0.2126 * em[0] + 0.7152 * em[1] + 0.0722 * em[2];
        if (lum > 0 && s.pt.area[t] > 0) {
            s.pt.lights.push_back(t);
            lw.push_back(lum * s.pt.area[t]);
        }
    }
    s.cdf.assign(lw.size() + 1, 0.0f);
    double tot = 0, acc = 0;
    for (double w : lw) tot += w;
    for (size_t k = 0; k < lw.size(); k++) {
        acc += lw[k];
        s.cdf[k + 1] = (float)(acc / tot);
    }
    if (!lw.empty()) s.cdf.back() = 1.0f;
    const uint32_t W = (uint32_t)cam[10], H = (uint32_t)cam[11];
    double f[3], r[3], u[3];
    for (int a = 0; a < 3; a++) f[a] = cam[3 + a] - cam[a];
    double l = std::sqrt(dot3(f, f));
    for (int a = 0; a < 3; a++) f[a] /= l;
    r[0] = f[1] * cam[8] - f[2] * cam[7];
    r[1] = f[2] * cam[6] - f[0] * cam[8];
    r[2] = f[0] * cam[7] - f[1] * cam[6];
    l = std::sqrt(dot3(r, r));
    for (int a = 0; a < 3; a++) r[a] /= l;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    const double th = std::tan(cam[9] * 0.5 * M_PI / 180.0), asp = (double)W / H, rad = cam[12];
    std::fill(img, img + 3 * (size_t)W * H, 0.0);
    for (uint32_t rep = 0; rep < repeats; rep++) {
        const uint64_t rkey = smix64(smix64(seed ^ 0x4252505400000000ull) + (uint64_t)first_repeat + rep);
#pragma omp parallel for schedule(dynamic, 1)
        for (int py = 0; py < (int)H; py++)
            for (uint32_t px = 0; px < W; px++) {
                const uint32_t pid = (uint32_t)py * W + px;
                const uint64_t key = smix64(rkey + pid);
                sty_pcg32 g = key_stream(key);
                const double u0 = (float)pcg_next(g) * 2.3283064e-10f, u1 = (float)pcg_next(g) * 2.3283064e-10f;
                const double fx = px + 0.5 + (u0 - 0.5) * rad, fy = py + 0.5 + (u1 - 0.5) * rad;
                const double sx = (2 * fx / W - 1) * th * asp, sy = (1 - 2 * fy / H) * th;
                double d[3];
                for (int a = 0; a < 3; a++) d[a] = f[a] + r[a] * sx + u[a] * sy;
                const double dl = std::sqrt(dot3(d, d));
                for (int a = 0; a < 3; a++) d[a] /= dl;
                const double o[3] = {cam[0], cam[1], cam[2]};
                double tt, b1, b2;
                const uint32_t h = hit_bf(s.pt, o, d, 1e30, 0xffffffffu, 0xffffffffu, &tt, &b1, &b2);
                if (h == 0xffffffffu) continue;
                double q[3];
                for (int a = 0; a < 3; a++) q[a] = o[a] + tt * d[a];
                D3 le;
                double mis;
                br_emitter(s, h, q, d, 0, o, 0.0, le, mis);
                const double wo[3] = {-d[0], -d[1], -d[2]};
                const D3 c = br_radiance(s, 0, q, h, wo, 0u, 0u, key, le);
                for (int k = 0; k < 3; k++) img[3 * (size_t)pid + k] += c[k] / repeats;
            }
    }
}

// ---- the principled BSDF (principled.rs:118-330), FP64 restatement -------------------------------
// Test infrastructure for STY_MAT_PRINCIPLED: the same closure (layers, blend modes, lobe choice),
// microfacet lobes, Fresnel terms and ggx_dielectric_s table (the mean of f/pdf of a unit-colour
// dielectric GGX reflection over the visible-normal sample, by the same 256 x 256 midpoint rule in
// u), all in FP64.
namespace {
typedef std::array<double, 3> P3;
inline P3 p3(double x, double y, double z) { return {x, y, z}; }
inline P3 padd(P3 a, P3 b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline P3 pmul(P3 a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
inline double pdot(P3 a, P3 b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline P3 pcross(P3 a, P3 b) { return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}; }
inline P3 pnorm(P3 a) { return pmul(a, 1.0 / std::sqrt(pdot(a, a))); }
inline bool psame(P3 a, P3 b) { return a[2] * b[2] > 0; }
inline double plerp(double a, double b, double t) { return a + (b - a) * t; }
const double kPiD = 3.14159265358979323846;

double p_d(P3 wh, double a) {
    const double c2 = wh[2] * wh[2], s2 = std::max(0.0, 1 - c2), tan2 = s2 / c2, e = tan2 / (a * a);
    const double inv = kPiD * a * a * c2 * c2 * (1 + e) * (1 + e);
    if (!std::isfinite(tan2) || !std::isfinite(inv) || inv == 0) return 0;
    return 1 / inv;
}
double p_lambda(P3 w, double a) {
    const double c2 = w[2] * w[2], s2 = std::max(0.0, 1 - c2);
    const double at = std::fabs(std::sqrt(s2) / w[2]);
    return std::isfinite(at) ? (-1 + std::sqrt(1 + a * a * at * at)) * 0.5 : 0.0;
}
double p_vpdf(P3 wo, P3 wh, double a) {
    return p_d(wh, a) / (1 + p_lambda(wo, a)) * std::fabs(pdot(wo, wh)) / std::fabs(wo[2]);
}
P3 p_sample_wh(P3 w, double a, double u0, double u1) {
    P3 wh = pnorm(p3(a * w[0], a * w[1], w[2]));
    if (wh[2] < 0) wh = pmul(wh, -1);
    const P3 t1 = wh[2] < 0.99999 ? pnorm(pcross(p3(0, 0, 1), wh)) : p3(1, 0, 0);
    const P3 t2 = pnorm(pcross(wh, t1));
    const double r = std::sqrt(u0), ph = u1 * 2 * kPiD;
    double px = r * std::cos(ph), py = r * std::sin(ph);
    const double h = std::sqrt(1 - px * px);
    py = h + (py - h) * ((1 + wh[2]) * 0.5);
    const double pz = std::sqrt(std::max(1 - (px * px + py * py), 0.0));
    const P3 nh = padd(padd(pmul(t1, px), pmul(t2, py)), pmul(wh, pz));
    return pnorm(p3(a * nh[0], a * nh[1], std::max(nh[2], 1e-6)));
}
inline P3 p_reflect(P3 w, P3 n) { return padd(pmul(n, 2 * pdot(w, n)), pmul(w, -1)); }
bool p_refract(P3 w, P3 n, double eta, P3 *wt) {
    double ci = pdot(w, n);
    const double e = ci >= 0 ? eta : 1 / eta;
    const P3 nn = ci >= 0 ? n : pmul(n, -1);
    ci = std::fabs(ci);
    const double s2t = std::max(1 - ci * ci, 0.0) / (e * e);
    if (s2t >= 1) return false;
    *wt = padd(pmul(w, -1 / e), pmul(nn, ci / e - std::sqrt(1 - s2t)));
    return true;
}
double p_fr_diel(double ci, double eta) {
    ci = std::min(std::max(ci, -1.0), 1.0);
    const double e = ci > 0 ? eta : 1 / eta;
    ci = std::fabs(ci);
    const double s2t = (1 - ci * ci) / (e * e);
    if (s2t >= 1) return 1;
    const double ct = std::sqrt(std::max(1 - s2t, 0.0));
    const double a = (e * ci - ct) / (e * ci + ct), b = (ci - e * ct) / (ci + e * ct);
    return std::min(std::max((a * a + b * b) * 0.5, 0.0), 1.0);
}
double p_fr_cond(double ci, double n, double k) {
    typedef std::complex<double> cd;
    ci = std::min(std::max(ci, 0.0), 0.999);
    const cd eta(n, k), s2t = cd(1 - ci * ci, 0) / (eta * eta), ct = std::sqrt(cd(1, 0) - s2t);
    const cd a = (eta * ci - ct) / (eta * ci + ct), b = (cd(ci, 0) - eta * ct) / (cd(ci, 0) + eta * ct);
    return (std::norm(a) + std::norm(b)) * 0.5;
}
inline double p_ior_from_f0(double f0) {
    const double s = std::sqrt(std::min(std::max(f0, 0.0), 0.99));
    return (1 + s) / (1 - s);
}
double p_albedo_sample(double rough, double mu, double ior, double u0, double u1) {
    const double a = std::max(rough * rough, 1e-4);
    const P3 wo = p3(std::sqrt(1 - mu * mu), 0, mu), wh = p_sample_wh(wo, a, u0, u1), wi = p_reflect(wo, wh);
    if (!psame(wo, wi)) return 0;
    P3 h = padd(wo, wi);
    if (pdot(h, wo) * pdot(wi, h) < 0 || wi[2] == 0) return 0;
    h = pnorm(h);
    const double F = p_fr_diel(pdot(wi, h[2] < 0 ? pmul(h, -1) : h), ior);
    const double G = 1 / (1 + p_lambda(wo, a) + p_lambda(wi, a));
    const double f = F * std::fabs(0.25 * p_d(h, a) * G / (wi[2] * wo[2])) * std::fabs(wi[2]);
    const double pdf = p_vpdf(wo, h, a) / (4 * std::fabs(pdot(wo, h)));
    return pdf > 0 ? f / pdf : 0;
}
struct PTab {
    std::vector<double> v;
};
const PTab &p_table() {
    static PTab t;
    static bool done = false;
    if (done) return t;
    const int N = 16, Q = 256;
    t.v.assign(N * N * N, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int cell = 0; cell < N * N * N; cell++) {
        auto coord = [&](int i) { return std::min(std::max((double)(float)((float)i / (float)(N - 1)), 1e-4), 0.9999); };
        const double r = coord(cell % N), mu = coord((cell / N) % N), z = coord(cell / (N * N));
        const double ior = p_ior_from_f0(z * z * z * z);
        double s = 0;
        for (int k = 0; k < Q * Q; k++) s += p_albedo_sample(r, mu, ior, (k % Q + 0.5) / Q, (k / Q + 0.5) / Q);
        t.v[cell] = s / (Q * Q);
    }
    done = true;
    return t;
}
double p_tab3(double x, double y, double z) {
    const PTab &t = p_table();
    const int N = 16;
    auto idx = [&](double c, int &i, int &j, double &w) {
        c = std::min(std::max(c, 0.0), 1.0) * (N - 1);
        i = (int)std::floor(c);
        j = std::min(i + 1, N - 1);
        w = c - i;
    };
    int xi, xj, yi, yj, zi, zj;
    double wx, wy, wz;
    idx(x, xi, xj, wx);
    idx(y, yi, yj, wy);
    idx(z, zi, zj, wz);
    auto at = [&](int a, int b, int c) { return t.v[a + N * b + N * N * c]; };
    auto l2 = [&](int c) {
        return (1 - wy) * ((1 - wx) * at(xi, yi, c) + wx * at(xj, yi, c)) + wy * ((1 - wx) * at(xi, yj, c) + wx * at(xj, yj, c));
    };
    return (1 - wz) * l2(zi) + wz * l2(zj);
}
double p_albedo(double rough, double mu, double eta) {
    const double z = std::sqrt(std::fabs((eta - 1) / (eta + 1)));
    return p_tab3(rough, std::fabs(std::min(std::max(mu, -0.999), 0.999)), z);
}
struct PCl {
    double base[3], tcol[3], alpha, rough, rough_d, metallic, trans, ior, seta, sf0, stint[3], stl, cn[3], ck[3];
    double cw, calpha, crough, crough_d, cior, ctint[3];
    bool glass;  // STY_MAT_GLASS: glass.rs alone (p_glass_eval / p_glass_sample)
};
PCl p_closure(const sty_scene_material &m) {
    PCl c;
    for (int i = 0; i < 3; i++) {
        c.base[i] = m.albedo[i];
        c.tcol[i] = std::sqrt((double)m.albedo[i]);
        c.stint[i] = m.specular_tint[i];
        c.ctint[i] = m.coat_tint[i];
    }
    c.rough = m.roughness;
    c.alpha = std::max(c.rough * c.rough, 1e-4);
    c.rough_d = std::sqrt(c.alpha);
    c.metallic = m.metallic;
    c.trans = m.transmission;
    c.ior = m.ior;
    double f0 = (c.ior - 1) / (c.ior + 1);
    f0 *= f0;
    double es = c.ior;
    if (m.specular_ior_level != 0.5f) {
        f0 *= 2.0 * m.specular_ior_level;
        es = p_ior_from_f0(f0);
    }
    c.sf0 = f0;
    c.seta = es;
    c.stl = c.stint[0] * 0.2126 + c.stint[1] * 0.7152 + c.stint[2] * 0.0722;
    for (int i = 0; i < 3; i++) {
        const double r = std::min(std::max(c.base[i], 0.0), 0.99), g = c.stint[i], rs = std::sqrt(r);
        const double nmin = (1 - r) / (1 + r), nmax = (1 + rs) / (1 - rs), n = nmax + (nmin - nmax) * g;
        c.cn[i] = n;
        c.ck[i] = std::sqrt(std::max(((n + 1) * (n + 1) * r - (n - 1) * (n - 1)) / (1 - r), 0.0));
    }
    c.cw = m.coat_weight;
    c.crough = m.coat_roughness;
    c.calpha = std::max(c.crough * c.crough, 1e-4);
    c.crough_d = std::sqrt(c.calpha);
    c.cior = m.coat_ior;
    c.glass = m.kind == STY_MAT_GLASS;
    return c;
}
double p_refl(P3 wo, P3 wi, double a, int fk, double eta, const double *n, const double *k, const double *col, double f[3]) {
    f[0] = f[1] = f[2] = 0;
    P3 wh = padd(wo, wi);
    const double co = wo[2], ci = wi[2];
    if (pdot(wh, wo) * pdot(wi, wh) < 0 || (wh[0] == 0 && wh[1] == 0 && wh[2] == 0) || ci == 0 || co == 0 || !psame(wo, wi))
        return 0;
    wh = pnorm(wh);
    const double cf = pdot(wi, wh[2] < 0 ? pmul(wh, -1) : wh);
    const double s = std::fabs(0.25 * p_d(wh, a) / (1 + p_lambda(wo, a) + p_lambda(wi, a)) / (ci * co)) * std::fabs(ci);
    for (int i = 0; i < 3; i++) f[i] = col[i] * (fk == 0 ? p_fr_diel(cf, eta) : p_fr_cond(std::fabs(cf), n[i], k[i])) * s;
    return p_vpdf(wo, wh, a) / (4 * std::fabs(pdot(wo, wh)));
}
double p_trans(P3 wo, P3 wi, double a, double eta, const double *col, double f[3]) {
    f[0] = f[1] = f[2] = 0;
    const double co = wo[2], ci = wi[2], e = co > 0 ? eta : 1 / eta;
    P3 wh = pnorm(padd(wo, pmul(wi, e)));
    if (wh[2] < 0) wh = pmul(wh, -1);
    const bool back = pdot(wh, wi) * ci < 0 || pdot(wh, wo) * co < 0;
    if (pdot(wh, wo) * pdot(wi, wh) > 0 || ci == 0 || co == 0 || back || psame(wo, wi)) return 0;
    const double F = p_fr_diel(pdot(wo, wh), eta), q = pdot(wi, wh) + pdot(wo, wh) / e, den = q * q * ci * co;
    const double G = 1 / (1 + p_lambda(wo, a) + p_lambda(wi, a));
    if (den != 0) {
        const double s = std::fabs(p_d(wh, a) * G / (e * e) * std::fabs(pdot(wi, wh)) * std::fabs(pdot(wo, wh)) / den) * std::fabs(ci);
        for (int i = 0; i < 3; i++) f[i] = (1 - F) * col[i] * s;
    }
    return q * q == 0 ? 0 : p_vpdf(wo, wh, a) * std::fabs(pdot(wi, wh)) / (q * q);
}
// glass.rs:13-44: BsdfMixture{a: MicrofacetTransmission(kt), b: MicrofacetReflection(kr), frac =
// fr_dielectric(cos wo, eta), additive}: f = f_t + f_r, pdf = lerp(pdf_t, pdf_r, frac); kr = kt =
// the node's colour
double p_glass_eval(const PCl &c, P3 wo, P3 wi, double f[3]) {
    double ft[3], fr[3];
    const double pt = p_trans(wo, wi, c.alpha, c.ior, c.base, ft);
    const double pr = p_refl(wo, wi, c.alpha, 0, c.ior, nullptr, nullptr, c.base, fr);
    for (int i = 0; i < 3; i++) f[i] = ft[i] + fr[i];
    return plerp(pt, pr, p_fr_diel(wo[2], c.ior));
}
double p_eval(const PCl &c, P3 wo, P3 wi, double f[3]) {
    if (c.glass) return p_glass_eval(c, wo, wi, f);
    const double mu = std::fabs(wo[2]), E = 1e-4;
    double f1[3], p1;
    {
        double fa[3] = {0, 0, 0}, fb[3] = {0, 0, 0}, pa = 0, pb = 0;
        if (c.trans < 1 - E && psame(wo, wi)) {
            const double k = std::fabs(wi[2]) / kPiD;
            for (int i = 0; i < 3; i++) fa[i] = c.base[i] * k;
            pa = k;
        }
        if (c.trans > E) {
            double ft[3], fr[3];
            const double pt = p_trans(wo, wi, c.alpha, c.ior, c.tcol, ft);
            const double pr = p_refl(wo, wi, c.alpha, 0, c.ior, nullptr, nullptr, c.base, fr);
            for (int i = 0; i < 3; i++) fb[i] = ft[i] + fr[i];
            pb = plerp(pt, pr, p_fr_diel(wo[2], c.ior));
        }
        for (int i = 0; i < 3; i++) f1[i] = plerp(fa[i], fb[i], c.trans);
        p1 = plerp(pa, pb, c.trans);
    }
    double f2[3], p2;
    {
        const double A = p_albedo(c.rough, mu, c.seta), frac = c.sf0 * c.stl * A;
        const double col[3] = {c.stint[0] * c.sf0, c.stint[1] * c.sf0, c.stint[2] * c.sf0};
        double fs[3];
        const double ps = p_refl(wo, wi, c.alpha, 0, c.seta, nullptr, nullptr, col, fs);
        for (int i = 0; i < 3; i++) f2[i] = f1[i] * (1 - c.stint[i] * c.sf0 * A) + fs[i];
        p2 = plerp(p1, ps, frac);
    }
    double f3[3], p3v;
    {
        double fa[3] = {0, 0, 0}, fm[3] = {0, 0, 0}, pa = 0, pm = 0;
        if (c.metallic < 1 - E) {
            for (int i = 0; i < 3; i++) fa[i] = f2[i];
            pa = p2;
        }
        if (c.metallic > E) {
            const double one[3] = {1, 1, 1};
            pm = p_refl(wo, wi, c.alpha, 1, 0, c.cn, c.ck, one, fm);
        }
        for (int i = 0; i < 3; i++) f3[i] = plerp(fa[i], fm[i], c.metallic);
        p3v = plerp(pa, pm, c.metallic);
    }
    const double A = p_albedo(c.crough, mu, c.cior), frac = c.cw * A;
    const double col[3] = {c.cw, c.cw, c.cw};
    double fc[3];
    const double pc = p_refl(wo, wi, c.calpha, 0, c.cior, nullptr, nullptr, col, fc);
    for (int i = 0; i < 3; i++) f[i] = f3[i] * plerp(1, c.ctint[i] * (1 - A), c.cw) + fc[i];
    return plerp(p3v, pc, frac);
}
inline bool p_choose_b(double frac, double &u) {
    if (u < frac) {
        u /= frac;
        return true;
    }
    u = (u - frac) / (1 - frac);
    return false;
}
bool p_sample(const PCl &c, P3 wo, double u, double u0, double u1, P3 *wi) {
    if (c.glass) {  // the mixture picks reflection with probability frac, else transmission
        const P3 wh = p_sample_wh(wo, c.alpha, u0, u1);
        if (p_choose_b(p_fr_diel(wo[2], c.ior), u)) {
            *wi = p_reflect(wo, wh);
            return psame(wo, *wi);
        }
        if (!p_refract(wo, wh, c.ior, wi)) return false;
        return !psame(wo, *wi);
    }
    const double mu = std::fabs(wo[2]);
    if (p_choose_b(c.cw * p_albedo(c.crough, mu, c.cior), u)) {
        *wi = p_reflect(wo, p_sample_wh(wo, c.calpha, u0, u1));
        return psame(wo, *wi);
    }
    if (p_choose_b(c.metallic, u) || p_choose_b(c.sf0 * c.stl * p_albedo(c.rough, mu, c.seta), u)) {
        *wi = p_reflect(wo, p_sample_wh(wo, c.alpha, u0, u1));
        return psame(wo, *wi);
    }
    if (p_choose_b(c.trans, u)) {
        const P3 wh = p_sample_wh(wo, c.alpha, u0, u1);
        if (p_choose_b(p_fr_diel(wo[2], c.ior), u)) {
            *wi = p_reflect(wo, wh);
            return psame(wo, *wi);
        }
        if (!p_refract(wo, wh, c.ior, wi)) return false;
        return !psame(wo, *wi);
    }
    const double r = std::sqrt(u0), ph = u1 * 2 * kPiD, x = r * std::cos(ph), y = r * std::sin(ph);
    P3 w = p3(x, y, std::sqrt(std::max(1 - x * x - y * y, 0.0)));
    if (!psame(wo, w)) w = pmul(w, -1);
    *wi = w;
    return true;
}
}  // namespace

extern "C" void orc_principled_table(double *out) {
    const PTab &t = p_table();
    std::copy(t.v.begin(), t.v.end(), out);
}
// shading frame: n x 3 wo / wi; f n x 3 (f * |cos_i|), pdf n
extern "C" void orc_principled_eval(const sty_scene_material *m, uint64_t n, const double *wo, const double *wi,
                                    double *f, double *pdf) {
    const PCl c = p_closure(*m);
    p_table();
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; i++)
        pdf[i] = p_eval(c, p3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), p3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), f + 3 * i);
}
// u: n x 3 (u_select, u0, u1); outputs wi, f, pdf (pdf 0 = invalid), as SurfaceClosure::sample
extern "C" void orc_principled_sample(const sty_scene_material *m, uint64_t n, const double *wo, const double *u,
                                      double *wi, double *f, double *pdf) {
    const PCl c = p_closure(*m);
    p_table();
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const P3 o = p3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        P3 w = p3(0, 0, 0);
        double p = 0, fv[3] = {0, 0, 0};
        if (p_sample(c, o, u[3 * i], u[3 * i + 1], u[3 * i + 2], &w)) p = p_eval(c, o, w, fv);
        if (!(p > 0)) {
            p = 0;
            fv[0] = fv[1] = fv[2] = 0;
        }
        for (int k = 0; k < 3; k++) {
            wi[3 * i + k] = w[k];
            f[3 * i + k] = fv[k];
        }
        pdf[i] = p;
    }
}
