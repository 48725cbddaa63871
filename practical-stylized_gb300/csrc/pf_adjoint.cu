// pf_adjoint.cu -- adjoint of the screen-space NL-PF filter + smoothed ramp style node.
//
// Forward (see include/sty_gb300.h): f_i = N_i / D_i with D_i = sum_j w_ij, N_i = sum_j w_ij in_j,
//   w_ij = exp(a_ij), a_ij = -rho_ij / (2 sx^2) - |p_i - p_j|^2 / (2 sp^2) - (1 - n_i.n_j) / sn^2,
//   out_i = sum_k sigmoid(s (lum(f_i) - t_k)) (c_k - c_{k-1}); image = spp mean; L = |image - T|^2.
// Backward, per valid record i with g_i = dL/dout_i = 2 (image - T) / spp:
//   style:  dL/dc_k += g_i (sig_k - sig_{k+1}),  dL/dt_k += -s sig'_k (g_i . dc_k),
//           dL/ds += sum_k sig'_k (lum_i - t_k) (g_i . dc_k),  h_i = dL/df_i = (sum_k s sig'_k g_i.dc_k) * Y
//           with Y the Rec.709 luminance weights;
//   filter: df_i/dtheta = sum_j dw_ij/dtheta (in_j - f_i) / D_i with dw/dsx = w rho / sx^3,
//           dw/dsp = w |dp|^2 / sp^3, dw/dsn = 2 w (1 - n.n) / sn^3.
// The kernel recomputes the neighbourhood weights in two sweeps over the staged candidate rows:
// sweep 1 rebuilds D_i, N_i (hence f_i and h_i), sweep 2 accumulates the three bandwidth sums.
// Per-thread results are reduced per block into a partial vector; a final single-block kernel sums
// the partials in a fixed order (deterministic).
#include <mutex>

#include "common.cuh"
#include "pf_screen.cuh"
#include "style.cuh"

namespace sty {
namespace {

constexpr int TW = 32, TH = 8, NT = TW * TH, CH = 4, NF = 7;  // staged: p(3) n(3) valid
constexpr int NG = 36;
constexpr float kL2E = 1.4426950408889634f;

struct AdjArgs {
    const float *pos[3], *nrm[3], *rad[3], *thr[3];
    const int32_t *valid;
    const float *in_next;
    const float *dimg;  // dL/dimage per pixel, interleaved rgb
    int W, H, R;
    uint32_t depth;
    float sx, sp, sn;
    float s, t[8], c[8][3];
    int nsteps;
    float *partials;  // [gridDim.x * gridDim.y][NG]
};

__device__ __forceinline__ float sigm(float x) { return 1.0f / (1.0f + expf(-x)); }

// One candidate row for 4 spp on packed FP32: the candidate pixel's 4 samples come in as one
// 16-byte load per field, and queries (0, 1) and (2, 3) share the lanes of `fma.rn.f32x2`.
// Sweep 0 accumulates (w, w in) into part, sweep 1 the three bandwidth sums into pe (as the scalar
// loop below, with the log2(e) factor folded into the exponent's scales).
__device__ __forceinline__ void pair_row4(const float *__restrict__ rowp, const float *__restrict__ rowi, int plane,
                                          int lx, int R, int dy, float isx2, float isp2, float isn2,
                                          const float (&qp)[4][3], const float (&qn)[4][3], const float (&h)[4][3],
                                          const float (&hf)[4], int sweep, float (&part)[4][4], float (&pe)[4][3]) {
    const float2 zero2 = make_float2(0.0f, 0.0f), one2 = make_float2(1.0f, 1.0f), m1 = make_float2(-1.0f, -1.0f);
    const float2 nisp2 = make_float2(-isp2 * kL2E, -isp2 * kL2E), nisn2 = make_float2(-isn2 * kL2E, -isn2 * kL2E);
    float2 qa[2][3], qb[2][3], hh[2][3], nhf[2];
#pragma unroll
    for (int p = 0; p < 2; p++) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            qa[p][k] = make_float2(qp[2 * p][k], qp[2 * p + 1][k]);
            qb[p][k] = make_float2(qn[2 * p][k], qn[2 * p + 1][k]);
            hh[p][k] = make_float2(h[2 * p][k], h[2 * p + 1][k]);
        }
        nhf[p] = make_float2(-hf[2 * p], -hf[2 * p + 1]);
    }
    float2 acc[2][4];
#pragma unroll
    for (int p = 0; p < 2; p++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[p][k] = zero2;
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const float rho = (float)(dx * dx + dy * dy);
        const float2 arho = make_float2(-rho * isx2 * kL2E, -rho * isx2 * kL2E), rho2 = make_float2(rho, rho);
        const int cb = (lx + R + dx) * 4;
        const float4 v[10] = {*reinterpret_cast<const float4 *>(rowp + cb),
                              *reinterpret_cast<const float4 *>(rowp + plane + cb),
                              *reinterpret_cast<const float4 *>(rowp + 2 * plane + cb),
                              *reinterpret_cast<const float4 *>(rowp + 3 * plane + cb),
                              *reinterpret_cast<const float4 *>(rowp + 4 * plane + cb),
                              *reinterpret_cast<const float4 *>(rowp + 5 * plane + cb),
                              *reinterpret_cast<const float4 *>(rowp + 6 * plane + cb),
                              *reinterpret_cast<const float4 *>(rowi + cb),
                              *reinterpret_cast<const float4 *>(rowi + plane + cb),
                              *reinterpret_cast<const float4 *>(rowi + 2 * plane + cb)};
#pragma unroll
        for (int t = 0; t < 4; t++) {
            float c[10];
#pragma unroll
            for (int f = 0; f < 10; f++) c[f] = t == 0 ? v[f].x : t == 1 ? v[f].y : t == 2 ? v[f].z : v[f].w;
#pragma unroll
            for (int p = 0; p < 2; p++) {
                const float2 ex = ffma2(make_float2(c[0], c[0]), m1, qa[p][0]);
                const float2 ey = ffma2(make_float2(c[1], c[1]), m1, qa[p][1]);
                const float2 ez = ffma2(make_float2(c[2], c[2]), m1, qa[p][2]);
                float2 d2 = ffma2(ex, ex, zero2);
                d2 = ffma2(ey, ey, d2);
                d2 = ffma2(ez, ez, d2);
                float2 dn = ffma2(qb[p][0], make_float2(c[3], c[3]), zero2);
                dn = ffma2(qb[p][1], make_float2(c[4], c[4]), dn);
                dn = ffma2(qb[p][2], make_float2(c[5], c[5]), dn);
                const float2 om = ffma2(dn, m1, one2);
                float2 a = ffma2(d2, nisp2, arho);
                a = ffma2(om, nisn2, a);
                const float2 w = ffma2(make_float2(ex2_approx(a.x), ex2_approx(a.y)), make_float2(c[6], c[6]), zero2);
                if (sweep == 0) {
                    acc[p][0] = ffma2(w, one2, acc[p][0]);
                    acc[p][1] = ffma2(w, make_float2(c[7], c[7]), acc[p][1]);
                    acc[p][2] = ffma2(w, make_float2(c[8], c[8]), acc[p][2]);
                    acc[p][3] = ffma2(w, make_float2(c[9], c[9]), acc[p][3]);
                } else {
                    float2 u = ffma2(hh[p][0], make_float2(c[7], c[7]), nhf[p]);
                    u = ffma2(hh[p][1], make_float2(c[8], c[8]), u);
                    u = ffma2(hh[p][2], make_float2(c[9], c[9]), u);
                    const float2 tt = ffma2(w, u, zero2);
                    acc[p][0] = ffma2(tt, rho2, acc[p][0]);
                    acc[p][1] = ffma2(tt, d2, acc[p][1]);
                    acc[p][2] = ffma2(tt, om, acc[p][2]);
                }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < 2; p++)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (sweep == 0) {
                part[2 * p][k] = acc[p][k].x;
                part[2 * p + 1][k] = acc[p][k].y;
            } else if (k < 3) {
                pe[2 * p][k] = acc[p][k].x;
                pe[2 * p + 1][k] = acc[p][k].y;
            }
        }
}

template <int S>
__global__ void __launch_bounds__(NT) k_pf_adjoint(const AdjArgs a) {
    extern __shared__ __align__(16) float sm[];
    __shared__ float red[NT / 32][NG];
    const int R = a.R, CW = TW + 2 * R, plane = CH * CW * S;
    float *sin_ = sm + NF * plane;  // staged in_j (3 planes)
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
    const int lx = threadIdx.x % TW, ly = threadIdx.x / TW;
    const int x = tx0 + lx, y = ty0 + ly;
    const bool inside = x < a.W && y < a.H;
    const size_t N = (size_t)a.W * a.H * S, dbase = (size_t)a.depth * N;
    const float isx2 = 1.0f / (2.0f * a.sx * a.sx), isp2 = 1.0f / (2.0f * a.sp * a.sp), isn2 = 1.0f / (a.sn * a.sn);

    float qp[S][3], qn[S][3];
    bool qv[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
        qv[s] = false;
        size_t g = 0;
        if (inside) {
            g = dbase + ((size_t)y * a.W + x) * S + s;
            qv[s] = a.valid[g] != 0;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            qp[s][k] = inside ? a.pos[k][g] : 0.0f;
            qn[s][k] = inside ? a.nrm[k][g] : 0.0f;
        }
    }
    float gsum[NG];
#pragma unroll
    for (int k = 0; k < NG; k++) gsum[k] = 0.0f;
    KahanF acc[S][4];
    float f[S][3], h[S][3], hf[S], invD[S];
    const int row_lo = ty0 - R, row_hi = ty0 + TH - 1 + R;

    for (int sweep = 0; sweep < 2; sweep++) {
        KahanF e[S][3];
#pragma unroll
        for (int s = 0; s < S; s++)
#pragma unroll
            for (int k = 0; k < 4; k++) {
                acc[s][k] = {0.0f, 0.0f};
                if (k < 3) e[s][k] = {0.0f, 0.0f};
            }
        for (int cy = row_lo; cy <= row_hi; cy += CH) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < plane; idx += NT) {
                const int r = idx / (CW * S), rem = idx - r * (CW * S), col = rem / S, s = rem - col * S;
                const int gy = cy + r, gx = tx0 - R + col;
                bool ok = gy >= 0 && gy < a.H && gx >= 0 && gx < a.W && gy <= row_hi;
                size_t j = 0;
                if (ok) {
                    j = ((size_t)gy * a.W + gx) * S + s;
                    ok = a.valid[dbase + j] != 0;
                }
                const size_t g = dbase + j;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    sm[k * plane + idx] = ok ? a.pos[k][g] : 0.0f;
                    sm[(3 + k) * plane + idx] = ok ? a.nrm[k][g] : 0.0f;
                    float in = 0.0f;
                    if (ok) {
                        in = a.rad[k][g];
                        if (a.in_next) in = fmaf(a.thr[k][g], a.in_next[k * N + j], in);
                    }
                    sin_[k * plane + idx] = in;
                }
                sm[6 * plane + idx] = ok ? 1.0f : 0.0f;
            }
            __syncthreads();
            for (int r = 0; r < CH; r++) {
                const int dy = cy + r - y;
                if (dy < -R || dy > R) continue;
                float part[S][4], pe[S][3];
#pragma unroll
                for (int s = 0; s < S; s++)
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        part[s][k] = 0.0f;
                        if (k < 3) pe[s][k] = 0.0f;
                    }
                const float *rowp = sm + r * CW * S;
                const float *rowi = sin_ + r * CW * S;
                if constexpr (S == 4) {
                    pair_row4(rowp, rowi, plane, lx, R, dy, isx2, isp2, isn2, qp, qn, h, hf, sweep, part, pe);
                } else {
                for (int dx = -R; dx <= R; dx++) {
                    const float rho = (float)(dx * dx + dy * dy);
                    const int cb = (lx + R + dx) * S;
#pragma unroll
                    for (int t = 0; t < S; t++) {
                        const float cv = rowp[6 * plane + cb + t];
                        const float cpx = rowp[cb + t], cpy = rowp[plane + cb + t], cpz = rowp[2 * plane + cb + t];
                        const float cnx = rowp[3 * plane + cb + t], cny = rowp[4 * plane + cb + t],
                                    cnz = rowp[5 * plane + cb + t];
                        const float ir = rowi[cb + t], ig = rowi[plane + cb + t], ib = rowi[2 * plane + cb + t];
#pragma unroll
                        for (int q = 0; q < S; q++) {
                            const float ex = qp[q][0] - cpx, ey = qp[q][1] - cpy, ez = qp[q][2] - cpz;
                            const float d2 = ex * ex + ey * ey + ez * ez;
                            const float one_m = 1.0f - (qn[q][0] * cnx + qn[q][1] * cny + qn[q][2] * cnz);
                            const float arg = -(rho * isx2 + d2 * isp2 + one_m * isn2);
                            const float w = cv * ex2_approx(arg * kL2E);
                            if (sweep == 0) {
                                part[q][0] += w;
                                part[q][1] = fmaf(w, ir, part[q][1]);
                                part[q][2] = fmaf(w, ig, part[q][2]);
                                part[q][3] = fmaf(w, ib, part[q][3]);
                            } else {
                                const float tt = w * (h[q][0] * ir + h[q][1] * ig + h[q][2] * ib - hf[q]);
                                pe[q][0] = fmaf(tt, rho, pe[q][0]);
                                pe[q][1] = fmaf(tt, d2, pe[q][1]);
                                pe[q][2] = fmaf(tt, one_m, pe[q][2]);
                            }
                        }
                    }
                }
                }
#pragma unroll
                for (int q = 0; q < S; q++) {
                    if (sweep == 0) {
#pragma unroll
                        for (int k = 0; k < 4; k++) acc[q][k].add(part[q][k]);
                    } else {
#pragma unroll
                        for (int k = 0; k < 3; k++) e[q][k].add(pe[q][k]);
                    }
                }
            }
        }
        if (sweep == 0) {
            // normalise, style forward + backward
#pragma unroll
            for (int q = 0; q < S; q++) {
                h[q][0] = h[q][1] = h[q][2] = 0.0f;
                hf[q] = 0.0f;
                invD[q] = 0.0f;
                if (!qv[q]) continue;
                const float D = acc[q][0].s;
                invD[q] = 1.0f / D;
                f[q][0] = acc[q][1].s / D;
                f[q][1] = acc[q][2].s / D;
                f[q][2] = acc[q][3].s / D;
                const float *gp = a.dimg + 3 * ((size_t)y * a.W + x);
                const float g[3] = {gp[0] / S, gp[1] / S, gp[2] / S};
                const float cl[3] = {fminf(fmaxf(f[q][0], 0.0f), 1e5f), fminf(fmaxf(f[q][1], 0.0f), 1e5f),
                                     fminf(fmaxf(f[q][2], 0.0f), 1e5f)};
                const float lum = cl[0] * 0.2126f + cl[1] * 0.7152f + cl[2] * 0.0722f;
                float dlum = 0.0f, prev[3] = {0.0f, 0.0f, 0.0f}, sg_prev = 0.0f;
                for (int k = 0; k < a.nsteps; k++) {
                    const float sg = sigm(a.s * (lum - a.t[k]));
                    const float dsg = sg * (1.0f - sg);
                    const float gdc = g[0] * (a.c[k][0] - prev[0]) + g[1] * (a.c[k][1] - prev[1]) +
                                      g[2] * (a.c[k][2] - prev[2]);
                    dlum += a.s * dsg * gdc;
                    gsum[0] += dsg * (lum - a.t[k]) * gdc;  // d/ds
                    gsum[1 + k] += -a.s * dsg * gdc;        // d/dt_k
                    // d out / d c_k = sig_k - sig_{k+1}: accumulate sig_k here, subtract at k+1
                    if (k > 0)
#pragma unroll
                        for (int ch = 0; ch < 3; ch++) gsum[9 + 3 * (k - 1) + ch] += g[ch] * (sg_prev - sg);
                    sg_prev = sg;
#pragma unroll
                    for (int ch = 0; ch < 3; ch++) prev[ch] = a.c[k][ch];
                }
#pragma unroll
                for (int ch = 0; ch < 3; ch++) gsum[9 + 3 * (a.nsteps - 1) + ch] += g[ch] * sg_prev;
                const float Y[3] = {0.2126f, 0.7152f, 0.0722f};
#pragma unroll
                for (int ch = 0; ch < 3; ch++) {
                    const bool act = f[q][ch] > 0.0f && f[q][ch] < 1e5f;
                    h[q][ch] = act ? dlum * Y[ch] : 0.0f;
                }
                hf[q] = h[q][0] * f[q][0] + h[q][1] * f[q][1] + h[q][2] * f[q][2];
            }
        } else {
#pragma unroll
            for (int q = 0; q < S; q++) {
                if (!qv[q]) continue;
                gsum[33] += e[q][0].s * invD[q] / (a.sx * a.sx * a.sx);
                gsum[34] += e[q][1].s * invD[q] / (a.sp * a.sp * a.sp);
                gsum[35] += 2.0f * e[q][2].s * invD[q] / (a.sn * a.sn * a.sn);
            }
        }
    }
    // block reduction of the 36 gradient entries
#pragma unroll
    for (int k = 0; k < NG; k++) {
        float v = gsum[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NG) {
        float v = 0.0f;
        for (int w = 0; w < NT / 32; w++) v += red[w][threadIdx.x];
        a.partials[(size_t)(blockIdx.y * gridDim.x + blockIdx.x) * NG + threadIdx.x] = v;
    }
}

// image = spp mean of out; dimg = 2 (image - target); loss partials per block
__global__ void k_img_loss(const float *out, int W, int H, int S, const float *target, float *dimg, float *lpart) {
    __shared__ float red[8];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)W * H * S;
    float l = 0.0f;
    if (p < W * H) {
        for (int c = 0; c < 3; c++) {
            float m = 0.0f;
            for (int s = 0; s < S; s++) m += out[c * N + (size_t)p * S + s];
            m /= S;
            const float d = m - target[3 * (size_t)p + c];
            dimg[3 * (size_t)p + c] = 2.0f * d;
            l += d * d;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        lpart[blockIdx.x] = t;
    }
}

// fixed-order compensated sum of per-block partial vectors
__global__ void k_reduce_partials(const float *partials, int nblocks, int width, float *outv) {
    const int k = threadIdx.x;
    if (k >= width) return;
    KahanF s = {0.0f, 0.0f};
    for (int b = 0; b < nblocks; b++) s.add(partials[(size_t)b * width + k]);
    outv[k] = s.s;
}

template <int S>
sty_status launch_adj(const AdjArgs &a, cudaStream_t st) {
    const int CW = TW + 2 * a.R;
    const size_t smem = (size_t)(NF + 3) * CH * CW * S * sizeof(float);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_pf_adjoint<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "attr k_pf_adjoint"));
    dim3 grid((a.W + TW - 1) / TW, (a.H + TH - 1) / TH);
    k_pf_adjoint<S><<<grid, NT, smem, st>>>(a);
    return check_launch("k_pf_adjoint");
}

}  // namespace
}  // namespace sty

using namespace sty;

extern "C" sty_status sty_pf_adjoint(const sty_pf_records *rec, uint32_t depth, int32_t radius, const float prm[36],
                                     uint32_t n_steps, const float *in_next, const float *target, float *grad,
                                     float *loss_out, void *stream) {
    clear_error();
    STY_ARG_CHECK(rec && prm && target && grad, "sty_pf_adjoint: null argument");
    STY_ARG_CHECK(n_steps >= 1 && n_steps <= 8, "n_steps must be in [1, 8]");
    STY_ARG_CHECK(radius >= 0 && radius <= 32, "radius must be in [0, 32]");
    STY_ARG_CHECK(prm[33] > 0.0f && prm[34] > 0.0f && prm[35] > 0.0f, "bandwidths must be > 0");
    STY_ARG_CHECK(depth < (uint32_t)rec->depths, "depth out of range");
    STY_ARG_CHECK(rec->spp == 1 || rec->spp == 2 || rec->spp == 4 || rec->spp == 8, "spp must be 1, 2, 4 or 8");
    cudaStream_t st = as_stream(stream);
    const int Wd = rec->width, Hd = rec->height, S = rec->spp;
    const size_t N = (size_t)Wd * Hd * S;
    // forward through the product filter (ramp node at this depth only)
    sty_style_program prog;
    memset(&prog, 0, sizeof(prog));
    prog.n_nodes = 1;
    sty_style_node &nd = prog.nodes[0];
    nd.kind = STY_STYLE_RAMP_SMOOTH;
    nd.depth_mask = 1u << (depth > 31 ? 31 : depth);
    nd.n = (int32_t)n_steps;
    nd.p[0] = prm[0];
    for (uint32_t k = 0; k < n_steps; k++) {
        nd.p[1 + k] = prm[1 + k];
        for (int c = 0; c < 3; c++) nd.p[9 + 3 * k + c] = prm[9 + 3 * k + c];
    }
    sty_pf_screen_params sp = {radius, prm[33], prm[34], prm[35]};
    const int gx = (Wd + 31) / 32, gy = (Hd + 7) / 8, nb = gx * gy;
    const int npix = Wd * Hd, lb = (npix + 255) / 256;
    float *out = nullptr, *dimg = nullptr, *parts = nullptr, *lparts = nullptr, *lsum = nullptr;
    sty_status s = check_cuda(cudaMallocAsync((void **)&out, 3 * N * 4, st), "alloc adjoint out");
    if (s == STY_OK) s = check_cuda(cudaMallocAsync((void **)&dimg, (size_t)npix * 3 * 4, st), "alloc dimg");
    if (s == STY_OK) s = check_cuda(cudaMallocAsync((void **)&parts, (size_t)nb * NG * 4, st), "alloc partials");
    if (s == STY_OK) s = check_cuda(cudaMallocAsync((void **)&lparts, (size_t)lb * 4, st), "alloc loss partials");
    if (s == STY_OK) s = check_cuda(cudaMallocAsync((void **)&lsum, 4, st), "alloc loss");
    if (s == STY_OK) s = sty_pf_screen_filter_depth(rec, depth, &sp, &prog, in_next, out, nullptr, stream);
    if (s == STY_OK) {
        k_img_loss<<<lb, 256, 0, st>>>(out, Wd, Hd, S, target, dimg, lparts);
        s = check_launch("k_img_loss");
    }
    if (s == STY_OK) {
        AdjArgs a;
        for (int k = 0; k < 3; k++) {
            a.pos[k] = rec->pos[k];
            a.nrm[k] = rec->nrm[k];
            a.rad[k] = rec->rad[k];
            a.thr[k] = rec->thr[k];
        }
        a.valid = rec->valid;
        a.in_next = in_next;
        a.dimg = dimg;
        a.W = Wd;
        a.H = Hd;
        a.R = radius;
        a.depth = depth;
        a.sx = prm[33];
        a.sp = prm[34];
        a.sn = prm[35];
        a.s = prm[0];
        for (int k = 0; k < 8; k++) {
            a.t[k] = prm[1 + k];
            for (int c = 0; c < 3; c++) a.c[k][c] = prm[9 + 3 * k + c];
        }
        a.nsteps = (int)n_steps;
        a.partials = parts;
        switch (S) {
            case 1: s = launch_adj<1>(a, st); break;
            case 2: s = launch_adj<2>(a, st); break;
            case 4: s = launch_adj<4>(a, st); break;
            default: s = launch_adj<8>(a, st); break;
        }
    }
    if (s == STY_OK) {
        k_reduce_partials<<<1, 64, 0, st>>>(parts, nb, NG, grad);
        s = check_launch("k_reduce_partials");
    }
    if (s == STY_OK) {
        k_reduce_partials<<<1, 32, 0, st>>>(lparts, lb, 1, lsum);
        s = check_launch("k_reduce_partials(loss)");
    }
    if (s == STY_OK && loss_out) {
        s = check_cuda(cudaMemcpyAsync(loss_out, lsum, 4, cudaMemcpyDeviceToHost, st), "read loss");
        if (s == STY_OK) s = check_cuda(cudaStreamSynchronize(st), "sync loss");
    }
    void *ptrs[] = {out, dimg, parts, lparts, lsum};
    for (void *p : ptrs)
        if (p) cudaFreeAsync(p, st);
    return s;
}

// ---- allocation-free variant ---------------------------------------------------------------
// For callers that cannot allocate device memory: a host integrator whose device memory is owned
// and budgeted by another runtime (the reference sizes its NL-PF scratch from the `vram` config key
// and allocates every buffer through its own device layer), or a render loop that must not fail on
// an allocation half-way through a frame. Their scratch lives in one fixed device array, reserved
// when the library is loaded on a device and held until the process exits.
namespace sty {
namespace {
constexpr size_t kNaMaxRecords = size_t(1) << 18;           // width * height * spp of the depth
constexpr size_t kNaMaxPixels = size_t(1) << 16;            // width * height
constexpr size_t kNaMaxBlocks = 4096;                       // 32 x 8 pixel tiles
constexpr size_t kNaMaxLossBlocks = kNaMaxPixels / 256;
constexpr size_t kNaOut = 0;                                // 3 * kNaMaxRecords floats
constexpr size_t kNaDimg = kNaOut + 3 * kNaMaxRecords;      // 3 * kNaMaxPixels
constexpr size_t kNaParts = kNaDimg + 3 * kNaMaxPixels;     // kNaMaxBlocks * 36
constexpr size_t kNaLParts = kNaParts + kNaMaxBlocks * NG;  // kNaMaxLossBlocks
constexpr size_t kNaLoss = kNaLParts + kNaMaxLossBlocks;    // 1 (padded)
constexpr size_t kNaFloats = kNaLoss + 64;                  // 1,130,816 floats = 4.31 MiB

// The scratch itself. Host code must not pass this name to a kernel: on the host it is only a
// stand-in for the symbol; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) float g_adjoint_scratch[kNaFloats];

// Device address of g_adjoint_scratch on the current device, looked up with that device current on
// the first call there (and again if the device's context was replaced: a device reset reloads the
// module, possibly at another address).
sty_status noalloc_scratch(float **out) {
    struct Entry {
        float *ptr = nullptr;
        uint64_t ctx = 0;
    };
    static Entry cache[64];
    static std::mutex mu;
    int dev = -1;
    STY_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return STY_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(mu);
    const uint64_t ctx = current_context_id();
    if (!cache[dev].ptr || ctx == 0 || cache[dev].ctx != ctx) {
        void *addr = nullptr;
        STY_TRY(check_cuda(cudaGetSymbolAddress(&addr, g_adjoint_scratch), "cudaGetSymbolAddress(adjoint scratch)"));
        cache[dev].ptr = static_cast<float *>(addr);
        cache[dev].ctx = current_context_id();
    }
    *out = cache[dev].ptr;
    return STY_OK;
}
}  // namespace
}  // namespace sty

extern "C" sty_status sty_pf_adjoint_noalloc(const sty_pf_records *rec, uint32_t depth, int32_t radius,
                                             const float prm[36], uint32_t n_steps, const float *in_next,
                                             const float *target, float *grad, float *loss_out, void *stream) {
    clear_error();
    STY_ARG_CHECK(rec && prm && target && grad, "sty_pf_adjoint_noalloc: null argument");
    STY_ARG_CHECK(n_steps >= 1 && n_steps <= 8, "n_steps must be in [1, 8]");
    STY_ARG_CHECK(radius >= 0 && radius <= 32, "radius must be in [0, 32]");
    STY_ARG_CHECK(prm[33] > 0.0f && prm[34] > 0.0f && prm[35] > 0.0f, "bandwidths must be > 0");
    STY_ARG_CHECK(depth < (uint32_t)rec->depths, "depth out of range");
    STY_ARG_CHECK(rec->spp == 1 || rec->spp == 2 || rec->spp == 4 || rec->spp == 8, "spp must be 1, 2, 4 or 8");
    STY_ARG_CHECK(rec->width > 0 && rec->height > 0, "empty image");
    const int Wd = rec->width, Hd = rec->height, S = rec->spp;
    const size_t N = (size_t)Wd * Hd * S, npix = (size_t)Wd * Hd;
    const int gx = (Wd + 31) / 32, gy = (Hd + 7) / 8;
    const size_t nb = (size_t)gx * gy, lb = (npix + 255) / 256;
    STY_ARG_CHECK(N <= kNaMaxRecords,
                  "sty_pf_adjoint_noalloc: %zu records per depth exceed the fixed scratch limit of %zu "
                  "(width * height * spp); use sty_pf_adjoint", N, kNaMaxRecords);
    STY_ARG_CHECK(npix <= kNaMaxPixels,
                  "sty_pf_adjoint_noalloc: %zu pixels exceed the fixed scratch limit of %zu; use sty_pf_adjoint",
                  npix, kNaMaxPixels);
    STY_ARG_CHECK(nb <= kNaMaxBlocks, "sty_pf_adjoint_noalloc: %zu tiles exceed the fixed scratch limit of %zu",
                  nb, kNaMaxBlocks);
    float *scratch = nullptr;
    STY_TRY(noalloc_scratch(&scratch));
    float *out = scratch + kNaOut, *dimg = scratch + kNaDimg, *parts = scratch + kNaParts;
    float *lparts = scratch + kNaLParts, *lsum = scratch + kNaLoss;
    cudaStream_t st = as_stream(stream);
    sty_style_program prog;
    memset(&prog, 0, sizeof(prog));
    prog.n_nodes = 1;
    sty_style_node &nd = prog.nodes[0];
    nd.kind = STY_STYLE_RAMP_SMOOTH;
    nd.depth_mask = 1u << (depth > 31 ? 31 : depth);
    nd.n = (int32_t)n_steps;
    nd.p[0] = prm[0];
    for (uint32_t k = 0; k < n_steps; k++) {
        nd.p[1 + k] = prm[1 + k];
        for (int c = 0; c < 3; c++) nd.p[9 + 3 * k + c] = prm[9 + 3 * k + c];
    }
    sty_pf_screen_params sp = {radius, prm[33], prm[34], prm[35]};
    // Every scratch region below is fully overwritten before it is read (no accumulation into
    // scratch), so nothing has to be cleared between calls.
    STY_TRY(sty_pf_screen_filter_depth(rec, depth, &sp, &prog, in_next, out, nullptr, stream));
    k_img_loss<<<(unsigned)lb, 256, 0, st>>>(out, Wd, Hd, S, target, dimg, lparts);
    STY_TRY(check_launch("k_img_loss"));
    AdjArgs a;
    for (int k = 0; k < 3; k++) {
        a.pos[k] = rec->pos[k];
        a.nrm[k] = rec->nrm[k];
        a.rad[k] = rec->rad[k];
        a.thr[k] = rec->thr[k];
    }
    a.valid = rec->valid;
    a.in_next = in_next;
    a.dimg = dimg;
    a.W = Wd;
    a.H = Hd;
    a.R = radius;
    a.depth = depth;
    a.sx = prm[33];
    a.sp = prm[34];
    a.sn = prm[35];
    a.s = prm[0];
    for (int k = 0; k < 8; k++) {
        a.t[k] = prm[1 + k];
        for (int c = 0; c < 3; c++) a.c[k][c] = prm[9 + 3 * k + c];
    }
    a.nsteps = (int)n_steps;
    a.partials = parts;
    switch (S) {
        case 1: STY_TRY(launch_adj<1>(a, st)); break;
        case 2: STY_TRY(launch_adj<2>(a, st)); break;
        case 4: STY_TRY(launch_adj<4>(a, st)); break;
        default: STY_TRY(launch_adj<8>(a, st)); break;
    }
    k_reduce_partials<<<1, 64, 0, st>>>(parts, (int)nb, NG, grad);
    STY_TRY(check_launch("k_reduce_partials"));
    k_reduce_partials<<<1, 32, 0, st>>>(lparts, (int)lb, 1, lsum);
    STY_TRY(check_launch("k_reduce_partials(loss)"));
    if (loss_out) {
        STY_TRY(check_cuda(cudaMemcpyAsync(loss_out, lsum, 4, cudaMemcpyDeviceToHost, st), "read loss"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync loss"));
    }
    return STY_OK;
}
