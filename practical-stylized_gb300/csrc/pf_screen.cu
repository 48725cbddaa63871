// pf_screen.cu -- screen-space NL-PF filter (one launch per path depth).
//
// Work decomposition: a CTA owns a TW x TH pixel tile, one thread per pixel, each thread owning
// the `S` spp records of its pixel as S independent queries. Candidate records of the tile's
// (TW + 2R) x (TH + 2R) neighbourhood are staged through shared memory CH rows at a time; while
// staging, every candidate is turned into (scaled position, normal, in_d) and invalid or
// off-image candidates get a far-away position so their weight underflows to exactly 0. The
// weight is evaluated in the log2 domain:
//   arg = cst(dx,dy) + n'_q . n_c - |p'_q - p'_c|^2,  w = 2^arg
// with p' = p * sqrt(log2(e) / (2 sigma_pos^2)), n'_q = n_q * log2(e) / sigma_nrm^2 and
// cst = -log2(e) * ((dx^2+dy^2) / (2 sigma_pixel^2) + 1 / sigma_nrm^2), so one candidate/query
// pair costs 9 FFMA/FADD for the exponent, one MUFU.EX2 and 4 accumulations. Sums run in plain
// FP32 across one candidate row (at most (2R+1) * S terms) and are then folded into
// Kahan-compensated totals.
#include <atomic>

#include "common.cuh"
#include "pf_screen.cuh"
#include "style.cuh"

namespace sty {
namespace {

constexpr int TW = 32;
constexpr int TH = 8;
constexpr int NT = TW * TH;
constexpr int CH = 4;  // candidate rows per shared-memory chunk
constexpr int NF = 9;  // staged fields: p'xyz, nxyz, in rgb
constexpr float kL2E = 1.4426950408889634f;
constexpr float kFar = 1e18f;  // staged position of an excluded candidate


template <int S>
struct Vec;
template <>
struct Vec<1> {
    static __device__ __forceinline__ void ld(const float *p, float (&v)[1]) { v[0] = p[0]; }
};
template <>
struct Vec<2> {
    static __device__ __forceinline__ void ld(const float *p, float (&v)[2]) {
        float2 a = *reinterpret_cast<const float2 *>(p);
        v[0] = a.x;
        v[1] = a.y;
    }
};
template <>
struct Vec<4> {
    static __device__ __forceinline__ void ld(const float *p, float (&v)[4]) {
        float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
    }
};
template <>
struct Vec<8> {
    static __device__ __forceinline__ void ld(const float *p, float (&v)[8]) {
        float4 a = *reinterpret_cast<const float4 *>(p);
        float4 b = *reinterpret_cast<const float4 *>(p + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
};

template <int S>
__global__ void __launch_bounds__(NT, S >= 8 ? 1 : 2) k_pf_screen(const ScreenArgs a, const sty_style_program style) {
    extern __shared__ __align__(16) float sm[];
    const int R = a.R;
    const int CW = TW + 2 * R;            // staged columns
    const int plane = CH * CW * S;        // floats per staged field
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
    const int lx = threadIdx.x % TW, ly = threadIdx.x / TW;
    const int x = tx0 + lx, y = ty0 + ly;
    const bool inside = (x < a.W) && (y < a.H);
    const size_t N = (size_t)a.W * a.H * S;
    const size_t dbase = (size_t)a.depth * N;

    // ---- query records of this pixel
    float qpx[S], qpy[S], qpz[S], qnx[S], qny[S], qnz[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
        if (inside) {
            const size_t g = dbase + ((size_t)y * a.W + x) * S + s;
            qpx[s] = a.pos[0][g] * a.pscale;
            qpy[s] = a.pos[1][g] * a.pscale;
            qpz[s] = a.pos[2][g] * a.pscale;
            qnx[s] = a.nrm[0][g] * a.nscale;
            qny[s] = a.nrm[1][g] * a.nscale;
            qnz[s] = a.nrm[2][g] * a.nscale;
        } else {
            qpx[s] = qpy[s] = qpz[s] = 0.0f;
            qnx[s] = qny[s] = qnz[s] = 0.0f;
        }
    }
    KahanF acc[S][4];
#pragma unroll
    for (int s = 0; s < S; s++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[s][c] = {0.0f, 0.0f};

    const int row_lo = ty0 - R, row_hi = ty0 + TH - 1 + R;  // inclusive candidate rows
    for (int cy = row_lo; cy <= row_hi; cy += CH) {
        __syncthreads();
        // ---- stage CH candidate rows
        for (int idx = threadIdx.x; idx < plane; idx += NT) {
            const int r = idx / (CW * S);
            const int rem = idx - r * (CW * S);
            const int col = rem / S;
            const int s = rem - col * S;
            const int gy = cy + r, gx = tx0 - R + col;
            float v[NF];
            bool ok = (gy >= 0) && (gy < a.H) && (gx >= 0) && (gx < a.W) && (gy <= row_hi);
            size_t j = 0;
            if (ok) {
                j = ((size_t)gy * a.W + gx) * S + s;
                ok = a.valid[dbase + j] != 0;
            }
            if (ok) {
                const size_t g = dbase + j;
                v[0] = a.pos[0][g] * a.pscale;
                v[1] = a.pos[1][g] * a.pscale;
                v[2] = a.pos[2][g] * a.pscale;
                v[3] = a.nrm[0][g];
                v[4] = a.nrm[1][g];
                v[5] = a.nrm[2][g];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float in = a.rad[c][g];
                    if (a.out_next) in = fmaf(a.thr[c][g], a.out_next[c * N + j], in);
                    v[6 + c] = in;
                }
            } else {
                v[0] = v[1] = v[2] = kFar;
                v[3] = v[4] = v[5] = 0.0f;
                v[6] = v[7] = v[8] = 0.0f;
            }
#pragma unroll
            for (int f = 0; f < NF; f++) sm[f * plane + idx] = v[f];
        }
        __syncthreads();
        // ---- accumulate
        for (int r = 0; r < CH; r++) {
            const int dy = cy + r - y;
            if (dy < -R || dy > R) continue;  // uniform across a warp (one warp = one pixel row)
            float part[S][4];
#pragma unroll
            for (int s = 0; s < S; s++)
#pragma unroll
                for (int c = 0; c < 4; c++) part[s][c] = 0.0f;
            const float cy_term = -(a.pix2 * (float)(dy * dy)) - a.nscale;
            const float *rowp = sm + (size_t)r * CW * S;
            for (int dx = -R; dx <= R; dx++) {
                const float cst = fmaf(-a.pix2, (float)(dx * dx), cy_term);
                const float *cp = rowp + (lx + R + dx) * S;
                float cpx[S], cpy[S], cpz[S], cnx[S], cny[S], cnz[S], cr[S], cg[S], cb[S];
                Vec<S>::ld(cp + 0 * plane, cpx);
                Vec<S>::ld(cp + 1 * plane, cpy);
                Vec<S>::ld(cp + 2 * plane, cpz);
                Vec<S>::ld(cp + 3 * plane, cnx);
                Vec<S>::ld(cp + 4 * plane, cny);
                Vec<S>::ld(cp + 5 * plane, cnz);
                Vec<S>::ld(cp + 6 * plane, cr);
                Vec<S>::ld(cp + 7 * plane, cg);
                Vec<S>::ld(cp + 8 * plane, cb);
#pragma unroll
                for (int t = 0; t < S; t++) {
#pragma unroll
                    for (int q = 0; q < S; q++) {
                        float arg = fmaf(qnx[q], cnx[t], cst);
                        arg = fmaf(qny[q], cny[t], arg);
                        arg = fmaf(qnz[q], cnz[t], arg);
                        const float ex = qpx[q] - cpx[t];
                        const float ey = qpy[q] - cpy[t];
                        const float ez = qpz[q] - cpz[t];
                        arg = fmaf(-ex, ex, arg);
                        arg = fmaf(-ey, ey, arg);
                        arg = fmaf(-ez, ez, arg);
                        const float w = ex2_approx(arg);
                        part[q][0] += w;
                        part[q][1] = fmaf(w, cr[t], part[q][1]);
                        part[q][2] = fmaf(w, cg[t], part[q][2]);
                        part[q][3] = fmaf(w, cb[t], part[q][3]);
                    }
                }
            }
#pragma unroll
            for (int s = 0; s < S; s++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[s][c].add(part[s][c]);
        }
    }
    if (!inside) return;
    // ---- epilogue: normalise, style, write
#pragma unroll
    for (int s = 0; s < S; s++) {
        const size_t j = ((size_t)y * a.W + x) * S + s;
        f3 f = {0.0f, 0.0f, 0.0f}, o = {0.0f, 0.0f, 0.0f};
        if (a.valid[dbase + j]) {
            const float sw = acc[s][0].s;
            f = {acc[s][1].s / sw, acc[s][2].s / sw, acc[s][3].s / sw};
            o = style_apply(style, a.depth, f);
        }
        a.out[j] = o.x;
        a.out[N + j] = o.y;
        a.out[2 * N + j] = o.z;
        if (a.filtered) {
            a.filtered[j] = f.x;
            a.filtered[N + j] = f.y;
            a.filtered[2 * N + j] = f.z;
        }
    }
}

// Many samples per pixel (S = 16): G = S / Q threads share a pixel, each owning Q of its S queries
// (one warp = 32 pixels of one row and one query group, so the row skip stays warp-uniform);
// candidate samples are read 4 at a time (16-byte loads), so registers stay within two CTAs per SM.
template <int S, int Q>
__global__ void __launch_bounds__(NT, 2) k_pf_screen_g(const ScreenArgs a, const sty_style_program style) {
    constexpr int G = S / Q;
    constexpr int GTH = NT / (TW * G);  // pixel rows per CTA
    extern __shared__ __align__(16) float sm[];
    const int R = a.R;
    const int CW = TW + 2 * R;
    const int plane = CH * CW * S;
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * GTH;
    const int lx = threadIdx.x % TW, grp = (threadIdx.x / TW) % G, ly = threadIdx.x / (TW * G);
    const int x = tx0 + lx, y = ty0 + ly;
    const bool inside = (x < a.W) && (y < a.H);
    const size_t N = (size_t)a.W * a.H * S;
    const size_t dbase = (size_t)a.depth * N;

    float qpx[Q], qpy[Q], qpz[Q], qnx[Q], qny[Q], qnz[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (inside) {
            const size_t g = dbase + ((size_t)y * a.W + x) * S + grp * Q + q;
            qpx[q] = a.pos[0][g] * a.pscale;
            qpy[q] = a.pos[1][g] * a.pscale;
            qpz[q] = a.pos[2][g] * a.pscale;
            qnx[q] = a.nrm[0][g] * a.nscale;
            qny[q] = a.nrm[1][g] * a.nscale;
            qnz[q] = a.nrm[2][g] * a.nscale;
        } else {
            qpx[q] = qpy[q] = qpz[q] = 0.0f;
            qnx[q] = qny[q] = qnz[q] = 0.0f;
        }
    }
    KahanF acc[Q][4];
#pragma unroll
    for (int q = 0; q < Q; q++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[q][c] = {0.0f, 0.0f};

    const int row_lo = ty0 - R, row_hi = ty0 + GTH - 1 + R;
    for (int cy = row_lo; cy <= row_hi; cy += CH) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < plane; idx += NT) {
            const int r = idx / (CW * S);
            const int rem = idx - r * (CW * S);
            const int col = rem / S;
            const int smp = rem - col * S;
            const int gy = cy + r, gx = tx0 - R + col;
            float v[NF];
            bool ok = (gy >= 0) && (gy < a.H) && (gx >= 0) && (gx < a.W) && (gy <= row_hi);
            size_t j = 0;
            if (ok) {
                j = ((size_t)gy * a.W + gx) * S + smp;
                ok = a.valid[dbase + j] != 0;
            }
            if (ok) {
                const size_t g = dbase + j;
                v[0] = a.pos[0][g] * a.pscale;
                v[1] = a.pos[1][g] * a.pscale;
                v[2] = a.pos[2][g] * a.pscale;
                v[3] = a.nrm[0][g];
                v[4] = a.nrm[1][g];
                v[5] = a.nrm[2][g];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float in = a.rad[c][g];
                    if (a.out_next) in = fmaf(a.thr[c][g], a.out_next[c * N + j], in);
                    v[6 + c] = in;
                }
            } else {
                v[0] = v[1] = v[2] = kFar;
                v[3] = v[4] = v[5] = 0.0f;
                v[6] = v[7] = v[8] = 0.0f;
            }
#pragma unroll
            for (int f = 0; f < NF; f++) sm[f * plane + idx] = v[f];
        }
        __syncthreads();
        for (int r = 0; r < CH; r++) {
            const int dy = cy + r - y;
            if (dy < -R || dy > R) continue;  // uniform across a warp
            float part[Q][4];
#pragma unroll
            for (int q = 0; q < Q; q++)
#pragma unroll
                for (int c = 0; c < 4; c++) part[q][c] = 0.0f;
            const float cy_term = -(a.pix2 * (float)(dy * dy)) - a.nscale;
            const float *rowp = sm + (size_t)r * CW * S;
            for (int dx = -R; dx <= R; dx++) {
                const float cst = fmaf(-a.pix2, (float)(dx * dx), cy_term);
                const float *cp0 = rowp + (lx + R + dx) * S;
#pragma unroll
                for (int tc = 0; tc < S; tc += 4) {
                    const float *cp = cp0 + tc;
                    float cpx[4], cpy[4], cpz[4], cnx[4], cny[4], cnz[4], cr[4], cg[4], cb[4];
                    Vec<4>::ld(cp + 0 * plane, cpx);
                    Vec<4>::ld(cp + 1 * plane, cpy);
                    Vec<4>::ld(cp + 2 * plane, cpz);
                    Vec<4>::ld(cp + 3 * plane, cnx);
                    Vec<4>::ld(cp + 4 * plane, cny);
                    Vec<4>::ld(cp + 5 * plane, cnz);
                    Vec<4>::ld(cp + 6 * plane, cr);
                    Vec<4>::ld(cp + 7 * plane, cg);
                    Vec<4>::ld(cp + 8 * plane, cb);
#pragma unroll
                    for (int t = 0; t < 4; t++) {
#pragma unroll
                        for (int q = 0; q < Q; q++) {
                            float arg = fmaf(qnx[q], cnx[t], cst);
                            arg = fmaf(qny[q], cny[t], arg);
                            arg = fmaf(qnz[q], cnz[t], arg);
                            const float ex = qpx[q] - cpx[t];
                            const float ey = qpy[q] - cpy[t];
                            const float ez = qpz[q] - cpz[t];
                            arg = fmaf(-ex, ex, arg);
                            arg = fmaf(-ey, ey, arg);
                            arg = fmaf(-ez, ez, arg);
                            const float w = ex2_approx(arg);
                            part[q][0] += w;
                            part[q][1] = fmaf(w, cr[t], part[q][1]);
                            part[q][2] = fmaf(w, cg[t], part[q][2]);
                            part[q][3] = fmaf(w, cb[t], part[q][3]);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < Q; q++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[q][c].add(part[q][c]);
        }
    }
    if (!inside) return;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const size_t j = ((size_t)y * a.W + x) * S + grp * Q + q;
        f3 f = {0.0f, 0.0f, 0.0f}, o = {0.0f, 0.0f, 0.0f};
        if (a.valid[dbase + j]) {
            const float sw = acc[q][0].s;
            f = {acc[q][1].s / sw, acc[q][2].s / sw, acc[q][3].s / sw};
            o = style_apply(style, a.depth, f);
        }
        a.out[j] = o.x;
        a.out[N + j] = o.y;
        a.out[2 * N + j] = o.z;
        if (a.filtered) {
            a.filtered[j] = f.x;
            a.filtered[N + j] = f.y;
            a.filtered[2 * N + j] = f.z;
        }
    }
}

template <int S, int Q>
sty_status launch_screen_g(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    constexpr int GTH = NT / (TW * (S / Q));
    const int CW = TW + 2 * a.R;
    const size_t smem = (size_t)NF * CH * CW * S * sizeof(float);
    STY_ARG_CHECK(smem <= 227 * 1024, "radius %d too large for %d samples per pixel", a.R, S);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_pf_screen_g<S, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem),
                       "cudaFuncSetAttribute(k_pf_screen_g)"));
    dim3 grid((a.W + TW - 1) / TW, (a.H + GTH - 1) / GTH);
    k_pf_screen_g<S, Q><<<grid, NT, smem, st>>>(a, style);
    return check_launch("k_pf_screen_g");
}

template <int S>
sty_status launch_screen(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    const int CW = TW + 2 * a.R;
    const size_t smem = (size_t)NF * CH * CW * S * sizeof(float);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_pf_screen<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_pf_screen)"));
    dim3 grid((a.W + TW - 1) / TW, (a.H + TH - 1) / TH);
    k_pf_screen<S><<<grid, NT, smem, st>>>(a, style);
    return check_launch("k_pf_screen");
}

sty_status validate(const sty_pf_records *rec, const sty_pf_screen_params *p) {
    STY_ARG_CHECK(rec && p, "null records or params");
    STY_ARG_CHECK(rec->width > 0 && rec->height > 0 && rec->depths > 0, "bad record dimensions %dx%d, depths %d",
                  rec->width, rec->height, rec->depths);
    STY_ARG_CHECK(rec->spp == 1 || rec->spp == 2 || rec->spp == 4 || rec->spp == 8 || rec->spp == 16,
                  "spp must be 1, 2, 4, 8 or 16 (got %d)", rec->spp);
    for (int c = 0; c < 3; c++)
        STY_ARG_CHECK(rec->pos[c] && rec->nrm[c] && rec->rad[c] && rec->thr[c], "null record field");
    STY_ARG_CHECK(rec->valid, "null valid field");
    STY_ARG_CHECK(p->radius >= 0 && p->radius <= 32, "radius must be in [0, 32] (got %d)", p->radius);
    STY_ARG_CHECK(p->sigma_pos > 0.0f && p->sigma_nrm > 0.0f, "sigma_pos and sigma_nrm must be > 0");
    STY_ARG_CHECK((size_t)rec->width * rec->height * rec->spp * rec->depths < (1ull << 40), "records too large");
    return STY_OK;
}

std::atomic<int32_t> g_screen_kernel{STY_SCREEN_KERNEL_AUTO};

// the kernel family the dispatch uses (AUTO resolved)
int32_t screen_kernel_choice() {
    const int32_t k = g_screen_kernel.load(std::memory_order_relaxed);
    return k == STY_SCREEN_KERNEL_AUTO ? STY_SCREEN_KERNEL_FP32 : k;
}

}  // namespace
}  // namespace sty

using namespace sty;

extern "C" {

sty_status sty_pf_screen_set_kernel(int32_t kernel) {
    clear_error();
    STY_ARG_CHECK(kernel == STY_SCREEN_KERNEL_AUTO || kernel == STY_SCREEN_KERNEL_FP32 ||
                      kernel == STY_SCREEN_KERNEL_TENSOR,
                  "sty_pf_screen_set_kernel: unknown kernel %d", kernel);
    g_screen_kernel.store(kernel, std::memory_order_relaxed);
    return STY_OK;
}

sty_status sty_pf_screen_filter_depth(const sty_pf_records *rec, uint32_t depth, const sty_pf_screen_params *params,
                                      const sty_style_program *style, const float *out_next, float *out,
                                      float *filtered, void *stream) {
    clear_error();
    STY_TRY(validate(rec, params));
    STY_ARG_CHECK(out, "sty_pf_screen_filter_depth: null out");
    STY_ARG_CHECK(depth < (uint32_t)rec->depths, "depth %u out of range (depths %d)", depth, rec->depths);
    STY_ARG_CHECK(style_program_valid(style), "invalid style program");
    sty_style_program prog;
    if (style)
        prog = *style;
    else
        memset(&prog, 0, sizeof(prog));
    ScreenArgs a;
    for (int c = 0; c < 3; c++) {
        a.pos[c] = rec->pos[c];
        a.nrm[c] = rec->nrm[c];
        a.rad[c] = rec->rad[c];
        a.thr[c] = rec->thr[c];
    }
    a.valid = rec->valid;
    a.out_next = out_next;
    a.out = out;
    a.filtered = filtered;
    a.W = rec->width;
    a.H = rec->height;
    a.R = params->radius;
    a.depth = depth;
    a.pscale = sqrtf(kL2E / (2.0f * params->sigma_pos * params->sigma_pos));
    a.nscale = kL2E / (params->sigma_nrm * params->sigma_nrm);
    a.pix2 = params->sigma_pixel > 0.0f ? kL2E / (2.0f * params->sigma_pixel * params->sigma_pixel) : 0.0f;
    a.status = device_status_ptr();
    STY_ARG_CHECK(a.status, "device status word unavailable (no CUDA device?)");
    cudaStream_t st = as_stream(stream);
    switch (rec->spp) {
        case 1: return launch_screen<1>(a, prog, st);
        case 2: return launch_screen<2>(a, prog, st);
        case 4:  // the warp-specialised kernel's shared-memory ring fits up to radius 24
            if (screen_kernel_choice() == STY_SCREEN_KERNEL_TENSOR && screen_tc_supports(a, 4))
                return launch_screen_tc(a, prog, st);
            return a.R <= 24 ? launch_screen_s4(a, prog, st) : launch_screen<4>(a, prog, st);
        case 8: return launch_screen<8>(a, prog, st);
        default: {  // the warp-specialised kernel where its shared-memory ring fits
            int dev = 0, optin = 0;
            STY_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
            STY_TRY(check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                               "cudaDeviceGetAttribute(max shared memory)"));
            return a.R <= screen_ws_max_radius(16, (size_t)optin) ? launch_screen_s16(a, prog, st)
                                                                  : launch_screen_g<16, 4>(a, prog, st);
        }
    }
}

sty_status sty_pf_screen_filter(const sty_pf_records *rec, const sty_pf_screen_params *params,
                                const sty_style_program *style, float *out, void *stream) {
    clear_error();
    STY_TRY(validate(rec, params));
    STY_ARG_CHECK(out, "sty_pf_screen_filter: null out");
    const size_t N = (size_t)rec->width * rec->height * rec->spp;
    for (int d = rec->depths - 1; d >= 0; d--) {
        const float *next = (d + 1 < rec->depths) ? out + (size_t)(d + 1) * 3 * N : nullptr;
        STY_TRY(sty_pf_screen_filter_depth(rec, (uint32_t)d, params, style, next, out + (size_t)d * 3 * N, nullptr,
                                           stream));
    }
    return STY_OK;
}

}  // extern "C"
