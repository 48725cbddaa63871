// pf_screen4.cu -- warp-specialised screen-space NL-PF filter for 4 spp.
//
// CTA = 32 x 16 pixel tile, 8 consumer + NPW producer warps:
//   * 8 consumer warps: thread (lx, ly) owns pixels A = (x0+lx, y0+2ly) and B = (x0+lx, y0+2ly+1),
//     i.e. 8 query records (2 pixels x 4 spp). A warp is one pixel-row pair, so every branch on
//     the candidate row is warp-uniform.
//   * producer warps: stream the (32+2R) x (16+2R) candidate halo, CH rows at a time, into a
//     double-buffered shared-memory ring guarded by mbarriers (full / empty per buffer). While
//     staging they transform each candidate once (recentred scaled position, normal, incoming
//     radiance in_d = rad + thr * out_{d+1} with the propagate fused in, weight factors).
// Kahan totals of the 8 queries live in shared memory (touched once per candidate row), which
// keeps the consumer under the 168 registers a 10-warp CTA can have per thread.
// All mbarrier waits are bounded (~2 s of %globaltimer); on expiry the thread records
// STY_DEV_WAIT_TIMEOUT in the device status word and leaves its loop, so a protocol fault ends
// the kernel with a status instead of hanging the GPU.
//
// Exponent forms (log2 domain, sigma factors folded into the scales):
//   expanded (default): positions recentred on the tile's mean c, p' = p*pscale - c*pscale,
//     arg = [cst(dx,dy) - nscale] + 2 p'_q.p'_c + n'_q.n_c
//     w   = 2^arg * m_c,  m_c = 2^(-|p'_c|^2)   (m_c and in*m_c staged per candidate)
//     The true weight also carries 2^(-|p'_q|^2); that factor is common to every term of a
//     query's numerator and denominator and cancels in the normalised result, so it is never
//     formed. -> 6 FFMA + 1 MUFU + 4 FFMA per pair.
//   direct (fallback): arg = cst - nscale + n'_q.n_c - |p'_q - p'_c|^2, w = 2^arg
//     -> 3 FADD + 6 FFMA + 1 MUFU + 4 FFMA per pair.
// The expanded form is used when every valid query of the tile has |p'_q|^2 <= kLimQ, which
// bounds the magnitude of the partial sums and hence the rounding error of the exponent
// (~1e-6 relative on the weight); candidates with |p'_c|^2 > kLimC then have weights below
// 2^-60 and are dropped exactly. Tiles whose own positions are spread wider (depth
// discontinuities in real scenes) take the direct form, which has no such bound.
#include "common.cuh"
#include "pf_screen.cuh"
#include "style.cuh"

namespace sty {
namespace {

constexpr int S = 4;
constexpr int TW = 32;
constexpr int TH = 16;
constexpr int NCW = 8;  // consumer warps
#ifndef STY_PF4_NPW
#define STY_PF4_NPW 4
#endif
#ifndef STY_PF4_NB
#define STY_PF4_NB 3
#endif
constexpr int NPW = STY_PF4_NPW;  // producer warps (10 or 12 warps both allow 168 registers)
constexpr int NC = NCW * 32;
constexpr int NP = NPW * 32;
constexpr int NTH = NC + NP;
constexpr int CH = 4;   // candidate rows per buffer
constexpr int NB = STY_PF4_NB;  // ring depth
constexpr int PU = 4;   // records staged per producer thread per batch (loads in flight)
constexpr int NF = 10;  // staged fields: p'(3) n(3) m, v(3)   [direct form: m = 1/0, v = in]
constexpr float kLimQ = 16.0f;
constexpr float kLimC = 120.0f;
constexpr float kFar = 1e18f;
constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
                 : "memory");
}
// Bounded wait for the phase with the given parity to complete. Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *status) {
    const uint32_t a = smem_addr(bar);
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = gtimer();
        else if ((it & 63) == 0 && gtimer() - t0 > kWaitNs) {
            atomicOr(status, (uint32_t)STY_DEV_WAIT_TIMEOUT);
            return false;
        }
    }
}

struct Smem {
    uint64_t full[NB];
    uint64_t empty[NB];
    float red[NCW][4];
    float cx, cy, cz;
    int mode;  // 0 = expanded, 1 = direct, 2 = no valid query
};

template <bool EXP, bool DA, bool DB>
__device__ __forceinline__ void row_pass(const float *__restrict__ rowp, int plane, int lx, int R, float pix2,
                                         const float (&qa)[8][3], const float (&qn)[8][3], float rbA, float rbB,
                                         float (&part)[8][4]) {
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const float cx = -pix2 * (float)(dx * dx);
        const float *cp = rowp + (lx + R + dx) * S;
        float c[NF][S];
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const float4 v = *reinterpret_cast<const float4 *>(cp + f * plane);
            c[f][0] = v.x;
            c[f][1] = v.y;
            c[f][2] = v.z;
            c[f][3] = v.w;
        }
        const float bA = rbA + cx, bB = rbB + cx;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if ((q < 4 && !DA) || (q >= 4 && !DB)) continue;
            const float base = q < 4 ? bA : bB;
#pragma unroll
            for (int t = 0; t < S; t++) {
                float arg;
                if (EXP) {
                    arg = fmaf(qa[q][0], c[0][t], base);
                    arg = fmaf(qa[q][1], c[1][t], arg);
                    arg = fmaf(qa[q][2], c[2][t], arg);
                    arg = fmaf(qn[q][0], c[3][t], arg);
                    arg = fmaf(qn[q][1], c[4][t], arg);
                    arg = fmaf(qn[q][2], c[5][t], arg);
                } else {
                    arg = fmaf(qn[q][0], c[3][t], base);
                    arg = fmaf(qn[q][1], c[4][t], arg);
                    arg = fmaf(qn[q][2], c[5][t], arg);
                    const float ex = qa[q][0] - c[0][t];
                    const float ey = qa[q][1] - c[1][t];
                    const float ez = qa[q][2] - c[2][t];
                    arg = fmaf(-ex, ex, arg);
                    arg = fmaf(-ey, ey, arg);
                    arg = fmaf(-ez, ez, arg);
                }
                const float e = ex2_approx(arg);
                part[q][0] = fmaf(e, c[6][t], part[q][0]);
                part[q][1] = fmaf(e, c[7][t], part[q][1]);
                part[q][2] = fmaf(e, c[8][t], part[q][2]);
                part[q][3] = fmaf(e, c[9][t], part[q][3]);
            }
        }
    }
}

// Packed FP32: d = a * b + c on both lanes (fma.rn.f32x2; each lane rounds exactly like fmaf),
// one issue slot for two FMAs.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// The expanded-form row pass on pairs of queries (spp samples 2p, 2p+1 of one pixel) with packed
// FMAs: each lane performs exactly the operation sequence of row_pass<true, ..>, so the sums are
// bit-identical; the candidate's fields are duplicated once per candidate for the four pairs.
template <bool DA, bool DB>
__device__ __forceinline__ void row_pass2(const float *__restrict__ rowp, int plane, int lx, int R, float pix2,
                                          const float2 (&qa2)[4][3], const float2 (&qn2)[4][3], float rbA, float rbB,
                                          float2 (&part2)[4][4]) {
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const float cx = -pix2 * (float)(dx * dx);
        const float *cp = rowp + (lx + R + dx) * S;
        float c[NF][S];
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const float4 v = *reinterpret_cast<const float4 *>(cp + f * plane);
            c[f][0] = v.x;
            c[f][1] = v.y;
            c[f][2] = v.z;
            c[f][3] = v.w;
        }
        const float bA = rbA + cx, bB = rbB + cx;
#pragma unroll
        for (int t = 0; t < S; t++) {
            float2 cd[NF];
#pragma unroll
            for (int f = 0; f < NF; f++) cd[f] = make_float2(c[f][t], c[f][t]);
#pragma unroll
            for (int qp = 0; qp < 4; qp++) {
                if ((qp < 2 && !DA) || (qp >= 2 && !DB)) continue;
                const float base = qp < 2 ? bA : bB;
                float2 arg = ffma2(qa2[qp][0], cd[0], make_float2(base, base));
                arg = ffma2(qa2[qp][1], cd[1], arg);
                arg = ffma2(qa2[qp][2], cd[2], arg);
                arg = ffma2(qn2[qp][0], cd[3], arg);
                arg = ffma2(qn2[qp][1], cd[4], arg);
                arg = ffma2(qn2[qp][2], cd[5], arg);
                const float2 e = make_float2(ex2_approx(arg.x), ex2_approx(arg.y));
                part2[qp][0] = ffma2(e, cd[6], part2[qp][0]);
                part2[qp][1] = ffma2(e, cd[7], part2[qp][1]);
                part2[qp][2] = ffma2(e, cd[8], part2[qp][2]);
                part2[qp][3] = ffma2(e, cd[9], part2[qp][3]);
            }
        }
    }
}

// Kahan totals: kst[(q * NC + ctid) * 2 + 0] = sums (w, r, g, b), [.. + 1] = compensations.
template <bool EXP>
__device__ __forceinline__ void consume_chunk(const float *__restrict__ buf, int plane, int cy0, int row_hi, int yA,
                                              int lx, int R, float pix2, float nscale, const float (&qa)[8][3],
                                              const float (&qn)[8][3], float4 *__restrict__ kst, int ctid) {
    for (int r = 0; r < CH; r++) {
        const int yy = cy0 + r;
        if (yy > row_hi) break;
        const int dyA = yy - yA, dyB = dyA - 1;
        const bool ia = dyA >= -R && dyA <= R;
        const bool ib = dyB >= -R && dyB <= R;
        if (!ia && !ib) continue;
        const float rbA = -pix2 * (float)(dyA * dyA) - nscale;
        const float rbB = -pix2 * (float)(dyB * dyB) - nscale;
        float part[8][4];
        const float *rowp = buf + r * (plane / CH);
        if (EXP) {
            float2 part2[4][4], qa2[4][3], qn2[4][3];
#pragma unroll
            for (int qp = 0; qp < 4; qp++) {
#pragma unroll
                for (int k = 0; k < 4; k++) part2[qp][k] = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    qa2[qp][k] = make_float2(qa[2 * qp][k], qa[2 * qp + 1][k]);
                    qn2[qp][k] = make_float2(qn[2 * qp][k], qn[2 * qp + 1][k]);
                }
            }
            if (ia && ib)
                row_pass2<true, true>(rowp, plane, lx, R, pix2, qa2, qn2, rbA, rbB, part2);
            else if (ia)
                row_pass2<true, false>(rowp, plane, lx, R, pix2, qa2, qn2, rbA, rbB, part2);
            else
                row_pass2<false, true>(rowp, plane, lx, R, pix2, qa2, qn2, rbA, rbB, part2);
#pragma unroll
            for (int qp = 0; qp < 4; qp++)
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    part[2 * qp][k] = part2[qp][k].x;
                    part[2 * qp + 1][k] = part2[qp][k].y;
                }
        } else {
#pragma unroll
            for (int q = 0; q < 8; q++)
#pragma unroll
                for (int k = 0; k < 4; k++) part[q][k] = 0.0f;
            if (ia && ib)
                row_pass<false, true, true>(rowp, plane, lx, R, pix2, qa, qn, rbA, rbB, part);
            else if (ia)
                row_pass<false, true, false>(rowp, plane, lx, R, pix2, qa, qn, rbA, rbB, part);
            else
                row_pass<false, false, true>(rowp, plane, lx, R, pix2, qa, qn, rbA, rbB, part);
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if ((q < 4 && !ia) || (q >= 4 && !ib)) continue;
            float4 *slot = kst + ((size_t)q * NC + ctid) * 2;
            float4 sm4 = slot[0], cm4 = slot[1];
            KahanF k0 = {sm4.x, cm4.x}, k1 = {sm4.y, cm4.y}, k2 = {sm4.z, cm4.z}, k3 = {sm4.w, cm4.w};
            k0.add(part[q][0]);
            k1.add(part[q][1]);
            k2.add(part[q][2]);
            k3.add(part[q][3]);
            slot[0] = make_float4(k0.s, k1.s, k2.s, k3.s);
            slot[1] = make_float4(k0.c, k1.c, k2.c, k3.c);
        }
    }
}

__global__ void __launch_bounds__(NTH, 1) k_pf_screen4(const ScreenArgs a, const sty_style_program style) {
    extern __shared__ __align__(16) float stage[];
    __shared__ Smem sh;
    const int R = a.R;
    const int CW = TW + 2 * R;
    const int plane = CH * CW * S;  // floats per field per buffer
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
    const int row_lo = ty0 - R, row_hi = ty0 + TH - 1 + R;
    const int nchunks = (row_hi - row_lo + 1 + CH - 1) / CH;
    const size_t N = (size_t)a.W * a.H * S;
    const size_t dbase = (size_t)a.depth * N;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const bool consumer = warp < NCW;

    if (tid == 0) {
        for (int b = 0; b < NB; b++) {
            mbar_init(&sh.full[b], NP);
            mbar_init(&sh.empty[b], NCW);
        }
    }

    // ---- queries (consumers) and the tile centre
    const int lx = lane, ly = warp;
    const int x = tx0 + lx, yA = ty0 + 2 * ly;
    float qp[8][3], qn[8][3];
    bool qv[8];
    float sx = 0.f, sy = 0.f, sz = 0.f, cnt = 0.f;
    if (consumer) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int y = yA + (q >> 2);
            const bool in = x < a.W && y < a.H;
            size_t g = 0;
            if (in) g = dbase + ((size_t)y * a.W + x) * S + (q & 3);
            qv[q] = in && a.valid[g] != 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                qp[q][k] = qv[q] ? a.pos[k][g] : 0.0f;
                qn[q][k] = qv[q] ? a.nrm[k][g] * a.nscale : 0.0f;
            }
            if (qv[q]) {
                sx += qp[q][0];
                sy += qp[q][1];
                sz += qp[q][2];
                cnt += 1.0f;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
            sz += __shfl_xor_sync(0xffffffffu, sz, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            sh.red[warp][0] = sx;
            sh.red[warp][1] = sy;
            sh.red[warp][2] = sz;
            sh.red[warp][3] = cnt;
        }
    }
    __syncthreads();
    if (tid == 0) {
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        for (int w = 0; w < NCW; w++)
            for (int k = 0; k < 4; k++) t[k] += sh.red[w][k];
        const float inv = t[3] > 0.f ? 1.0f / t[3] : 0.0f;
        sh.cx = t[0] * inv * a.pscale;
        sh.cy = t[1] * inv * a.pscale;
        sh.cz = t[2] * inv * a.pscale;
        sh.mode = t[3] > 0.f ? 0 : 2;
    }
    __syncthreads();
    const float ccx = sh.cx, ccy = sh.cy, ccz = sh.cz;
    float qmax = 0.0f;
    if (consumer) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            qp[q][0] = qp[q][0] * a.pscale - ccx;
            qp[q][1] = qp[q][1] * a.pscale - ccy;
            qp[q][2] = qp[q][2] * a.pscale - ccz;
            if (qv[q]) qmax = fmaxf(qmax, qp[q][0] * qp[q][0] + qp[q][1] * qp[q][1] + qp[q][2] * qp[q][2]);
        }
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 16));
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 8));
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 4));
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 2));
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 1));
        if (lane == 0 && !(qmax <= kLimQ)) atomicExch(&sh.mode, sh.mode == 2 ? 2 : 1);
    }
    __syncthreads();
    const int mode = sh.mode;

    if (mode == 2) {  // no valid record in the tile: outputs are zero
        if (consumer) {
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int y = yA + (q >> 2);
                if (x >= a.W || y >= a.H) continue;
                const size_t j = ((size_t)y * a.W + x) * S + (q & 3);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    a.out[c * N + j] = 0.0f;
                    if (a.filtered) a.filtered[c * N + j] = 0.0f;
                }
            }
        }
        return;
    }
    const bool expf_mode = mode == 0;

    if (!consumer) {
        // ================= producer warps =================
        const int ptid = tid - NC;
        for (int k = 0; k < nchunks; k++) {
            const int b = k % NB;
            if (k >= NB && !mbar_wait(&sh.empty[b], ((k / NB) - 1) & 1, a.status)) return;
            float *buf = stage + (size_t)b * NF * plane;
            const int cy0 = row_lo + k * CH;
            for (int base = ptid; base < plane; base += NP * PU) {
                // issue every load of PU records before using any of them
                size_t jj[PU];
                bool inimg[PU];
                int vv[PU];
                float raw[PU][12], on[PU][3];
#pragma unroll
                for (int u = 0; u < PU; u++) {
                    const int idx = base + u * NP;
                    const int r = idx / (CW * S);
                    const int rem = idx - r * (CW * S);
                    const int col = rem / S;
                    const int s = rem - col * S;
                    const int gy = cy0 + r, gx = tx0 - R + col;
                    inimg[u] = idx < plane && gy >= 0 && gy < a.H && gx >= 0 && gx < a.W && gy <= row_hi;
                    jj[u] = inimg[u] ? ((size_t)gy * a.W + gx) * S + s : 0;  // index 0 is always in bounds
                }
#pragma unroll
                for (int u = 0; u < PU; u++) {
                    const size_t g = dbase + jj[u];
                    vv[u] = a.valid[g];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        raw[u][c] = a.pos[c][g];
                        raw[u][3 + c] = a.nrm[c][g];
                        raw[u][6 + c] = a.rad[c][g];
                        raw[u][9 + c] = a.thr[c][g];
                        on[u][c] = a.out_next ? a.out_next[c * N + jj[u]] : 0.0f;
                    }
                }
#pragma unroll
                for (int u = 0; u < PU; u++) {
                    const int idx = base + u * NP;
                    if (idx >= plane) break;
                    const bool ok = inimg[u] && vv[u] != 0;
                    float v[NF];
                    if (ok) {
                        const float px = raw[u][0] * a.pscale - ccx;
                        const float py = raw[u][1] * a.pscale - ccy;
                        const float pz = raw[u][2] * a.pscale - ccz;
                        float in[3];
#pragma unroll
                        for (int c = 0; c < 3; c++) in[c] = fmaf(raw[u][9 + c], on[u][c], raw[u][6 + c]);
                        v[3] = raw[u][3];
                        v[4] = raw[u][4];
                        v[5] = raw[u][5];
                        if (expf_mode) {
                            const float d2 = px * px + py * py + pz * pz;
                            if (d2 <= kLimC) {
                                const float m = ex2_approx(-d2);
                                v[0] = px; v[1] = py; v[2] = pz;
                                v[6] = m;
                                v[7] = in[0] * m; v[8] = in[1] * m; v[9] = in[2] * m;
                            } else {  // weight < 2^-60 for every query of this tile: dropped exactly
                                v[0] = v[1] = v[2] = 0.0f;
                                v[6] = v[7] = v[8] = v[9] = 0.0f;
                            }
                        } else {
                            v[0] = px; v[1] = py; v[2] = pz;
                            v[6] = 1.0f;
                            v[7] = in[0]; v[8] = in[1]; v[9] = in[2];
                        }
                    } else {
                        const float far = expf_mode ? 0.0f : kFar;
                        v[0] = v[1] = v[2] = far;
                        v[3] = v[4] = v[5] = 0.0f;
                        v[6] = v[7] = v[8] = v[9] = 0.0f;
                    }
#pragma unroll
                    for (int f = 0; f < NF; f++) buf[f * plane + idx] = v[f];
                }
            }
            mbar_arrive(&sh.full[b]);
        }
        // drain: wait until the consumers released the last buffers (keeps every phase balanced)
        for (int k = (nchunks > NB ? nchunks - NB : 0); k < nchunks; k++)
            if (!mbar_wait(&sh.empty[k % NB], (k / NB) & 1, a.status)) return;
        return;
    }

    // ================= consumer warps =================
    float4 *kst = reinterpret_cast<float4 *>(stage + (size_t)NB * NF * plane);
    float qa[8][3];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const float f = expf_mode ? 2.0f : 1.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) qa[q][k] = f * qp[q][k];
        kst[((size_t)q * NC + tid) * 2 + 0] = make_float4(0.f, 0.f, 0.f, 0.f);
        kst[((size_t)q * NC + tid) * 2 + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    bool failed = false;
    for (int k = 0; k < nchunks; k++) {
        const int b = k % NB;
        if (!mbar_wait(&sh.full[b], (k / NB) & 1, a.status)) {
            failed = true;
            break;
        }
        const float *buf = stage + (size_t)b * NF * plane;
        const int cy0 = row_lo + k * CH;
        if (expf_mode)
            consume_chunk<true>(buf, plane, cy0, row_hi, yA, lx, R, a.pix2, a.nscale, qa, qn, kst, tid);
        else
            consume_chunk<false>(buf, plane, cy0, row_hi, yA, lx, R, a.pix2, a.nscale, qa, qn, kst, tid);
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh.empty[b]);
    }

    // ---- epilogue
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int y = yA + (q >> 2);
        if (x >= a.W || y >= a.H) continue;
        const size_t j = ((size_t)y * a.W + x) * S + (q & 3);
        f3 f = {0.0f, 0.0f, 0.0f}, o = {0.0f, 0.0f, 0.0f};
        if (qv[q]) {
            if (failed) {
                f = {__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
                o = f;
            } else {
                const float4 t = kst[((size_t)q * NC + tid) * 2 + 0];
                f = {t.y / t.x, t.z / t.x, t.w / t.x};
                o = style_apply(style, a.depth, f);
            }
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

}  // namespace

sty_status launch_screen_s4(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    const int CW = TW + 2 * a.R;
    const size_t smem = (size_t)NB * NF * CH * CW * S * sizeof(float) + (size_t)8 * NC * 2 * sizeof(float4);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_pf_screen4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_pf_screen4)"));
    dim3 grid((a.W + TW - 1) / TW, (a.H + TH - 1) / TH);
    k_pf_screen4<<<grid, NTH, smem, st>>>(a, style);
    return check_launch("k_pf_screen4");
}

}  // namespace sty
