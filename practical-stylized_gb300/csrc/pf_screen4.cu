// pf_screen4.cu -- warp-specialised screen-space NL-PF filter for 4 and 16 spp.
//
// CTA = 32 x (12 / G) pixel tile, 12 consumer + NPW producer warps, G = spp / 4 query groups:
//   * consumer warp w owns pixel row y0 + w / G and query group w % G; lane l owns pixel x0 + l
//     and 4 of its query records (samples 4 (w % G) .. 4 (w % G) + 3), so every branch on the
//     candidate row is warp-uniform. Three consumer warps per scheduler hide the latency of the
//     dependent exponent chains and the MUFU round trips.
//   * producer warps: stream the (32+2R) x (12+2R) candidate halo, CH rows at a time, into a
//     shared-memory ring of 3 to 6 buffers (the deepest that fits) guarded by mbarriers (full /
//     empty per buffer). While
//     staging they transform each candidate once (recentred scaled position, normal, incoming
//     radiance in_d = rad + thr * out_{d+1} with the propagate fused in, weight factors).
// Packed FP32: a candidate pixel's samples arrive 4 at a time as one 16-byte shared load per
// field; the consumer pairs samples (0, 1) and (2, 3) of each quad in the two lanes of
// `fma.rn.f32x2` against its query duplicated in both lanes, so the candidate pair needs no
// register moves. Kahan totals of the 4 queries live in shared memory (touched once per
// candidate row).
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
//     -> 9 FFMA + 1 MUFU + 4 FFMA per pair, packed in pairs like the expanded form.
// The expanded form is used when every valid query of the tile has |p'_q|^2 <= kLimQ, which
// bounds the magnitude of the partial sums and hence the rounding error of the exponent
// (~1e-6 relative on the weight); candidates with |p'_c|^2 > kLimC then lie at
// |p'_q - p'_c|^2 >= (sqrt(kLimC) - sqrt(kLimQ))^2 ~ 48 from every query, so their weights are
// below 2^-48 and they are dropped. Tiles whose own positions are spread wider (depth
// discontinuities in real scenes) take the direct form, which has no such bound.
#include "common.cuh"
#include "pf_screen.cuh"
#include "style.cuh"

namespace sty {
namespace {

#ifndef STY_PF4_TW
#define STY_PF4_TW 32
#endif
#ifndef STY_PF4_CH
#define STY_PF4_CH 2
#endif
#ifndef STY_PF4_NCW
#define STY_PF4_NCW 12
#endif
constexpr int NCW = STY_PF4_NCW;  // consumer warps (16, at 96 registers, measured 14.8 ms vs 13.7)
constexpr int TW = STY_PF4_TW;  // tile width: TW / 32 consumer warps share a pixel row
constexpr int WPR = TW / 32;
// tile height at S samples per pixel: the S / 4 query groups of a pixel row take one warp each
template <int S>
constexpr int tile_h() { return NCW / (WPR * (S / 4)); }
// Positions are recentred on the tile's mean before the exponent; wider tiles put the queries
// further from it and lose FP32 digits of |p'_q - p'_c| on spread-out tiles (measured: 128-pixel
// tiles miss 1e-5 on such data, 32 and 64 keep it).
static_assert(TW % 32 == 0 && TW <= 64 && NCW % (WPR * 4) == 0, "tile shape");
#ifndef STY_PF4_NPW
#define STY_PF4_NPW 4
#endif
#ifndef STY_PF4_PU
#define STY_PF4_PU 4
#endif
constexpr int NPW = STY_PF4_NPW;  // producer warps (16 warps: 128 registers a thread)
constexpr int NC = NCW * 32;
constexpr int NP = NPW * 32;
constexpr int NTH = NC + NP;
// candidate rows per buffer (one at 16 spp, whose rows are 4x longer)
template <int S>
constexpr int rows_per_buf() { return S >= 16 ? 1 : STY_PF4_CH; }
// Shared-memory layout of a staged candidate row, per field: the samples in quads (4 floats, one
// 16-byte load), quad-major -- quad t of every column, then quad t + 1 -- so the 32 lanes of a
// consumer warp, which read the same quad of 32 adjacent columns, read 512 contiguous bytes (no
// bank conflicts; column-major rows of 16 samples put the lanes 64 bytes apart, 4 on a bank
// group). Quads are `quad_stride` floats apart: 4 columns of padding past the row spread the
// producers' scattered stores over the banks. At 4 spp there is one quad and no padding.
template <int S>
__host__ __device__ constexpr int quad_stride(int cw) { return cw * 4 + (S > 4 ? 4 : 0); }
template <int S>
__host__ __device__ constexpr int row_floats(int cw) { return (S / 4) * quad_stride<S>(cw); }
constexpr int kMaxNB = 6;  // ring depth: the deepest of 6 .. 3 buffers that fits in shared memory
constexpr int PU = STY_PF4_PU;  // records staged per producer thread per batch (loads in flight)
constexpr int NF = 10;  // staged fields: p'(3) n(3) m, v(3)   [direct form: m = 1/0, v = in]
constexpr int NQ = 4;   // query records per consumer thread
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
    uint64_t full[kMaxNB];
    uint64_t empty[kMaxNB];
    float red[NCW][4];
    float cx, cy, cz;
    int mode;  // 0 = expanded, 1 = direct, 2 = no valid query
};

// One candidate row, expanded form: for every dx the candidate pixel's samples, 4 at a time, taken
// as the pairs (0, 1) and (2, 3) of the quad; part2[q][k].x / .y collect the even / odd samples of
// query q (w, w*in).
template <int S>
__device__ __forceinline__ void row_pass_exp(const float *__restrict__ rowp, int plane, int qs, int lx, int R, float pix2,
                                             const float2 (&qa2)[NQ][3], const float2 (&qn2)[NQ][3], float rb,
                                             float2 (&part2)[NQ][4]) {
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const float base = rb - pix2 * (float)(dx * dx);
        const float2 base2 = make_float2(base, base);
#pragma unroll 1
    for (int tq = 0; tq < S; tq += 4) {
        const float *cp = rowp + (tq >> 2) * qs + (lx + R + dx) * 4;
        float4 v[NF];
#pragma unroll
        for (int f = 0; f < NF; f++) v[f] = *reinterpret_cast<const float4 *>(cp + f * plane);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float2 c[NF];
#pragma unroll
            for (int f = 0; f < NF; f++) c[f] = h == 0 ? make_float2(v[f].x, v[f].y) : make_float2(v[f].z, v[f].w);
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                float2 arg = ffma2(qa2[q][0], c[0], base2);
                arg = ffma2(qa2[q][1], c[1], arg);
                arg = ffma2(qa2[q][2], c[2], arg);
                arg = ffma2(qn2[q][0], c[3], arg);
                arg = ffma2(qn2[q][1], c[4], arg);
                arg = ffma2(qn2[q][2], c[5], arg);
                const float2 e = make_float2(ex2_approx(arg.x), ex2_approx(arg.y));
                part2[q][0] = ffma2(e, c[6], part2[q][0]);
                part2[q][1] = ffma2(e, c[7], part2[q][1]);
                part2[q][2] = ffma2(e, c[8], part2[q][2]);
                part2[q][3] = ffma2(e, c[9], part2[q][3]);
            }
        }
    }
    }
}

// One candidate row, direct form (fallback tiles) on packed FP32, the same sample pairing as the
// expanded form. The exponent is formed negated, na = -arg: with qm = -p'_q and qnm = -n'_q held
// per query, na = -base - n'_q.n_c + |p'_c - p'_q|^2 takes one FFMA2 per term (c - q = fma(1, c, -q)
// rounds exactly like q - c, negated), so na is bit for bit the negation of the scalar form's
// arg and w = 2^(-na). -> 9 FFMA2 + 2 MUFU + 4 FFMA2 per pair of pairs.
template <int S>
__device__ __forceinline__ void row_pass_dir(const float *__restrict__ rowp, int plane, int qs, int lx, int R, float pix2,
                                             const float2 (&qm2)[NQ][3], const float2 (&qnm2)[NQ][3], float rb,
                                             float2 (&part2)[NQ][4]) {
    const float2 one2 = make_float2(1.0f, 1.0f);
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const float base = rb - pix2 * (float)(dx * dx);
        const float2 nbase2 = make_float2(-base, -base);
#pragma unroll 1
    for (int tq = 0; tq < S; tq += 4) {
        const float *cp = rowp + (tq >> 2) * qs + (lx + R + dx) * 4;
        float4 v[NF];
#pragma unroll
        for (int f = 0; f < NF; f++) v[f] = *reinterpret_cast<const float4 *>(cp + f * plane);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float2 c[NF];
#pragma unroll
            for (int f = 0; f < NF; f++) c[f] = h == 0 ? make_float2(v[f].x, v[f].y) : make_float2(v[f].z, v[f].w);
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                float2 na = ffma2(qnm2[q][0], c[3], nbase2);
                na = ffma2(qnm2[q][1], c[4], na);
                na = ffma2(qnm2[q][2], c[5], na);
                const float2 ex = ffma2(one2, c[0], qm2[q][0]);
                const float2 ey = ffma2(one2, c[1], qm2[q][1]);
                const float2 ez = ffma2(one2, c[2], qm2[q][2]);
                na = ffma2(ex, ex, na);
                na = ffma2(ey, ey, na);
                na = ffma2(ez, ez, na);
                const float2 e = make_float2(ex2_approx(-na.x), ex2_approx(-na.y));
                part2[q][0] = ffma2(e, c[6], part2[q][0]);
                part2[q][1] = ffma2(e, c[7], part2[q][1]);
                part2[q][2] = ffma2(e, c[8], part2[q][2]);
                part2[q][3] = ffma2(e, c[9], part2[q][3]);
            }
        }
    }
    }
}

// Kahan totals: kst[(q * NC + ctid) * 2 + 0] = sums (w, r, g, b), [.. + 1] = compensations.
template <int S, bool EXP>
__device__ __forceinline__ void consume_chunk(const float *__restrict__ buf, int plane, int qs, int cy0, int row_hi, int y,
                                              int lx, int R, float pix2, float nscale, const float2 (&qa2)[NQ][3],
                                              const float2 (&qn2)[NQ][3], float4 *__restrict__ kst, int ctid) {
    constexpr int CH = rows_per_buf<S>();
    for (int r = 0; r < CH; r++) {
        const int yy = cy0 + r;
        if (yy > row_hi) break;
        const int dy = yy - y;
        if (dy < -R || dy > R) continue;
        const float rb = -pix2 * (float)(dy * dy) - nscale;
        const float *rowp = buf + r * (plane / CH);  // plane = CH x row_floats
        float part[NQ][4];
        float2 part2[NQ][4];
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
            for (int k = 0; k < 4; k++) part2[q][k] = make_float2(0.0f, 0.0f);
        if (EXP)
            row_pass_exp<S>(rowp, plane, qs, lx, R, pix2, qa2, qn2, rb, part2);
        else
            row_pass_dir<S>(rowp, plane, qs, lx, R, pix2, qa2, qn2, rb, part2);
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
            for (int k = 0; k < 4; k++) part[q][k] = part2[q][k].x + part2[q][k].y;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
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

template <int S, int NB>
__global__ void __launch_bounds__(NTH, 1) k_pf_screen4(const ScreenArgs a, const sty_style_program style) {
    constexpr int G = S / 4;
    constexpr int TH = tile_h<S>();
    constexpr int CH = rows_per_buf<S>();
    extern __shared__ __align__(16) float stage[];
    __shared__ Smem sh;
    const int R = a.R;
    const int CW = TW + 2 * R;
    const int QS = quad_stride<S>(CW);
    const int plane = CH * row_floats<S>(CW);  // floats per field per buffer
    const int NREC = CH * CW * S;               // candidate records per buffer
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
    const int lx = lane + 32 * (warp % WPR);
    const int grp = (warp / WPR) % G;  // query group: samples 4 grp .. 4 grp + 3
    const int x = tx0 + lx, y = ty0 + warp / (WPR * G);
    float qp[NQ][3], qn[NQ][3];
    bool qv[NQ];
    float sx = 0.f, sy = 0.f, sz = 0.f, cnt = 0.f;
    if (consumer) {
        const bool in = x < a.W && y < a.H;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            size_t g = 0;
            if (in) g = dbase + ((size_t)y * a.W + x) * S + grp * NQ + q;
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
        for (int q = 0; q < NQ; q++) {
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
        if (consumer && x < a.W && y < a.H) {
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const size_t j = ((size_t)y * a.W + x) * S + grp * NQ + q;
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
            for (int base = ptid; base < NREC; base += NP * PU) {
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
                    inimg[u] = idx < NREC && gy >= 0 && gy < a.H && gx >= 0 && gx < a.W && gy <= row_hi;
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
                    if (idx >= NREC) break;
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
                            } else {  // weight < 2^-48 for every query of this tile: dropped exactly
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
                    const int r = idx / (CW * S), rem = idx - r * (CW * S);
                    const int col = rem / S, sm = rem - col * S;
                    const int sidx = r * (plane / CH) + (sm >> 2) * QS + col * 4 + (sm & 3);
#pragma unroll
                    for (int f = 0; f < NF; f++) buf[f * plane + sidx] = v[f];
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
    // expanded form: (2 p'_q, n'_q); direct form: (-p'_q, -n'_q) (row_pass_dir forms the negated exponent)
    float2 qa2[NQ][3], qn2[NQ][3];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const float f = expf_mode ? 2.0f : -1.0f, fn = expf_mode ? 1.0f : -1.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            qa2[q][k] = make_float2(f * qp[q][k], f * qp[q][k]);
            qn2[q][k] = make_float2(fn * qn[q][k], fn * qn[q][k]);
        }
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
            consume_chunk<S, true>(buf, plane, QS, cy0, row_hi, y, lx, R, a.pix2, a.nscale, qa2, qn2, kst, tid);
        else
            consume_chunk<S, false>(buf, plane, QS, cy0, row_hi, y, lx, R, a.pix2, a.nscale, qa2, qn2, kst, tid);
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh.empty[b]);
    }

    // ---- epilogue
    if (x >= a.W || y >= a.H) return;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const size_t j = ((size_t)y * a.W + x) * S + grp * NQ + q;
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

template <int S>
sty_status launch_screen_ws(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    constexpr int CH = rows_per_buf<S>();
    constexpr int TH = tile_h<S>();
    const int CW = TW + 2 * a.R;
    auto smem_for = [&](int nb) {
        return (size_t)nb * NF * CH * row_floats<S>(CW) * sizeof(float) + (size_t)NQ * NC * 2 * sizeof(float4);
    };
    int dev = 0, optin = 0;
    STY_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    STY_TRY(check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                       "cudaDeviceGetAttribute(max shared memory)"));
    const size_t room = (size_t)optin - sizeof(Smem);
    int nb = kMaxNB;
    while (nb > 3 && smem_for(nb) > room) nb--;
    const size_t smem = smem_for(nb);
    if (smem > room) {
        set_error("k_pf_screen4: radius %d at %d spp needs %zu bytes of shared memory (%zu available)", a.R, S, smem,
                  room);
        return STY_ERR_ARG;
    }
    auto kern = nb == 6   ? k_pf_screen4<S, 6>
                : nb == 5 ? k_pf_screen4<S, 5>
                : nb == 4 ? k_pf_screen4<S, 4>
                          : k_pf_screen4<S, 3>;
    STY_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_pf_screen4)"));
    dim3 grid((a.W + TW - 1) / TW, (a.H + TH - 1) / TH);
    kern<<<grid, NTH, smem, st>>>(a, style);
    return check_launch("k_pf_screen4");
}

}  // namespace

sty_status launch_screen_s4(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    return launch_screen_ws<4>(a, style, st);
}
sty_status launch_screen_s16(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    return launch_screen_ws<16>(a, style, st);
}
// largest radius the warp-specialised kernel serves at `spp` samples (its shared-memory ring of 3
// buffers and the Kahan totals must fit)
int screen_ws_max_radius(int spp, size_t optin) {
    const int CH = spp >= 16 ? 1 : STY_PF4_CH;
    for (int R = 32; R >= 0; R--) {
        const int rf = spp >= 16 ? row_floats<16>(TW + 2 * R) : row_floats<4>(TW + 2 * R);
        const size_t need = (size_t)3 * NF * CH * rf * sizeof(float) + (size_t)NQ * NC * 2 * sizeof(float4);
        if (need + sizeof(Smem) <= optin) return R;
    }
    return -1;
}

}  // namespace sty
