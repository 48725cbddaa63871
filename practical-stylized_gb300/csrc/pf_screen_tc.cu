// pf_screen_tc.cu -- screen-space NL-PF filter (4 spp, radius 15-16) with its logits on the tcgen05
// tensor cores.
//
// The filter of one query q over its window is an attention-shaped product:
//   out_q = sum_c w_qc in_c / sum_c w_qc,   w_qc = 2^(S_qc),
//   S_qc  = -|p'_q - p'_c|^2 + nscale (n_q . n_c - 1) - pix2 |x_q - x_c|^2  (inside the window)
// (positions pre-scaled by pscale = sqrt(log2 e / 2 sigma_pos^2), so S is in the log2 domain; the
// same weights as the packed-FMA kernel in pf_screen4.cu). Terms that depend on q alone cancel in
// the normalised result, so with positions recentred on the tile's mean c and normals on its mean
// normal nbar, S (less those terms) is a bilinear form of a query feature row and a candidate
// feature row:
//   q = (2 p'_q, nscale (n_q - nbar), 2 pix2 y_q, 1)       (y_q, y_c tile-centred pixel rows)
//   c = (p'_c, n_c - nbar, y_c, b_c),  b_c = -|p'_c|^2 + nscale (nbar . n_c - 1) - pix2 y_c^2
// plus the horizontal term, which is taken as a table: the 8 query columns of a tile make it a
// rank-8 product onehot(x_q) . M[x_c] with M[k][x_c] = -pix2 (k - x_c)^2 inside |k - x_c| <= R and
// -2^14 outside (2^S underflows to 0), so the tensor cores also apply the window's x bounds.
// Invalid candidates (and those with |p'_c|^2 > kLimC, whose weights are below 2^-48 for every
// query of the tile, as in the packed-FMA kernel's expanded form) get b_c = -2^14.
//
// FP32-level accuracy of the logits from TF32 operands (10-bit mantissas) comes from the 3-pass
// split hi . hi + hi . lo + lo . hi (hi = RN-to-TF32, lo = x - hi, which the tensor core truncates):
//   S = [qh | qh | ql | onehot | onehot] . [ch | cl | ch | Mh | Ml]     (K = 40: 5 MMAs of K 8, N 160)
// The weights and the weighted sums stay on the CUDA cores in FP32: w = ex2(S) and two packed FMAs
// per pair against the candidates' incoming radiance, broadcast from shared memory. Rows of the
// window outside |y_q - y_c| <= R are skipped by the warps that own those queries. Every
// kKahanRows window rows each thread adds its FP32 partial sums into Kahan totals.
//
// Measured on GB300 (1920x1080 x 4 spp, radius 16): 16.5 ms per depth launch against 13.8 ms for
// the packed-FMA kernel. Reading the logits as 16x256b fragments gives a thread 4 queries, so a
// radiance load feeds 8 pairs; read one query per thread (32x32b) every pair needed its own
// warp-uniform shared-memory load (4 bytes per wavefront, 1920 wavefronts per window row) and the
// kernel took 22.5 ms with the shared-memory pipe 65 % busy. What remains is pipeline latency: the
// stages overlap imperfectly and every tile fills and drains the pipeline (without the sums the
// same kernel still takes 12.5 ms). Putting the sums on the tensor cores as well (split-TF32
// P . [v_hi | v_lo] with P written back to TMEM) needs 40 MMAs of N = 16 per window row; a TF32
// tcgen05.mma of M = 128, K = 8 costs its issuing thread ~63 cycles and holds the tensor pipe ~39
// cycles whatever its N (full rate only from N = 160: 80 cycles), so those sums alone cost more
// pipe time than the whole packed-FMA kernel (measured 33-36 ms per launch).
//
// CTA = one 8 x 4 pixel tile = 128 queries = the 128 TMEM lanes (lane = 32 row + 4 x + sample),
// 15 warps:
//   warps 0-7   epilogue: warp w owns lanes 32 (w % 4) .. +31 (pixel row w % 4) and half w / 4 of
//               the window row's 160 candidates, read as 16x256b fragments: per 8-candidate block a
//               thread holds 4 queries (lanes t/4, t/4 + 8, 16 + t/4, 24 + t/4 of the quarter) x 2
//               candidates (2 (t % 4), +1), so one 8-byte radiance load per channel serves 8 pairs;
//               then w = ex2(S) and the sums on packed FMAs; warps 0-3 also write the query
//               features (into TMEM: the A operand of the logits) and the outputs.
//   warps 8-12  producers: the window row's candidate feature image (K-major core matrices, no
//               swizzle) and radiance row, from the raw ring, into a ring of kNS stages.
//   warp 13     lane 0 issues the logits of each window row into one of 2 TMEM buffers of 160
//               columns (A = the query features in TMEM columns 320-359, B = the candidate image).
//   warp 14     lane 0 copies each window row's 16 record fields (pos, nrm, rad, thr, valid,
//               out_next) from HBM into a raw ring of kNR stages with cp.async.bulk.
// Every mbarrier wait is bounded (~2 s); on expiry the thread records STY_DEV_WAIT_TIMEOUT and
// leaves its loop, and the outputs of the tile become NaN; the MMA thread waits (bounded) for its
// last commit and the loader for its last copies before the CTA ends.
//
// Tiles whose queries lie too far from their mean (|p'_q|^2 > kLimQ: the bilinear form would lose
// digits to cancellation) take the direct form on the CUDA cores inside the same CTA.
#include "common.cuh"
#include "pf_screen.cuh"
#include "style.cuh"
#include "tc.cuh"

namespace sty {
namespace {
using namespace tc;

constexpr int kS = 4;                 // samples per pixel
constexpr int kTX = 8, kTY = 4;       // query tile in pixels
constexpr int kM = kTX * kTY * kS;    // 128 queries = MMA rows
constexpr int kK = 40;                // logit features
constexpr int kNCol = 160;            // candidates per window row at radius 15-16 (40 px x 4)
constexpr int kEW = 8, kPW = 5;       // epilogue and producer warps (one candidate per producer thread)
constexpr int kNH = kNCol / (kEW / 4); // candidates per epilogue warp (2 warps share a TMEM lane quarter)
constexpr int kMmaWarp = kEW + kPW;   // warp 13: MMA issue
constexpr int kLoadWarp = kMmaWarp + 1;  // warp 14: bulk copies of the raw record rows
constexpr int kKahanRows = 4;         // window rows summed in FP32 before a Kahan step
constexpr int kNT = (kLoadWarp + 1) * 32;
constexpr int kNS = 4;                // staging ring depth (feature images and radiance rows)
constexpr int kNR = 4;                // raw ring depth (record rows)
constexpr int kNB = 2;                // TMEM logit buffers
constexpr uint32_t kColQ = kNB * kNCol;  // TMEM columns of the query features (A operand of the logits)
constexpr float kBig = 16384.0f;
constexpr float kLimQ = 16.0f, kLimC = 120.0f;

// operand images: element (row, k) of a K-major image with 40 columns sits at
// (row / 8) * 1280 + (k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4 bytes (LBO 128, SBO 1280)
constexpr uint32_t kRowGroup = kK / 4 * 128;           // 1280
constexpr uint32_t kCfBytes = kNCol / 8 * kRowGroup;   // 25600
constexpr uint32_t kVBytes = 3 * kNCol * 4;            // incoming radiance, [channel][candidate]
constexpr uint32_t kStageBytes = kCfBytes + kVBytes;   // 27520
constexpr int kNpxMax = kNCol / 4;                     // 40 candidate pixels per window row
constexpr uint32_t kTabBytes = kNpxMax * 16 * 4;       // horizontal table: Mh[8], Ml[8] per pixel
// raw ring: per window row the 40 candidate pixels' records as copied from HBM, 16 fields x 160
// values (pos 0-2, nrm 3-5, rad 6-8, thr 9-11, valid 12, out_next 13-15)
constexpr int kNF = 16;
constexpr uint32_t kRawField = kNCol * 4;           // 640 bytes
constexpr uint32_t kRawBytes = kNF * kRawField;     // 10240
constexpr uint32_t kSmemBytes = kNS * kStageBytes + kTabBytes + kNR * kRawBytes;
static_assert(kColQ + kK <= 512, "TMEM budget");

__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t m, uint32_t n) {
    // D f32 (bit 4), A / B TF32 (bits 7-9, 10-12 = 2), both K-major, N>>3 (bits 17-22), M>>4 (24-28)
    return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}
// A operand from TMEM (lanes = rows, one TF32 column per K element)
__device__ __forceinline__ void mma_tf32_ts(uint32_t d, uint32_t a_tmem, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tmem_st16u(uint32_t taddr, const uint32_t *r) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
        "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}
__device__ __forceinline__ void tmem_st8u(uint32_t taddr, const uint32_t *r) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// 16x256b fragments: per 8 columns, thread t gets (lane t / 4, columns 2 (t % 4), +1) and
// (lane t / 4 + 8, the same columns); repetition i covers columns 8 i .. 8 i + 7 (registers 4 i ..)
__device__ __forceinline__ void tmem_ld_frag4(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.16x256b.x4.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_frag2(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.16x256b.x2.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
// weights and sums of nb 8-candidate blocks: lo / hi = the fragments of lane halves 0 / 1,
// vr = the radiance row at this thread's first candidate column
template <int nb>
__device__ __forceinline__ void frag_sums(const uint32_t *lo, const uint32_t *hi, const float *vr, float2 (&acc)[4][4]) {
    const float2 one2 = make_float2(1.0f, 1.0f);
#pragma unroll
    for (int i = 0; i < nb; i++) {
        float2 w[4];
        w[0] = make_float2(ex2_approx(__uint_as_float(lo[4 * i])), ex2_approx(__uint_as_float(lo[4 * i + 1])));
        w[1] = make_float2(ex2_approx(__uint_as_float(lo[4 * i + 2])), ex2_approx(__uint_as_float(lo[4 * i + 3])));
        w[2] = make_float2(ex2_approx(__uint_as_float(hi[4 * i])), ex2_approx(__uint_as_float(hi[4 * i + 1])));
        w[3] = make_float2(ex2_approx(__uint_as_float(hi[4 * i + 2])), ex2_approx(__uint_as_float(hi[4 * i + 3])));
        const float2 r2 = *reinterpret_cast<const float2 *>(vr + 8 * i);
        const float2 g2 = *reinterpret_cast<const float2 *>(vr + kNCol + 8 * i);
        const float2 b2 = *reinterpret_cast<const float2 *>(vr + 2 * kNCol + 8 * i);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            acc[q][0] = ffma2(w[q], r2, acc[q][0]);
            acc[q][1] = ffma2(w[q], g2, acc[q][1]);
            acc[q][2] = ffma2(w[q], b2, acc[q][2]);
            acc[q][3] = ffma2(w[q], one2, acc[q][3]);
        }
    }
}
__device__ __forceinline__ void mbar_init1(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// untiled bulk copy global -> shared (both addresses and the size multiples of 16 bytes), completing
// its bytes on `bar`
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive1(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}
// x = hi + lo with hi rounded to TF32 (nearest, ties away) and lo = x - hi exact in FP32
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}
// byte offset of element (row, 4 k4) in a 40-column K-major image (16-byte group k4)
__device__ __forceinline__ uint32_t kimg_off(int row, int k4) {
    return (uint32_t)(row >> 3) * kRowGroup + (uint32_t)k4 * 128u + (uint32_t)(row & 7) * 16u;
}
// one 40-feature row: [a | b | c | d | e], 8 features each
__device__ __forceinline__ void store_row40(uint8_t *dst, const float (&a)[8], const float (&b)[8], const float (&c)[8],
                                            const float4 d0, const float4 d1, const float4 e0, const float4 e1) {
    *reinterpret_cast<float4 *>(dst + 0 * 128) = make_float4(a[0], a[1], a[2], a[3]);
    *reinterpret_cast<float4 *>(dst + 1 * 128) = make_float4(a[4], a[5], a[6], a[7]);
    *reinterpret_cast<float4 *>(dst + 2 * 128) = make_float4(b[0], b[1], b[2], b[3]);
    *reinterpret_cast<float4 *>(dst + 3 * 128) = make_float4(b[4], b[5], b[6], b[7]);
    *reinterpret_cast<float4 *>(dst + 4 * 128) = make_float4(c[0], c[1], c[2], c[3]);
    *reinterpret_cast<float4 *>(dst + 5 * 128) = make_float4(c[4], c[5], c[6], c[7]);
    *reinterpret_cast<float4 *>(dst + 6 * 128) = d0;
    *reinterpret_cast<float4 *>(dst + 7 * 128) = d1;
    *reinterpret_cast<float4 *>(dst + 8 * 128) = e0;
    *reinterpret_cast<float4 *>(dst + 9 * 128) = e1;
}

struct SmemTc {
    uint64_t stage_full[kNS], stage_empty[kNS];
    uint64_t raw_full[kNR], raw_empty[kNR];
    uint64_t s_full[kNB], s_empty[kNB];
    uint64_t qf_ready;
    uint32_t tmem_slot;
    float red[4][8];        // per query warp: sum p'(3), sum n(3), count
    float part[kEW / 4][kM][4];  // per column half, each query's totals
};

__global__ void __launch_bounds__(kNT, 1) k_pf_screen_tc(const ScreenArgs a, const sty_style_program style) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ SmemTc sh;
    uint8_t *stage = smem;
    float *tab = reinterpret_cast<float *>(smem + kNS * kStageBytes);
    uint8_t *raw = smem + kNS * kStageBytes + kTabBytes;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int R = a.R;
    const int npx = kTX + 2 * R;  // candidate pixels per window row (<= 40)
    const int nrows = kTY + 2 * R;
    const int tx0 = blockIdx.x * kTX, ty0 = blockIdx.y * kTY;
    const size_t N = (size_t)a.W * a.H * kS;
    const size_t dbase = (size_t)a.depth * N;

    if (tid == 0) {
        for (int s = 0; s < kNS; s++) {
            mbar_init1(&sh.stage_full[s], kPW * 32);
            mbar_init1(&sh.stage_empty[s], 1 + kEW);  // the logits' commit + every epilogue warp
        }
        for (int r = 0; r < kNR; r++) {
            mbar_init1(&sh.raw_full[r], 1);  // the loader's arrive.expect_tx + the copies' bytes
            mbar_init1(&sh.raw_empty[r], kPW * 32);
        }
        for (int b = 0; b < kNB; b++) {
            mbar_init1(&sh.s_full[b], 1);
            mbar_init1(&sh.s_empty[b], kEW);
        }
        mbar_init1(&sh.qf_ready, kM);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&sh.tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // ---- queries (threads 0-127 = TMEM lanes) and the tile's mean position / normal
    const bool is_q = tid < kM;
    const int qrow = tid >> 5, qx = (tid & 31) >> 2, qs = tid & 3;
    const int x = tx0 + qx, y = ty0 + qrow;
    size_t qj = 0;
    bool qv = false;
    float qp[3] = {0.f, 0.f, 0.f}, qn[3] = {0.f, 0.f, 0.f};
    if (is_q) {
        const bool in = x < a.W && y < a.H;
        qj = in ? ((size_t)y * a.W + x) * kS + qs : 0;
        qv = in && a.valid[dbase + qj] != 0;
        if (qv) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                qp[k] = a.pos[k][dbase + qj] * a.pscale;
                qn[k] = a.nrm[k][dbase + qj];
            }
        }
        float v[7] = {qp[0], qp[1], qp[2], qn[0], qn[1], qn[2], qv ? 1.0f : 0.0f};
#pragma unroll
        for (int k = 0; k < 7; k++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < 7; k++) sh.red[warp][k] = v[k];
    } else if (warp >= kEW && warp < kMmaWarp) {
        // producers: the horizontal table
        for (int i = tid - kEW * 32; i < kNpxMax * 8; i += kPW * 32) {
            const int p = i >> 3, k = i & 7;
            const int d = k - (p - R);  // query column minus candidate column
            const float m = (p < npx && d >= -R && d <= R) ? -a.pix2 * (float)(d * d) : -kBig;
            float hi, lo;
            split_tf32(m, hi, lo);
            tab[p * 16 + k] = hi;
            tab[p * 16 + 8 + k] = lo;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sh.tmem_slot;
    float t7[7];
#pragma unroll
    for (int k = 0; k < 7; k++) t7[k] = sh.red[0][k] + sh.red[1][k] + sh.red[2][k] + sh.red[3][k];
    if (t7[6] == 0.0f) {  // no valid query in the tile: outputs are zero
        if (is_q && x < a.W && y < a.H)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                a.out[c * N + qj] = 0.0f;
                if (a.filtered) a.filtered[c * N + qj] = 0.0f;
            }
        fence_before();
        __syncthreads();
        fence_after();
        if (warp == kMmaWarp) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
        return;
    }
    const float inv = 1.0f / t7[6];
    const float cx = t7[0] * inv, cy = t7[1] * inv, cz = t7[2] * inv;
    const float nbx = t7[3] * inv, nby = t7[4] * inv, nbz = t7[5] * inv;
    float q2 = 0.0f;
    if (is_q) {
        qp[0] -= cx;
        qp[1] -= cy;
        qp[2] -= cz;
        if (qv) q2 = qp[0] * qp[0] + qp[1] * qp[1] + qp[2] * qp[2];
    }
    const bool direct = __syncthreads_or(is_q && qv && !(q2 <= kLimQ)) != 0;

    bool failed = false;
    float acc_out[4] = {0.f, 0.f, 0.f, 0.f};  // r, g, b, weight (threads 0-127)
    if (direct) {
        // ---- direct form on the CUDA cores (tiles spread wider than the bilinear form allows)
        if (is_q && qv) {
            KahanF k0 = {0.f, 0.f}, k1 = {0.f, 0.f}, k2 = {0.f, 0.f}, k3 = {0.f, 0.f};
            const float nq[3] = {qn[0] * a.nscale, qn[1] * a.nscale, qn[2] * a.nscale};
            for (int dy = -R; dy <= R; dy++) {
                const int gy = y + dy;
                if (gy < 0 || gy >= a.H) continue;
                const float rb = -a.pix2 * (float)(dy * dy) - a.nscale;
                for (int dx = -R; dx <= R; dx++) {
                    const int gx = x + dx;
                    if (gx < 0 || gx >= a.W) continue;
                    const float base = rb - a.pix2 * (float)(dx * dx);
                    for (int s = 0; s < kS; s++) {
                        const size_t j = ((size_t)gy * a.W + gx) * kS + s;
                        if (a.valid[dbase + j] == 0) continue;
                        float arg = base;
#pragma unroll
                        for (int k = 0; k < 3; k++) arg = fmaf(nq[k], a.nrm[k][dbase + j], arg);
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            const float e = a.pos[k][dbase + j] * a.pscale - (k == 0 ? cx : k == 1 ? cy : cz) - qp[k];
                            arg = fmaf(-e, e, arg);
                        }
                        const float w = ex2_approx(arg);
                        float in[3];
#pragma unroll
                        for (int c = 0; c < 3; c++)
                            in[c] = fmaf(a.thr[c][dbase + j], a.out_next ? a.out_next[c * N + j] : 0.0f,
                                         a.rad[c][dbase + j]);
                        k0.add(w * in[0]);
                        k1.add(w * in[1]);
                        k2.add(w * in[2]);
                        k3.add(w);
                    }
                }
            }
            acc_out[0] = k0.s;
            acc_out[1] = k1.s;
            acc_out[2] = k2.s;
            acc_out[3] = k3.s;
        }
    } else if (warp >= kEW && warp < kMmaWarp) {
        // ================= producers: operand images from the raw rows =================
        const int n = tid - kEW * 32;  // this thread's candidate: pixel n / 4, sample n % 4
        const int p = n >> 2;
        const bool colin = p < npx && tx0 - R + p >= 0 && tx0 - R + p < a.W;
        const float4 *trow = reinterpret_cast<const float4 *>(tab + p * 16);
        const int vp = n / 3, vch = n - vp * 3;  // radiance item (n < 120): pixel vp, channel vch
        const bool vcolin = n < 120 && vp < npx && tx0 - R + vp >= 0 && tx0 - R + vp < a.W;
        for (int k = 0; k < nrows; k++) {
            const int s = k % kNS, r = k % kNR;
            if (k >= kNS && !mbar_wait(&sh.stage_empty[s], ((k / kNS) - 1) & 1, a.status)) {
                failed = true;
                break;
            }
            if (!mbar_wait(&sh.raw_full[r], (k / kNR) & 1, a.status)) {
                failed = true;
                break;
            }
            const float *rw = reinterpret_cast<const float *>(raw + r * kRawBytes);
            const int gy = ty0 - R + k;
            const bool rowin = gy >= 0 && gy < a.H;
            const float ycl = (float)(k - R) - 1.5f;
            float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, -kBig};
            if (rowin && colin && __float_as_int(rw[12 * kNCol + n]) != 0) {
                const float px = rw[0 * kNCol + n] * a.pscale - cx;
                const float py = rw[1 * kNCol + n] * a.pscale - cy;
                const float pz = rw[2 * kNCol + n] * a.pscale - cz;
                const float nx = rw[3 * kNCol + n], ny = rw[4 * kNCol + n], nz = rw[5 * kNCol + n];
                const float d2 = px * px + py * py + pz * pz;
                if (d2 <= kLimC) {
                    f[0] = px;
                    f[1] = py;
                    f[2] = pz;
                    f[3] = nx - nbx;
                    f[4] = ny - nby;
                    f[5] = nz - nbz;
                    f[6] = ycl;
                    f[7] = a.nscale * (nbx * nx + nby * ny + nbz * nz) - d2 + (-a.pix2 * ycl * ycl - a.nscale);
                }
            }
            float hi[8], lo[8];
#pragma unroll
            for (int i = 0; i < 8; i++) split_tf32(f[i], hi[i], lo[i]);
            uint8_t *st_base = stage + s * kStageBytes;
            store_row40(st_base + kimg_off(n, 0), hi, lo, hi, trow[0], trow[1], trow[2], trow[3]);
            if (n < 120) {  // incoming radiance in = rad + thr * out_next of the pixel's 4 samples, one channel
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (rowin && vcolin) {
                    const int4 vl = *reinterpret_cast<const int4 *>(rw + 12 * kNCol + vp * 4);
                    const float4 rd = *reinterpret_cast<const float4 *>(rw + (6 + vch) * kNCol + vp * 4);
                    const float4 th = *reinterpret_cast<const float4 *>(rw + (9 + vch) * kNCol + vp * 4);
                    const float4 on = a.out_next ? *reinterpret_cast<const float4 *>(rw + (13 + vch) * kNCol + vp * 4)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                    v.x = vl.x != 0 ? fmaf(th.x, on.x, rd.x) : 0.0f;
                    v.y = vl.y != 0 ? fmaf(th.y, on.y, rd.y) : 0.0f;
                    v.z = vl.z != 0 ? fmaf(th.z, on.z, rd.z) : 0.0f;
                    v.w = vl.w != 0 ? fmaf(th.w, on.w, rd.w) : 0.0f;
                }
                *reinterpret_cast<float4 *>(st_base + kCfBytes + (vch * kNCol + vp * 4) * 4) = v;
            }
            fence_async_smem();
            mbar_arrive1(&sh.stage_full[s]);
            mbar_arrive1(&sh.raw_empty[r]);
        }
    } else if (warp == kLoadWarp) {
        // ================= loader: one bulk copy per record field and window row =================
        if (lane == 0) {
            const int x_lo = tx0 - R;
            const int gx0 = x_lo > 0 ? x_lo : 0, gx1 = x_lo + npx < a.W ? x_lo + npx : a.W;
            const uint32_t raw0 = smem_u32(raw) + (uint32_t)(gx0 - x_lo) * 16u;
            const int nf = a.out_next ? kNF : 13;
            int last = -1;
            for (int k = 0; k < nrows; k++) {
                const int r = k % kNR;
                if (k >= kNR && !mbar_wait(&sh.raw_empty[r], ((k / kNR) - 1) & 1, a.status)) {
                    failed = true;
                    break;
                }
                const int gy = ty0 - R + k;
                if (gy >= 0 && gy < a.H && gx1 > gx0) {
                    const uint32_t bytes = (uint32_t)(gx1 - gx0) * 16u;
                    mbar_expect_tx(&sh.raw_full[r], bytes * (uint32_t)nf);
                    const size_t e0 = dbase + ((size_t)gy * a.W + gx0) * kS;
                    const uint32_t dst = raw0 + (uint32_t)r * kRawBytes;
                    for (int c = 0; c < 3; c++) {
                        bulk_g2s(dst + (0 + c) * kRawField, a.pos[c] + e0, bytes, &sh.raw_full[r]);
                        bulk_g2s(dst + (3 + c) * kRawField, a.nrm[c] + e0, bytes, &sh.raw_full[r]);
                        bulk_g2s(dst + (6 + c) * kRawField, a.rad[c] + e0, bytes, &sh.raw_full[r]);
                        bulk_g2s(dst + (9 + c) * kRawField, a.thr[c] + e0, bytes, &sh.raw_full[r]);
                        if (a.out_next)
                            bulk_g2s(dst + (13 + c) * kRawField, a.out_next + (size_t)c * N + (e0 - dbase), bytes,
                                     &sh.raw_full[r]);
                    }
                    bulk_g2s(dst + 12 * kRawField, a.valid + e0, bytes, &sh.raw_full[r]);
                } else {
                    mbar_arrive1(&sh.raw_full[r]);  // a row outside the image: nothing to copy
                }
                last = k;
            }
            // no copy may still be in flight when the CTA ends
            for (int k = last - kNR + 1 > 0 ? last - kNR + 1 : 0; k <= last; k++)
                mbar_wait(&sh.raw_full[k % kNR], (k / kNR) & 1, a.status);
        }
    } else if (warp == kMmaWarp) {
        // ================= MMA issue (one thread): the logits of every window row =================
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(kM, kNCol);
            const uint32_t st_addr = smem_u32(stage);
            int last = -1;
            bool ok = mbar_wait(&sh.qf_ready, 0, a.status);
            for (int k = 0; ok && k < nrows; k++) {
                const int b = k % kNB;
                if (!mbar_wait(&sh.stage_full[k % kNS], (k / kNS) & 1, a.status) ||
                    (k >= kNB && !mbar_wait(&sh.s_empty[b], ((k / kNB) - 1) & 1, a.status))) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t cf = st_addr + (uint32_t)(k % kNS) * kStageBytes;
                const uint32_t d = tmem + (uint32_t)b * kNCol;
#pragma unroll
                for (int kk = 0; kk < kK / 8; kk++)
                    mma_tf32_ts(d, tmem + kColQ + 8u * kk, make_desc(cf + kk * 256u, 128u, kRowGroup), idesc,
                                kk > 0 ? 1u : 0u);
                mma_commit(&sh.s_full[b]);
                mma_commit(&sh.stage_empty[k % kNS]);
                last = k;
            }
            if (!ok) {
                failed = true;
                // let the MMAs already issued finish before the columns are released
                if (last >= 0) mbar_wait(&sh.s_full[last % kNB], (last / kNB) & 1, a.status);
            }
        }
    } else {
        // ================= epilogue warps 0-7 =================
        const int qw = warp & 3, h = warp >> 2;
        const int tq = lane >> 2, tc = lane & 3;  // fragment row group and column pair
        const uint32_t colh = (uint32_t)h * kNH;
        if (h == 0) {
            // this thread's query feature row (lane = query)
            float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (qv) {
                f[0] = 2.0f * qp[0];
                f[1] = 2.0f * qp[1];
                f[2] = 2.0f * qp[2];
                f[3] = a.nscale * (qn[0] - nbx);
                f[4] = a.nscale * (qn[1] - nby);
                f[5] = a.nscale * (qn[2] - nbz);
                f[6] = 2.0f * a.pix2 * ((float)qrow - 1.5f);
                f[7] = 1.0f;
            }
            float hi[8], lo[8];
#pragma unroll
            for (int i = 0; i < 8; i++) split_tf32(f[i], hi[i], lo[i]);
            float oh[8];
#pragma unroll
            for (int i = 0; i < 8; i++) oh[i] = (qv && i == qx) ? 1.0f : 0.0f;
            // the row [qh | qh | ql | onehot | onehot] into TMEM (lane = query): the logits' A operand
            uint32_t row[kK];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                row[i] = __float_as_uint(hi[i]);
                row[8 + i] = __float_as_uint(hi[i]);
                row[16 + i] = __float_as_uint(lo[i]);
                row[24 + i] = __float_as_uint(oh[i]);
                row[32 + i] = __float_as_uint(oh[i]);
            }
            const uint32_t qa = tmem + ((uint32_t)(warp * 32) << 16) + kColQ;
            tmem_st16u(qa, row);
            tmem_st16u(qa + 16u, row + 16);
            tmem_st8u(qa + 32u, row + 32);
            tmem_wait_st();
            fence_before();
            mbar_arrive1(&sh.qf_ready);
        }
        // acc[q][c]: query q of this thread (lanes tq, tq + 8, 16 + tq, 24 + tq of the quarter), channel
        // c (r, g, b, weight); the two halves hold this thread's two candidate columns
        float2 acc[4][4];
        KahanF tot[4][4];
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                acc[q][c] = make_float2(0.f, 0.f);
                tot[q][c] = {0.f, 0.f};
            }
        for (int k = 0; k < nrows; k++) {
            const int b = k % kNB, s = k % kNS;
            if (!mbar_wait(&sh.s_full[b], (k / kNB) & 1, a.status)) {
                failed = true;
                break;
            }
            fence_after();
            const bool rows_in = k >= qw && k <= 2 * R + qw;  // |y_q - y_c| <= R for this warp's pixel row
            if (rows_in) {
                const uint32_t s0 = tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)b * kNCol + colh;
                const uint32_t s1 = s0 + (16u << 16);
                const float *vr =
                    reinterpret_cast<const float *>(stage + s * kStageBytes + kCfBytes) + colh + 2 * tc;
                uint32_t f0[16], f1[16];
                tmem_ld_frag4(s0, f0);
                tmem_ld_frag4(s1, f1);
                tmem_wait_ld();
                frag_sums<4>(f0, f1, vr, acc);
                tmem_ld_frag4(s0 + 32u, f0);
                tmem_ld_frag4(s1 + 32u, f1);
                tmem_wait_ld();
                frag_sums<4>(f0, f1, vr + 32, acc);
                tmem_ld_frag2(s0 + 64u, f0);
                tmem_ld_frag2(s1 + 64u, f1);
                tmem_wait_ld();
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive1(&sh.s_empty[b]);  // every logit of the row is in registers
                frag_sums<2>(f0, f1, vr + 64, acc);
            } else {
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive1(&sh.s_empty[b]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive1(&sh.stage_empty[s]);  // done with the radiance row
            if (k % kKahanRows == kKahanRows - 1 || k == nrows - 1) {
#pragma unroll
                for (int q = 0; q < 4; q++)
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        tot[q][c].add(acc[q][c].x + acc[q][c].y);
                        acc[q][c] = make_float2(0.f, 0.f);
                    }
            }
        }
        // each query's totals: add over the 4 column pairs (lanes tq * 4 + 0..3), then over the two
        // column halves (warps w and w + 4) through shared memory
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int ql = qw * 32 + (q >> 1) * 16 + (q & 1) * 8 + tq;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float v = tot[q][c].s - tot[q][c].c;
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                v += __shfl_xor_sync(0xffffffffu, v, 2);
                if (tc == 0) sh.part[h][ql][c] = v;
            }
        }
        bar_sync_n(1, kEW * 32);
        if (h == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) acc_out[c] = sh.part[0][tid][c] + sh.part[1][tid][c];
        }
    }

    // ---- outputs (threads 0-127), then release TMEM
    const bool any_failed = __syncthreads_or(failed) != 0;
    if (is_q && x < a.W && y < a.H) {
        f3 f = {0.0f, 0.0f, 0.0f}, o = {0.0f, 0.0f, 0.0f};
        if (qv) {
            if (any_failed) {
                f = {__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
                o = f;
            } else {
                const float iw = 1.0f / acc_out[3];
                f = {acc_out[0] * iw, acc_out[1] * iw, acc_out[2] * iw};
                o = style_apply(style, a.depth, f);
            }
        }
        a.out[qj] = o.x;
        a.out[N + qj] = o.y;
        a.out[2 * N + qj] = o.z;
        if (a.filtered) {
            a.filtered[qj] = f.x;
            a.filtered[N + qj] = f.y;
            a.filtered[2 * N + qj] = f.z;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == kMmaWarp) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

}  // namespace

// the bulk copies need every record plane (and out_next) on a 16-byte boundary
bool screen_tc_supports(const ScreenArgs &a, int spp) {
    if (spp != kS || (a.R != 15 && a.R != 16)) return false;
    auto al = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
    for (int c = 0; c < 3; c++)
        if (!al(a.pos[c]) || !al(a.nrm[c]) || !al(a.rad[c]) || !al(a.thr[c])) return false;
    return al(a.valid) && (a.out_next == nullptr || al(a.out_next));
}

sty_status launch_screen_tc(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st) {
    if (!screen_tc_supports(a, kS)) {
        set_error("k_pf_screen_tc: radius %d at 4 spp with 16-byte aligned planes required (radius 15 or 16)", a.R);
        return STY_ERR_ARG;
    }
    const size_t smem = kSmemBytes;
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_pf_screen_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_pf_screen_tc)"));
    dim3 grid((a.W + kTX - 1) / kTX, (a.H + kTY - 1) / kTY);
    k_pf_screen_tc<<<grid, kNT, smem, st>>>(a, style);
    return check_launch("k_pf_screen_tc");
}

}  // namespace sty
