// nrc_tc.cu -- the BF16 tcgen05 paths of the NRC MLP: inference and the fused training step, FP32
// accumulation in TMEM.
//
// Inference: persistent CTAs, one warpgroup per 128-sample tile (one sample per TMEM lane /
// thread), every layer's weights as BF16 UMMA operand images in shared memory, the activations in
// TMEM as the next layer's A operand (k_nrc_fwd_tc). Training: forward, loss gradient, backward and
// weight gradient of a tile in one kernel, the activations as shared-memory images (k_nrc_train_tc,
// one tile at a time; k_nrc_train_ws, two tiles in flight per SM).
// Operand images are K-major with no swizzle: an R x 64 matrix is stored as R/8 x 8 "core matrices"
// of 8 rows x 16 bytes, core matrix (rb, kb) at byte ((rb * 8) + kb) * 128, so the leading
// (K-direction) byte offset is 128 and the stride (8-row) byte offset is 1024.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "nrc.cuh"
#include "tc.cuh"

namespace sty {
namespace {
using namespace tc;

constexpr int W = kNrcWidth;
constexpr int TM = 128;                      // samples per tile (MMA M)
constexpr int kTileBytes = TM * W * 2;       // 16 KB activation tile
// byte offset of element (row, k) in a K-major no-swizzle image with 64 columns
__host__ __device__ __forceinline__ uint32_t img_off(uint32_t row, uint32_t k) {
    return (((row >> 3) * 8u + (k >> 3)) * 128u) + (row & 7u) * 16u + (k & 7u) * 2u;
}

// Frequency-encoding plan: encoded column pair p (columns 2p, 2p+1) is (sin, cos) of
// pi * 2^k * x[pdim[p]], with pfirst[p] marking k = 0 (a fresh sincospif; later octaves by the
// double-angle identities, in the order of nrc_encode); pdim = 0xff pads the row with zeros.
struct EncPlan {
    uint8_t pdim[kNrcWidth / 2];
    uint8_t pfirst[kNrcWidth / 2];
};
EncPlan make_plan(const NrcNet &n) {
    EncPlan e;
    int p = 0;
    for (int d = 0; d < n.in_dims; d++)
        for (uint32_t k = 0; k < n.freqs[d] && p < kNrcWidth / 2; k++, p++) {
            e.pdim[p] = (uint8_t)d;
            e.pfirst[p] = k == 0;
        }
    for (; p < kNrcWidth / 2; p++) {
        e.pdim[p] = 0xff;
        e.pfirst[p] = 0;
    }
    return e;
}

// the packed BF16 encoding of one sample (x = its input row, or nullptr for a padding row): column
// pair p in q[p] (sin in the low half)
__device__ __forceinline__ void encode_row_pack(const EncPlan &e, const float *x, uint32_t (&q)[kNrcWidth / 2]) {
    float s = 0.0f, c = 0.0f;
#pragma unroll
    for (int p = 0; p < kNrcWidth / 2; p++) {
        const uint32_t d = e.pdim[p];
        float vs = 0.0f, vc = 0.0f;
        if (d != 0xffu && x) {
            if (e.pfirst[p]) {
                sincospif(x[d], &s, &c);
            } else {
                const float s2 = 2.0f * s * c;
                c = fmaf(-2.0f * s, s, 1.0f);
                s = s2;
            }
            vs = s;
            vc = c;
        }
        q[p] = pack2_bf16(vs, vc);
    }
}

// The same encoding with the frequency table of the neural-cache workload network (11 inputs,
// octaves 4,4,4,3,3,3,3,2,2,2,2 -> 64 columns) fixed at compile time: every pair lands in a static
// register, no per-pair branch or table lookup.
constexpr int kC4Dims = 11;
__device__ constexpr int kC4Freqs[kC4Dims] = {4, 4, 4, 3, 3, 3, 3, 2, 2, 2, 2};
bool is_c4(const NrcNet &n) {
    if (n.in_dims != kC4Dims) return false;
    const int f[kC4Dims] = {4, 4, 4, 3, 3, 3, 3, 2, 2, 2, 2};
    for (int d = 0; d < kC4Dims; d++)
        if ((int)n.freqs[d] != f[d]) return false;
    return true;
}
// the packed BF16 encoding of an input row held in registers (has = false: a padding row of zeros)
__device__ __forceinline__ void encode_c4_pack(const float (&xin)[kC4Dims], bool has, uint32_t (&q)[kNrcWidth / 2]) {
    int o = 0;
#pragma unroll
    for (int d = 0; d < kC4Dims; d++) {
        float s, c;
        sincospif(xin[d], &s, &c);
#pragma unroll
        for (int k = 0; k < kC4Freqs[d]; k++) {
            q[o++] = has ? pack2_bf16(s, c) : 0u;
            const float s2 = 2.0f * s * c;
            c = fmaf(-2.0f * s, s, 1.0f);
            s = s2;
        }
    }
}
__device__ __forceinline__ void store_row(const uint32_t (&q)[kNrcWidth / 2], uint8_t *img, uint32_t row) {
#pragma unroll
    for (int kb = 0; kb < 8; kb++)
        *reinterpret_cast<uint4 *>(img + img_off(row, kb * 8)) =
            make_uint4(q[kb * 4], q[kb * 4 + 1], q[kb * 4 + 2], q[kb * 4 + 3]);
}
__device__ __forceinline__ void encode_any_pack(const EncPlan &e, bool c4, const float *x, uint32_t (&q)[kNrcWidth / 2]) {
    if (c4) {
        float xin[kC4Dims];
#pragma unroll
        for (int d = 0; d < kC4Dims; d++) xin[d] = x ? x[d] : 0.0f;
        encode_c4_pack(xin, x != nullptr, q);
    } else {
        encode_row_pack(e, x, q);
    }
}
// encode one sample into row `row` of a K-major image, one 16-byte store per 8 columns
__device__ __forceinline__ void encode_any(const NrcNet &n, const EncPlan &e, bool c4, const float *x, uint8_t *img,
                                           uint32_t row) {
    uint32_t q[kNrcWidth / 2];
    encode_any_pack(e, c4, x, q);
    store_row(q, img, row);
}
__device__ __forceinline__ void encode_row(const EncPlan &e, const float *x, uint8_t *img, uint32_t row) {
    uint32_t q[kNrcWidth / 2];
    encode_row_pack(e, x, q);
    store_row(q, img, row);
}


struct TcArgs {
    NrcNet n;
    EncPlan plan;
    int c4;  // the workload's frequency table: use encode_row_c4
    const uint16_t *wimg;  // global weight image
    uint64_t count;
    const float *input;
    float *output;
    uint32_t *status;
};

// Inference: one CTA per SM, kFwdWG warpgroups sharing one copy of the weight images in shared
// memory; each warpgroup owns one 128-sample tile at a time: 96 TMEM columns (a 64-column FP32
// accumulator and the next layer's A operand, 32 columns of BF16 pairs: element k of row m in lane
// m, column k / 2, half k % 2), an mbarrier and a named barrier. The activations never touch shared
// memory: per layer the warpgroup tcgen05.ld's its accumulator rows, applies ReLU and BF16 rounding
// and tcgen05.st's the row as the next layer's A; thread 0 issues 4 x tcgen05.mma (A from TMEM at
// +8 columns per K = 16 step, B the layer's weight image; N = 64, or 16 for the output layer) and
// commits to the mbarrier. Shared memory then carries only the B operands (2 KB per MMA instead of
// 6 KB plus a 16 KB activation store per layer); 5 tiles are in flight per SM (5 x 96 of the 512
// TMEM columns).
constexpr int kFwdWG = 5;
constexpr uint32_t kFwdCols = 96;
__device__ __forceinline__ void mma_bf16_ts(uint32_t tmem_d, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc));
}
// one row (32 lanes of this warp, 32 columns) of BF16 pairs into TMEM
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&q)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(q[0]), "r"(q[1]), "r"(q[2]), "r"(q[3]), "r"(q[4]), "r"(q[5]), "r"(q[6]), "r"(q[7]), "r"(q[8]), "r"(q[9]),
        "r"(q[10]), "r"(q[11]), "r"(q[12]), "r"(q[13]), "r"(q[14]), "r"(q[15]), "r"(q[16]), "r"(q[17]), "r"(q[18]),
        "r"(q[19]), "r"(q[20]), "r"(q[21]), "r"(q[22]), "r"(q[23]), "r"(q[24]), "r"(q[25]), "r"(q[26]), "r"(q[27]),
        "r"(q[28]), "r"(q[29]), "r"(q[30]), "r"(q[31])
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__global__ void __launch_bounds__(128 * kFwdWG, 1) k_nrc_fwd_tc(const TcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[kFwdWG];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, wg = tid >> 7, t = tid & 127;
    const uint32_t bar_id = 1u + (uint32_t)wg;
    const int L = a.n.layers;
    const uint32_t wbytes = (uint32_t)(L * W * W + kNrcOutPad * W) * 2u;
    uint8_t *wimg = smem;

    for (uint32_t o = tid * 16u; o < wbytes; o += 128u * kFwdWG * 16u)
        *reinterpret_cast<uint4 *>(wimg + o) =
            *reinterpret_cast<const uint4 *>(reinterpret_cast<const uint8_t *>(a.wimg) + o);
    if (tid == 0) {
        for (int g = 0; g < kFwdWG; g++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[g])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot + kFwdCols * (uint32_t)wg;  // accumulator
    const uint32_t areg = tmem + 64u;                            // A operand of the next layer
    const uint32_t lane_off = ((uint32_t)(warp & 3) * 32u) << 16;
    const uint32_t wbase = smem_u32(wimg);
    uint64_t *bar = &mbar[wg];
    uint32_t phase = 0;
    bool failed = false;  // uniform over the warpgroup (decided through bar.red.and)

    const uint64_t ntiles = (a.count + TM - 1) / TM;
    for (uint64_t tile = (uint64_t)blockIdx.x * kFwdWG + wg; tile < ntiles && !failed;
         tile += (uint64_t)gridDim.x * kFwdWG) {
        const uint64_t row = tile * TM + t;
        {
            uint32_t q[kNrcWidth / 2];
            encode_any_pack(a.plan, a.c4 != 0, row < a.count ? a.input + row * a.n.in_dims : nullptr, q);
            tmem_st32(areg + lane_off, q);
        }
        fence_before();
        wg_sync(bar_id);
        for (int l = 0; l <= L; l++) {
            const bool out_layer = l == L;
            if (t == 0) {
                fence_after();
                const uint32_t wl = wbase + (uint32_t)l * W * W * 2u;
                const uint32_t idesc = out_layer ? idesc_bf16(TM, kNrcOutPad) : idesc_bf16(TM, W);
#pragma unroll
                for (int kk = 0; kk < 4; kk++)
                    mma_bf16_ts(tmem, areg + 8u * kk, make_desc(wl + kk * 256u), idesc, kk > 0 ? 1u : 0u);
                mma_commit(bar);
            }
            const bool got = mbar_wait(bar, phase, a.status);
            if (!wg_sync_and(bar_id, got)) {
                failed = true;
                break;
            }
            phase ^= 1u;
            fence_after();
            if (!out_layer) {
                uint32_t q[kNrcWidth / 2];
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    float v[32];
                    tmem_ld32(tmem + lane_off + half * 32u, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < 16; j++) q[half * 16 + j] = pack2_relu_bf16(v[2 * j], v[2 * j + 1]);
                }
                tmem_st32(areg + lane_off, q);
            } else {
                float v[16];
                tmem_ld16(tmem + lane_off, v);
                tmem_wait_ld();
                if (row < a.count)
                    for (int c = 0; c < a.n.out_dims; c++) a.output[row * a.n.out_dims + c] = v[c];
            }
            fence_before();
            wg_sync(bar_id);
        }
    }
    if (failed) {
        // the last commit never arrived within the limit: give the MMA one more bounded wait before
        // the accumulator columns are released
        mbar_wait(bar, phase, a.status);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem_slot) : "memory");
}

// ---- fused BF16 training step --------------------------------------------------------------
// One CTA (one warpgroup) per SM, persistent over tiles of 128 samples of the batch. Per tile:
//   forward   act_{l+1} = relu(act_l W_l^T) (M=128, N=64, K=64), every act_l kept in shared memory
//             as a K-major image; pred = act_L W_out^T (N=16); g = dLoss/dpred (relative L2)
//   backward  dH_{L-1} = g W_out (K=16), dP_l = dH_l * [act_{l+1} > 0], dH_{l-1} = dP_l W_l
//             (B = the forward weight image read MN-major)
//   gradient  dW_l += dP_l^T act_l (M=64, N=64, K=128; both images read MN-major) and
//             dW_out^T += act_L^T g (M=64, N=16), accumulated in TMEM across the CTA's tiles.
// TMEM columns: 0-63 forward / backward accumulator (M=128: lane = sample); 64 + 64 l the M=64
// accumulator of dW_l (row j in lane (j / 16) * 32 + j % 16); 64 + 64 L the dW_out^T accumulator.
// At the end each CTA stores its sums to part + blockIdx.x * np (the flat parameter order) and the
// caller adds the CTAs' partials in order, so the gradient is deterministic for a device.
struct TrainArgs {
    NrcNet n;
    EncPlan plan;
    int c4;
    const uint16_t *wimg;
    uint32_t B;
    const float *input, *target;
    float *part;  // [gridDim.x][np]
    size_t np;
    float *loss;
    uint32_t *status;
};

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

__global__ void __launch_bounds__(128, 1) k_nrc_train_tc(const TrainArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ float red[4];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int L = a.n.layers, O = a.n.out_dims;
    const uint32_t wbytes = (uint32_t)(L * W * W + kNrcOutPad * W) * 2u;
    uint8_t *wimg = smem;
    uint8_t *acts = smem + ((wbytes + 1023u) & ~1023u);  // L + 1 activation images
    uint8_t *dtile = acts + (size_t)(L + 1) * kTileBytes;  // g, then dP_l
    for (uint32_t o = tid * 16u; o < wbytes; o += 128u * 16u)
        *reinterpret_cast<uint4 *>(wimg + o) =
            *reinterpret_cast<const uint4 *>(reinterpret_cast<const uint8_t *>(a.wimg) + o);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t lane_base = tmem + (((uint32_t)warp * 32u) << 16);
    const uint32_t wbase = smem_u32(wimg), abase = smem_u32(acts), dbase = smem_u32(dtile);
    const uint32_t wout = wbase + (uint32_t)L * W * W * 2u;
    const uint32_t c_out = 64u + 64u * (uint32_t)L;
    const float norm = 1.0f / ((float)a.B * (float)O);
    uint32_t phase = 0;
    bool failed = false;
    float lsum = 0.0f;
    bool first = true;  // first tile of this CTA: the dW accumulators start from zero

    // wait for the MMAs committed so far; CTA-uniform result
    auto sync_mma = [&]() -> bool {
        const bool got = mbar_wait(&mbar, phase, a.status);
        phase ^= 1u;
        if (!__syncthreads_and(got)) return false;
        fence_after();
        return true;
    };
    auto publish = [&]() {  // generic-proxy smem writes -> visible to the next MMAs
        fence_async_smem();
        fence_before();
        __syncthreads();
    };

    const uint32_t ntiles = (a.B + TM - 1) / TM;
    for (uint32_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const uint32_t row = tile * TM + tid;
        const bool valid = row < a.B;
        encode_any(a.n, a.plan, a.c4 != 0, valid ? a.input + (size_t)row * a.n.in_dims : nullptr, acts, tid);
        publish();
        // ---- forward
        for (int l = 0; l <= L && !failed; l++) {
            const bool out_layer = l == L;
            if (tid == 0) {
                fence_after();
                const uint32_t al = abase + (uint32_t)l * kTileBytes, wl = wbase + (uint32_t)l * W * W * 2u;
                const uint32_t idesc = out_layer ? idesc_bf16(TM, kNrcOutPad) : idesc_bf16(TM, W);
#pragma unroll
                for (int kk = 0; kk < 4; kk++)
                    mma_bf16(tmem, make_desc(al + kk * 256u), make_desc(wl + kk * 256u), idesc, kk > 0 ? 1u : 0u);
                mma_commit(&mbar);
            }
            if (!sync_mma()) {
                failed = true;
                break;
            }
            if (!out_layer) {
                uint8_t *nxt = acts + (size_t)(l + 1) * kTileBytes;
                float v[32];
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    tmem_ld32(lane_base + half * 32u, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int kb = 0; kb < 4; kb++) {
                        const uint4 q = make_uint4(pack2_relu_bf16(v[kb * 8 + 0], v[kb * 8 + 1]),
                                                   pack2_relu_bf16(v[kb * 8 + 2], v[kb * 8 + 3]),
                                                   pack2_relu_bf16(v[kb * 8 + 4], v[kb * 8 + 5]),
                                                   pack2_relu_bf16(v[kb * 8 + 6], v[kb * 8 + 7]));
                        *reinterpret_cast<uint4 *>(nxt + img_off(tid, half * 32 + kb * 8)) = q;
                    }
                }
            } else {
                // loss gradient of the relative L2 loss (prediction treated as a constant in the
                // denominator) into columns 0..15 of dtile; rows past the batch give zero
                float v[16], gr[16];
                tmem_ld16(lane_base, v);
                tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < 16; c++) {
                    gr[c] = 0.0f;
                    if (valid && c < O) {
                        const float p = v[c], t = a.target[(size_t)row * O + c];
                        const float den = p * p + 0.01f;
                        lsum += (p - t) * (p - t) / den;
                        gr[c] = 2.0f * (p - t) / den * norm;
                    }
                }
#pragma unroll
                for (int kb = 0; kb < 2; kb++) {
                    const uint4 q = make_uint4(pack2_bf16(gr[kb * 8 + 0], gr[kb * 8 + 1]),
                                               pack2_bf16(gr[kb * 8 + 2], gr[kb * 8 + 3]),
                                               pack2_bf16(gr[kb * 8 + 4], gr[kb * 8 + 5]),
                                               pack2_bf16(gr[kb * 8 + 6], gr[kb * 8 + 7]));
                    *reinterpret_cast<uint4 *>(dtile + img_off(tid, kb * 8)) = q;
                }
            }
            publish();
        }
        if (failed) break;
        // ---- output layer: dW_out^T += act_L^T g ; dH_{L-1} = g W_out
        if (tid == 0) {
            fence_after();
            const uint32_t aL = abase + (uint32_t)L * kTileBytes;
#pragma unroll 1
            for (int kk = 0; kk < TM / 16; kk++)
                mma_bf16(tmem + c_out, make_desc_mn(aL + kk * 2048u), make_desc_mn(dbase + kk * 2048u),
                         idesc_bf16(64, kNrcOutPad, 1, 1), (first && kk == 0) ? 0u : 1u);
            mma_bf16(tmem, make_desc(dbase), make_desc_mn(wout), idesc_bf16(TM, W, 0, 1), 0u);
            mma_commit(&mbar);
        }
        if (!sync_mma()) {
            failed = true;
            break;
        }
        // ---- hidden layers, last to first
        for (int l = L - 1; l >= 0; l--) {
            {
                // dP_l = dH_l * [act_{l+1} > 0] -> dtile
                const uint8_t *hl = acts + (size_t)(l + 1) * kTileBytes;
                float v[32];
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    tmem_ld32(lane_base + half * 32u, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int kb = 0; kb < 4; kb++) {
                        const uint32_t off = img_off(tid, half * 32 + kb * 8);
                        const uint4 h = *reinterpret_cast<const uint4 *>(hl + off);
                        const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
                        uint32_t o[4];
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const float d0 = bf16_lo(hw[e]) > 0.0f ? v[kb * 8 + 2 * e] : 0.0f;
                            const float d1 = bf16_hi(hw[e]) > 0.0f ? v[kb * 8 + 2 * e + 1] : 0.0f;
                            o[e] = pack2_bf16(d0, d1);
                        }
                        *reinterpret_cast<uint4 *>(dtile + off) = make_uint4(o[0], o[1], o[2], o[3]);
                    }
                }
            }
            publish();
            if (tid == 0) {
                fence_after();
                const uint32_t al = abase + (uint32_t)l * kTileBytes;
#pragma unroll 1
                for (int kk = 0; kk < TM / 16; kk++)
                    mma_bf16(tmem + 64u + 64u * (uint32_t)l, make_desc_mn(dbase + kk * 2048u),
                             make_desc_mn(al + kk * 2048u), idesc_bf16(64, W, 1, 1), (first && kk == 0) ? 0u : 1u);
                if (l > 0) {
                    const uint32_t wl = wbase + (uint32_t)l * W * W * 2u;
#pragma unroll
                    for (int kk = 0; kk < 4; kk++)
                        mma_bf16(tmem, make_desc(dbase + kk * 256u), make_desc_mn(wl + kk * 2048u),
                                 idesc_bf16(TM, W, 0, 1), kk > 0 ? 1u : 0u);
                }
                mma_commit(&mbar);
            }
            if (!sync_mma()) {
                failed = true;
                break;
            }
        }
        first = false;
    }
    if (failed) {
        mbar_wait(&mbar, phase, a.status);
    } else if (!first) {
        // this CTA's weight-gradient sums -> part[blockIdx.x]; M=64 rows live in lanes 0-15 of each
        // warp's quarter: row j = 16 * warp + lane
        float *dst = a.part + (size_t)blockIdx.x * a.np;
        const int j = 16 * warp + lane;
        for (int l = 0; l < L; l++) {
            float v[32];
#pragma unroll
            for (int half = 0; half < 2; half++) {
                tmem_ld32(lane_base + 64u + 64u * (uint32_t)l + half * 32u, v);
                tmem_wait_ld();
                if (lane < 16) {
                    float *d = dst + nrc_w_offset(l) + (size_t)j * W + half * 32;
#pragma unroll
                    for (int k = 0; k < 32; k += 4)
                        *reinterpret_cast<float4 *>(d + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
                }
            }
        }
        float v[16];
        tmem_ld16(lane_base + c_out, v);  // row = input column k, column = output c
        tmem_wait_ld();
        if (lane < 16)
            for (int c = 0; c < O; c++) dst[nrc_w_offset(L) + (size_t)c * W + j] = v[c];
    } else {
        // no tile: zero partials keep the ordered sum exact
        for (size_t p = tid; p < a.np; p += 128) a.part[(size_t)blockIdx.x * a.np + p] = 0.0f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) red[warp] = lsum;
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0 && a.loss) atomicAdd(a.loss, (red[0] + red[1] + red[2] + red[3]) * (1.0f / ((float)a.B * (float)O)));
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// Training with two tiles in flight per SM (networks of at most kWsMaxLayers hidden layers):
// warps 0-3 and 4-7 are two epilogue warpgroups, each walking every other tile of the CTA with its
// own activation images and 64-column TMEM accumulator (tile 2p in slot 0, tile 2p + 1 in slot 1).
// Three threads issue the MMAs: lane 0 of warp 8 + s the forward and dH products of slot s, lane 0
// of warp 10 every weight-gradient product. The hand-offs are mbarriers only: the issuers wait on
// ready[s] (the slot's 128 epilogue threads arrive once step k's operands are in shared memory) and
// arrive on done[s] (count 2: slot s's forward issuer and the weight-gradient issuer, each with a
// commit after its MMAs of step k or a plain arrive when it has none). One slot's epilogue overlaps
// the other's MMAs. The weight-gradient issuer alternates the slots step by step, so its MMAs reach
// each TMEM accumulator in the CTA's tile order: the per-CTA sums are those of k_nrc_train_tc bit
// for bit. (A thread issues an MMA every ~100 cycles here, so one issuer for a tile pair's 178 MMAs
// was the critical path.) The epilogue loads its next tile's input row and targets with
// non-reorderable loads a tile ahead, and for the workload's encoder keeps the tile's packed
// encoding in registers (act_0 is stored from them twice; the next tile's encoding is computed
// while the dW_0 products run), so neither a global load nor the sines sit on the step chain.
// Per slot, L images hold the L + 1 activations (act_L reuses act_0's image; act_0 is re-encoded
// for dW_0), dP_l overwrites act_{l+1} in place, and the 128 x 16 loss gradient g has its own
// compact image (2 core matrices per 8-row group: SBO 256 read K-major, LBO 256 read MN-major).
// TMEM: columns 0-63 / 64-127 the slots' accumulators, 128 + 64 l the dW_l sums, 128 + 64 L dW_out^T.
constexpr int kWsMaxLayers = 5;
std::atomic<int32_t> g_train_kernel{STY_NRC_TRAIN_KERNEL_AUTO};
bool one_tile_selected() { return g_train_kernel.load(std::memory_order_relaxed) == STY_NRC_TRAIN_KERNEL_ONE_TILE; }
constexpr uint32_t kGBytes = TM * kNrcOutPad * 2;  // 4 KB
constexpr int kWsThreads = 352;
__host__ __device__ inline int ws_images(int L) { return L < 2 ? 2 : L; }
__host__ __device__ inline uint32_t ws_slot_bytes(int L) { return (uint32_t)ws_images(L) * kTileBytes + kGBytes; }
__device__ __forceinline__ uint32_t g_off(uint32_t row, uint32_t kb) {  // 8 columns kb*8.. of row
    return ((row >> 3) * 2u + kb) * 128u + (row & 7u) * 16u;
}
// a global load issued where it is written (an asm volatile is not moved past the other volatile
// asm of the step loop), so its latency overlaps the steps before the value's first use
__device__ __forceinline__ float ld_early(const float *p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1) k_nrc_train_ws(const TrainArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t done[2], ready[2];
    __shared__ uint32_t tmem_slot;
    __shared__ float red[8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int L = a.n.layers, O = a.n.out_dims, nimg = ws_images(L);
    const uint32_t wbytes = (uint32_t)(L * W * W + kNrcOutPad * W) * 2u;
    uint8_t *wimg = smem;
    uint8_t *slots = smem + ((wbytes + 1023u) & ~1023u);
    for (uint32_t o = tid * 16u; o < wbytes; o += kWsThreads * 16u)
        *reinterpret_cast<uint4 *>(wimg + o) =
            *reinterpret_cast<const uint4 *>(reinterpret_cast<const uint8_t *>(a.wimg) + o);
    if (tid == 0) {
        for (int s = 0; s < 2; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(smem_u32(&done[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(&ready[s])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t wbase = smem_u32(wimg), sbase = smem_u32(slots);
    const uint32_t wout = wbase + (uint32_t)L * W * W * 2u;
    const uint32_t c_dw = 128u, c_out = 128u + 64u * (uint32_t)L;
    const uint32_t ntiles = (a.B + TM - 1) / TM;
    const uint32_t nt = blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
    const int nsteps = 2 * L + 2;
    bool failed = false;
    float lsum = 0.0f;

    if (warp >= 8) {
        // ---- MMA issuers: warp 8 + s forward + dH of slot s, warp 10 the weight gradients
        if (lane == 0) {
            const bool wgrad = warp == 10;
            const int own = warp - 8;  // the forward issuer's slot
            uint32_t rph[2] = {0u, 0u}, narr[2] = {0u, 0u};
            for (uint32_t i = 0; i < nt && !failed; i += 2) {
                const int nslot = i + 1 < nt ? 2 : 1;
                for (int k = 0; k < nsteps && !failed; k++) {
                    for (int s = 0; s < nslot; s++) {
                        if (!wgrad && s != own) continue;
                        if (!mbar_wait(&ready[s], rph[s], a.status)) {
                            failed = true;
                            break;
                        }
                        rph[s] ^= 1u;
                        fence_after();
                        const uint32_t acc = tmem + 64u * (uint32_t)s;
                        const uint32_t ab = sbase + (uint32_t)s * ws_slot_bytes(L);
                        const uint32_t gb = ab + (uint32_t)nimg * kTileBytes;
                        auto img = [&](int j) { return ab + (uint32_t)(j % nimg) * kTileBytes; };
                        bool issued = false;
                        if (!wgrad) {
                            if (k <= L) {  // forward layer k
                                const uint32_t al = img(k), wl = wbase + (uint32_t)k * W * W * 2u;
                                const uint32_t idesc = k == L ? idesc_bf16(TM, kNrcOutPad) : idesc_bf16(TM, W);
#pragma unroll
                                for (int kk = 0; kk < 4; kk++)
                                    mma_bf16(acc, make_desc(al + kk * 256u), make_desc(wl + kk * 256u), idesc,
                                             kk > 0 ? 1u : 0u);
                                issued = true;
                            } else if (k == L + 1) {  // dH_{L-1} = g W_out
                                mma_bf16(acc, make_desc(gb, 128, 256), make_desc_mn(wout), idesc_bf16(TM, W, 0, 1), 0u);
                                issued = true;
                            } else if (2 * L + 1 - k > 0) {  // dH_{l-1} = dP_l W_l
                                const int l = 2 * L + 1 - k;
                                const uint32_t dp = img(l + 1), wl = wbase + (uint32_t)l * W * W * 2u;
#pragma unroll
                                for (int kk = 0; kk < 4; kk++)
                                    mma_bf16(acc, make_desc(dp + kk * 256u), make_desc_mn(wl + kk * 2048u),
                                             idesc_bf16(TM, W, 0, 1), kk > 0 ? 1u : 0u);
                                issued = true;
                            }
                        } else if (k > L) {
                            const bool first = i + (uint32_t)s == 0;  // the CTA's first tile starts the sums
                            if (k == L + 1) {  // dW_out^T += act_L^T g
                                const uint32_t aL = img(L);
#pragma unroll 1
                                for (int kk = 0; kk < TM / 16; kk++)
                                    mma_bf16(tmem + c_out, make_desc_mn(aL + kk * 2048u),
                                             make_desc(gb + kk * 512u, 256, 128), idesc_bf16(64, kNrcOutPad, 1, 1),
                                             (first && kk == 0) ? 0u : 1u);
                            } else {  // dW_l += dP_l^T act_l
                                const int l = 2 * L + 1 - k;
                                const uint32_t dp = img(l + 1), al = img(l);
#pragma unroll 1
                                for (int kk = 0; kk < TM / 16; kk++)
                                    mma_bf16(tmem + c_dw + 64u * (uint32_t)l, make_desc_mn(dp + kk * 2048u),
                                             make_desc_mn(al + kk * 2048u), idesc_bf16(64, W, 1, 1),
                                             (first && kk == 0) ? 0u : 1u);
                            }
                            issued = true;
                        }
                        if (issued) mma_commit(&done[s]);
                        else mbar_arrive(&done[s]);
                        narr[s]++;
                    }
                }
            }
            if (failed)  // drain: this thread's MMAs complete before TMEM is released
                for (int s = 0; s < 2; s++)
                    if (narr[s]) mbar_wait(&done[s], (narr[s] - 1u) & 1u, a.status);
        }
        __syncwarp();
    } else {
        // ---- epilogue warpgroup s: one sample row per thread
        const int s = warp >> 2, r = tid & 127;
        const bool c4 = a.c4 != 0;
        const uint32_t lane_base = tmem + (((uint32_t)(warp & 3) * 32u) << 16) + 64u * (uint32_t)s;
        uint8_t *ab = slots + (size_t)s * ws_slot_bytes(L);
        uint8_t *gimg = ab + (size_t)nimg * kTileBytes;
        auto img = [&](int j) { return ab + (size_t)(j % nimg) * kTileBytes; };
        const float norm = 1.0f / ((float)a.B * (float)O);
        uint32_t dph = 0;
        auto publish = [&]() {
            fence_async_smem();
            fence_before();
            mbar_arrive(&ready[s]);
        };
        auto row_of = [&](uint32_t i) { return (blockIdx.x + i * gridDim.x) * TM + (uint32_t)r; };
        // input rows (workload encoder) and targets, loaded a tile ahead; q = the tile's packed encoding
        float xr[kC4Dims], tr[kNrcOutPad];
        uint32_t q[kNrcWidth / 2];
        auto valid_row = [&](uint32_t i) { return i < nt && row_of(i) < a.B; };
        auto load_x = [&](uint32_t i) {
            const bool v = c4 && valid_row(i);
            const float *p = a.input + (size_t)row_of(i) * kC4Dims;
#pragma unroll
            for (int d = 0; d < kC4Dims; d++) xr[d] = v ? ld_early(p + d) : 0.0f;
        };
        auto load_t = [&](uint32_t i) {
            const bool v = valid_row(i);
            const float *p = a.target + (size_t)row_of(i) * O;
#pragma unroll
            for (int c = 0; c < kNrcOutPad; c++) tr[c] = (v && c < O) ? ld_early(p + c) : 0.0f;
        };
        auto encode0 = [&](bool valid, const float *xin) {
            if (c4) store_row(q, img(0), (uint32_t)r);
            else encode_row(a.plan, xin, img(0), (uint32_t)r);
        };
        load_x((uint32_t)s);
        load_t((uint32_t)s);
        if (c4) encode_c4_pack(xr, valid_row((uint32_t)s), q);
        load_x((uint32_t)s + 2u);
        for (uint32_t i = (uint32_t)s; i < nt && !failed; i += 2) {
            const uint32_t row = row_of(i);
            const bool valid = row < a.B;
            const float *xin = valid ? a.input + (size_t)row * a.n.in_dims : nullptr;
            encode0(valid, xin);
            publish();
            for (int k = 0; k < nsteps; k++) {
                const bool got = __all_sync(0xffffffffu, mbar_wait(&done[s], dph, a.status));
                dph ^= 1u;
                if (!got) {
                    failed = true;
                    break;
                }
                fence_after();
                if (k == nsteps - 1) break;  // dW_0 done: the slot's images are free
                if (k < L) {  // act_{k+1} = relu(acc)
                    uint8_t *nxt = img(k + 1);
                    float v[2][32];
                    tmem_ld32(lane_base, v[0]);
                    tmem_ld32(lane_base + 32u, v[1]);
                    tmem_wait_ld();
#pragma unroll
                    for (int half = 0; half < 2; half++)
#pragma unroll
                        for (int kb = 0; kb < 4; kb++) {
                            const float *u = v[half] + kb * 8;
                            const uint4 q = make_uint4(pack2_relu_bf16(u[0], u[1]), pack2_relu_bf16(u[2], u[3]),
                                                       pack2_relu_bf16(u[4], u[5]), pack2_relu_bf16(u[6], u[7]));
                            *reinterpret_cast<uint4 *>(nxt + img_off((uint32_t)r, half * 32 + kb * 8)) = q;
                        }
                } else if (k == L) {  // relative-L2 loss gradient -> g (rows past the batch give zero)
                    float v[16], gr[16];
                    tmem_ld16(lane_base, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int c = 0; c < 16; c++) {
                        gr[c] = 0.0f;
                        if (valid && c < O) {
                            const float p = v[c], t = tr[c];
                            const float den = p * p + 0.01f;
                            lsum += (p - t) * (p - t) / den;
                            gr[c] = 2.0f * (p - t) / den * norm;
                        }
                    }
#pragma unroll
                    for (int kb = 0; kb < 2; kb++)
                        *reinterpret_cast<uint4 *>(gimg + g_off((uint32_t)r, (uint32_t)kb)) =
                            make_uint4(pack2_bf16(gr[kb * 8 + 0], gr[kb * 8 + 1]), pack2_bf16(gr[kb * 8 + 2], gr[kb * 8 + 3]),
                                       pack2_bf16(gr[kb * 8 + 4], gr[kb * 8 + 5]), pack2_bf16(gr[kb * 8 + 6], gr[kb * 8 + 7]));
                    load_t(i + 2);
                } else {  // dP_l = dH_l * [act_{l+1} > 0] in place of act_{l+1}, l = 2L - k
                    const int l = 2 * L - k;
                    uint8_t *hl = img(l + 1);
                    float v[2][32];
                    tmem_ld32(lane_base, v[0]);
                    tmem_ld32(lane_base + 32u, v[1]);
                    tmem_wait_ld();
#pragma unroll
                    for (int half = 0; half < 2; half++)
#pragma unroll
                        for (int kb = 0; kb < 4; kb++) {
                            const uint32_t off = img_off((uint32_t)r, half * 32 + kb * 8);
                            const uint4 h = *reinterpret_cast<const uint4 *>(hl + off);
                            const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
                            uint32_t o[4];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const float d0 = bf16_lo(hw[e]) > 0.0f ? v[half][kb * 8 + 2 * e] : 0.0f;
                                const float d1 = bf16_hi(hw[e]) > 0.0f ? v[half][kb * 8 + 2 * e + 1] : 0.0f;
                                o[e] = pack2_bf16(d0, d1);
                            }
                            *reinterpret_cast<uint4 *>(hl + off) = make_uint4(o[0], o[1], o[2], o[3]);
                        }
                    // act_L took act_0's image: store act_0 again for dW_0 (its image's last reader,
                    // the step of dW_{L-1}, has completed)
                    if (l == 0 && L % nimg == 0) encode0(valid, xin);
                }
                publish();
                if (k == 2 * L && c4) {  // the next tile's encoding, while the dW_0 products run
                    encode_c4_pack(xr, valid_row(i + 2), q);
                    load_x(i + 4);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0 && warp < 8) red[warp] = lsum;
    fence_before();
    const bool ok = __syncthreads_and(!failed);
    fence_after();
    if (ok && warp < 8) {
        float *dst = a.part + (size_t)blockIdx.x * a.np;
        if (nt == 0) {
            for (size_t p = tid; p < a.np; p += 256) dst[p] = 0.0f;
        } else {
            // M=64 accumulator row j lives in lane (j / 16) * 32 + j % 16: row j = 16 * (warp % 4) + lane
            const uint32_t qbase = tmem + (((uint32_t)(warp & 3) * 32u) << 16);
            const int j = 16 * (warp & 3) + lane;
            for (int l = warp >> 2; l < L; l += 2) {
                float v[2][32];
                tmem_ld32(qbase + c_dw + 64u * (uint32_t)l, v[0]);
                tmem_ld32(qbase + c_dw + 64u * (uint32_t)l + 32u, v[1]);
                tmem_wait_ld();
                if (lane < 16) {
                    float *d = dst + nrc_w_offset(l) + (size_t)j * W;
#pragma unroll
                    for (int half = 0; half < 2; half++)
#pragma unroll
                        for (int k = 0; k < 32; k += 4)
                            *reinterpret_cast<float4 *>(d + half * 32 + k) =
                                make_float4(v[half][k], v[half][k + 1], v[half][k + 2], v[half][k + 3]);
                }
            }
            if (warp < 4) {
                float v[16];
                tmem_ld16(qbase + c_out, v);  // row = input column k, column = output c
                tmem_wait_ld();
                if (lane < 16)
                    for (int c = 0; c < O; c++) dst[nrc_w_offset(L) + (size_t)c * W + j] = v[c];
            }
        }
    }
    if (tid == 0 && a.loss && ok) {
        float t = 0.0f;
        for (int w = 0; w < 8; w++) t += red[w];
        atomicAdd(a.loss, t * (1.0f / ((float)a.B * (float)O)));
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// FP32 [out][in] -> BF16 K-major images; output layer padded to 16 rows of zeros
__global__ void k_pack(NrcNet n, const float *w, uint16_t *img) {
    const int L = n.layers;
    const uint32_t total = (uint32_t)(L * W * W + kNrcOutPad * W);
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    uint32_t l, r, k;
    if (e < (uint32_t)(L * W * W)) {
        l = e / (W * W);
        r = (e % (W * W)) / W;
        k = e % W;
    } else {
        l = L;
        r = (e - L * W * W) / W;
        k = (e - L * W * W) % W;
    }
    float val = 0.0f;
    if (l < (uint32_t)L) val = w[nrc_w_offset(l) + r * W + k];
    else if (r < (uint32_t)n.out_dims) val = w[nrc_w_offset(L) + r * W + k];
    const __nv_bfloat16_raw b = __float2bfloat16_rn(val);
    const uint32_t base = l * W * W;  // elements; the output image (16 rows) starts after layer L-1
    img[base + img_off(r, k) / 2] = b.x;
}

}  // namespace

size_t nrc_tc_image_elems(const NrcNet &n) { return (size_t)n.layers * W * W + (size_t)kNrcOutPad * W; }

sty_status nrc_tc_pack(const NrcNet &n, const float *w, uint16_t *img, cudaStream_t st) {
    const uint32_t total = (uint32_t)nrc_tc_image_elems(n);
    k_pack<<<(total + 255) / 256, 256, 0, st>>>(n, w, img);
    return check_launch("k_pack");
}

sty_status nrc_tc_forward(const NrcNet &n, const uint16_t *img, uint64_t count, const float *input, float *output,
                          cudaStream_t st) {
    TcArgs a;
    a.n = n;
    a.plan = make_plan(n);
    a.c4 = is_c4(n) ? 1 : 0;
    a.wimg = img;
    a.count = count;
    a.input = input;
    a.output = output;
    a.status = device_status_ptr();
    if (!a.status) {
        set_error("device status word unavailable");
        return STY_ERR_CUDA;
    }
    const size_t wbytes = nrc_tc_image_elems(n) * 2;
    // at least 120 KB so that one CTA (and its 512 TMEM columns) owns the SM
    const size_t smem = std::max<size_t>(((wbytes + 1023) & ~(size_t)1023) + 1024, 122880);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_nrc_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "attr k_nrc_fwd_tc"));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t ntiles = (count + TM - 1) / TM;
    const uint64_t ctas = (ntiles + kFwdWG - 1) / kFwdWG;
    const uint64_t grid = ctas < (uint64_t)sms ? ctas : (uint64_t)sms;
    k_nrc_fwd_tc<<<(unsigned)grid, 128 * kFwdWG, smem, st>>>(a);
    return check_launch("k_nrc_fwd_tc");
}

size_t nrc_tc_train_smem(const NrcNet &n) {
    const size_t wbytes = nrc_tc_image_elems(n) * 2;
    const size_t need = ((wbytes + 1023) & ~(size_t)1023) + (size_t)(n.layers + 2) * kTileBytes + 1024;
    // at least 120 KB so that one CTA (and its 512 TMEM columns) owns the SM
    return need < 122880 ? 122880 : need;
}

uint32_t nrc_tc_train_ctas(uint32_t B) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t ntiles = (B + TM - 1) / TM;
    return ntiles < (uint32_t)sms ? ntiles : (uint32_t)sms;
}

sty_status nrc_tc_train(const NrcNet &n, const uint16_t *img, uint32_t B, const float *input, const float *target,
                        float *part, size_t np, float *loss, uint32_t ctas, cudaStream_t st) {
    if (n.layers > kNrcTcTrainMaxLayers) {
        set_error("tensor-core training supports at most %d hidden layers", kNrcTcTrainMaxLayers);
        return STY_ERR_ARG;
    }
    TrainArgs a;
    a.n = n;
    a.plan = make_plan(n);
    a.c4 = is_c4(n) ? 1 : 0;
    a.wimg = img;
    a.B = B;
    a.input = input;
    a.target = target;
    a.part = part;
    a.np = np;
    a.loss = loss;
    a.status = device_status_ptr();
    if (!a.status) {
        set_error("device status word unavailable");
        return STY_ERR_CUDA;
    }
    if (n.layers <= kWsMaxLayers && !one_tile_selected()) {
        const size_t wbytes = nrc_tc_image_elems(n) * 2;
        const size_t smem = ((wbytes + 1023) & ~(size_t)1023) + 2 * (size_t)ws_slot_bytes(n.layers) + 1024;
        STY_TRY(check_cuda(cudaFuncSetAttribute(k_nrc_train_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "attr k_nrc_train_ws"));
        k_nrc_train_ws<<<ctas, kWsThreads, smem, st>>>(a);
        return check_launch("k_nrc_train_ws");
    }
    const size_t smem = nrc_tc_train_smem(n);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_nrc_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "attr k_nrc_train_tc"));
    k_nrc_train_tc<<<ctas, 128, smem, st>>>(a);
    return check_launch("k_nrc_train_tc");
}

}  // namespace sty

using namespace sty;

sty_status sty_nrc_set_train_kernel(int32_t kernel) {
    clear_error();
    STY_ARG_CHECK(kernel == STY_NRC_TRAIN_KERNEL_AUTO || kernel == STY_NRC_TRAIN_KERNEL_ONE_TILE,
                  "sty_nrc_set_train_kernel: unknown kernel %d", kernel);
    g_train_kernel.store(kernel, std::memory_order_relaxed);
    return STY_OK;
}
