// nrc_grid.cu -- the reference's NL-NRC network (crates/akari_integrator/src/nrc_pt.rs:1159-1352):
// a Composite encoding of the 20 + max_depth inputs -- multiresolution hash grid on the position,
// one-blob on the next `blob_dims` inputs, identity on the rest -- and a ReLU MLP of width H without
// biases, linear output, relative L2, Adam + exponential decay, EMA weights for inference.
//
// Encoding (definitions restated from the published papers: tiny-cuda-nn is not available):
//   hash grid: level l: s_l = N_min b^l - 1, r_l = ceil(s_l) + 1, u = clamp(x, 0, 1) s_l + 0.5,
//     trilinear over the 8 corners of floor(u); as in tiny-cuda-nn, s_l is the FP32 evaluation
//     exp2(l log2 b) N_min - 1 and u = fma(x, s_l, 0.5) in FP32; table T_l = min(roundup8(r_l^3),
//     2^log2T) entries of F features, dense index when r_l^3 <= T_l else (c.x ^ c.y 2654435761 ^
//     c.z 805459861) in 32-bit arithmetic, both mod T_l. The forward reads FP16 copies of the
//     tables; the backward scatters w * dL/dfeature into the FP32 table gradient with atomics.
//   one-blob: bin k of B gets the mass of N(x, (1/B)^2) over [k/B, (k+1)/B] (erf).
// Inference (networks with H in {32, 64, 128}): k_grid_tiles writes the encoding as 128-row MMA
// operand tiles, k_grid_mlp_tc runs every layer on the tensor cores with the weights in shared
// memory. Training and other widths: the layer-by-layer path -- the encoding as row-major 16-bit
// [rows][E] (k_grid_enc, k_blob_ident), each layer product a tcgen05 GEMM with FP32 accumulation
// and a fused epilogue (gemm_tc.cu: ReLU into the next layer's 16-bit input; in the backward the
// ReLU mask of the layer below; the weight gradients reduced over the batch in a fixed order),
// 16-bit activations kept for the backward; output padded to 16. The MLP operands are BF16, or
// FP16 with STY_NRC_GRID_FP16 (tiny-cuda-nn's precision, with its loss scale of 128 on the
// backward so the per-sample gradients of a 2^16 batch stay out of the FP16 subnormals).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "gemm_tc.cuh"
#include "nrc.cuh"
#include "tc.cuh"

namespace sty {
namespace {
using namespace tc;

constexpr int kMaxLevels = 32;
constexpr int kOpad = 16;         // output columns of the layer-by-layer path (the MMA's N granule)
constexpr float kFp16LossScale = 128.0f;

struct GridGeo {
    int in_dims, levels, feats, blob_dims, bins, out_w;
    float scale[kMaxLevels];
    uint32_t res[kMaxLevels], size[kMaxLevels], off[kMaxLevels];
    int dense[kMaxLevels];
};

// Table entry of corner (cx, cy, cz) of level l. Hashed levels have power-of-two tables, so the
// modulo is a mask; a dense index is at most r + r^2 + r^3 < 2 T_l (corners reach r = the
// resolution), so one conditional subtraction is the modulo.
__device__ __forceinline__ uint32_t grid_index(const GridGeo &g, int l, uint32_t cx, uint32_t cy, uint32_t cz) {
    const uint32_t size = g.size[l];
    uint32_t h;
    if (g.dense[l]) {
        h = cx + cy * g.res[l] + cz * g.res[l] * g.res[l];
        h = h >= size ? h - size : h;
    } else {
        h = (cx ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (size - 1u);
    }
    return g.off[l] + h;
}

// F FP16 features of one table entry, as raw 32-bit words (F = 1: the low half)
template <int F>
struct RawEntry {
    uint32_t w[F >= 2 ? F / 2 : 1];
};
template <int F>
__device__ __forceinline__ RawEntry<F> load_entry(const __half *p) {
    RawEntry<F> r;
    if constexpr (F == 1) {
        r.w[0] = __ldg(reinterpret_cast<const unsigned short *>(p));
    } else if constexpr (F == 2) {
        r.w[0] = __ldg(reinterpret_cast<const unsigned int *>(p));
    } else if constexpr (F == 4) {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(p));
        r.w[0] = v.x;
        r.w[1] = v.y;
    } else {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
        r.w[0] = v.x;
        r.w[1] = v.y;
        r.w[2] = v.z;
        r.w[3] = v.w;
    }
    return r;
}
__device__ __forceinline__ float half_lo(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu))); }
__device__ __forceinline__ float half_hi(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w >> 16))); }

// Trilinear interpolation of level l at x (clamped to [0, 1]) from the FP16 tables, in three parts
// so that callers can keep several levels' loads in flight: the cell and FP32 weights, the 8
// corner loads, and acc[f] = sum_k w_k t_k[f] in corner order k = 0..7 (FMA).
__device__ __forceinline__ void level_cell(const GridGeo &g, int l, float x0, float x1, float x2, uint32_t (&c)[3],
                                           float (&w)[3]) {
    const float xs[3] = {x0, x1, x2};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float u = fmaf(fminf(fmaxf(xs[a], 0.0f), 1.0f), g.scale[l], 0.5f);
        const float f = floorf(u);
        c[a] = (uint32_t)f;
        w[a] = u - f;
    }
}
// For F = 2 and 4 the two x-neighbours k, k + 1 are fetched as one aligned two-entry load whenever
// they form such a pair (entries 2i and 2i + 1: a hashed level with c.x even always does, a dense
// level half the time; level offsets are multiples of 8 entries), else as two loads. The gathers
// are bound by L2 sector throughput, and this saves about a quarter of the sectors.
template <int F>
__device__ __forceinline__ void level_loads(const GridGeo &g, int l, const uint32_t (&c)[3],
                                            const __half *__restrict__ tab, RawEntry<F> (&e)[8]) {
    if constexpr (F == 2 || F == 4) {
        constexpr int kW = F / 2;
#pragma unroll
        for (int k = 0; k < 8; k += 2) {
            const uint32_t cy = c[1] + ((k >> 1) & 1), cz = c[2] + (k >> 2);
            const uint32_t i0 = grid_index(g, l, c[0], cy, cz), i1 = grid_index(g, l, c[0] + 1u, cy, cz);
            const RawEntry<2 * F> p = load_entry<2 * F>(tab + (size_t)(i0 & ~1u) * F);
            const bool hi = (i0 & 1u) != 0;  // i0 is the upper entry of the pair
#pragma unroll
            for (int w = 0; w < kW; w++) e[k].w[w] = hi ? p.w[kW + w] : p.w[w];
            if ((i0 ^ i1) == 1u) {
#pragma unroll
                for (int w = 0; w < kW; w++) e[k + 1].w[w] = hi ? p.w[w] : p.w[kW + w];
            } else {
                e[k + 1] = load_entry<F>(tab + (size_t)i1 * F);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++)
            e[k] = load_entry<F>(tab + (size_t)grid_index(g, l, c[0] + (k & 1), c[1] + ((k >> 1) & 1), c[2] + (k >> 2)) * F);
    }
}
template <int F>
__device__ __forceinline__ void level_sum(const RawEntry<F> (&e)[8], const float (&w)[3], float (&acc)[F]) {
#pragma unroll
    for (int f = 0; f < F; f++) acc[f] = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float wt = ((k & 1) ? w[0] : 1.0f - w[0]) * (((k >> 1) & 1) ? w[1] : 1.0f - w[1]) *
                         ((k >> 2) ? w[2] : 1.0f - w[2]);
#pragma unroll
        for (int f = 0; f < F; f++) {
            const uint32_t word = e[k].w[f / 2];
            acc[f] = fmaf(wt, (f & 1) ? half_hi(word) : half_lo(word), acc[f]);
        }
    }
}
template <int F>
__device__ __forceinline__ void gather_level(const GridGeo &g, int l, float x0, float x1, float x2,
                                             const __half *__restrict__ tab, float (&acc)[F]) {
    uint32_t c[3];
    float w[3];
    level_cell(g, l, x0, x1, x2, c, w);
    RawEntry<F> e[8];
    level_loads<F>(g, l, c, tab, e);
    level_sum<F>(e, w, acc);
}
// one-blob: mass of N(v, (1 / bins)^2) below bin edge k / bins
__device__ __forceinline__ float blob_cdf(int k, int bins, float v) {
    const float inv = 1.0f / ((1.0f / bins) * 1.41421356237f);
    return 0.5f * (1.0f + erff(((float)k / bins - v) * inv));
}
// encoded value of non-grid column G + r of input row xs: one-blob bin, identity or padding
__device__ __forceinline__ float extra_column(const GridGeo &g, int r, const float *xs) {
    const int nblob = g.blob_dims * g.bins, nident = g.in_dims - 3 - g.blob_dims;
    if (r < nblob) {
        const float v = xs[3 + r / g.bins];
        const int b = r % g.bins;
        return blob_cdf(b + 1, g.bins, v) - blob_cdf(b, g.bins, v);
    }
    if (r < nblob + nident) return xs[3 + g.blob_dims + (r - nblob)];
    return 0.0f;
}

// one thread per (sample, level): the level's F features into enc[s][l F ..]
template <int F>
__global__ void k_grid_enc(uint64_t n, const float *__restrict__ x, GridGeo g, const __half *__restrict__ tab,
                           uint16_t *__restrict__ enc, bool f16) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n * (uint64_t)g.levels) return;
    const uint64_t s = t / g.levels;
    const int l = (int)(t % g.levels);
    const float *xs = x + s * g.in_dims;
    float acc[F];
    gather_level<F>(g, l, xs[0], xs[1], xs[2], tab, acc);
    uint16_t *o = enc + s * g.out_w + (size_t)l * F;
#pragma unroll
    for (int f = 0; f < F; f++) o[f] = to16(acc[f], f16);
}
// one thread per (row, non-grid column): one-blob bins, identity dims, zero padding; consecutive
// threads write consecutive columns of a row
__global__ void k_blob_ident(uint64_t n, const float *__restrict__ x, GridGeo g, uint16_t *__restrict__ enc, bool f16) {
    const int G = g.levels * g.feats, nx = g.out_w - G;
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n * (uint64_t)nx) return;
    const uint64_t s = t / (uint64_t)nx;
    const int r = (int)(t % (uint64_t)nx);
    enc[s * g.out_w + G + r] = to16(extra_column(g, r, x + s * g.in_dims), f16);
}
// the hash-grid part of the backward: gtab[entry][f] += w * denc[s][l F + f], one vector atomic per
// corner for F >= 2 (the table gradient starts at a multiple of 16 floats: n_mlp = H (E + ...))
template <int F>
__global__ void k_grid_bwd(uint64_t n, const float *__restrict__ x, GridGeo g, const float *__restrict__ denc,
                           float *__restrict__ gtab) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n * (uint64_t)g.levels) return;
    const uint64_t s = t / g.levels;
    const int l = (int)(t % g.levels);
    const float *xs = x + s * g.in_dims;
    float w[3];
    uint32_t c[3];
    level_cell(g, l, xs[0], xs[1], xs[2], c, w);
    float d[F];
#pragma unroll
    for (int f = 0; f < F; f++) d[f] = denc[s * g.out_w + (size_t)l * F + f];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float wt = ((k & 1) ? w[0] : 1.0f - w[0]) * (((k >> 1) & 1) ? w[1] : 1.0f - w[1]) *
                         ((k >> 2) ? w[2] : 1.0f - w[2]);
        float *e = gtab + (size_t)grid_index(g, l, c[0] + (k & 1), c[1] + ((k >> 1) & 1), c[2] + (k >> 2)) * F;
        if constexpr (F == 4 || F == 8) {
#pragma unroll
            for (int h = 0; h < F / 4; h++)
                atomicAdd(reinterpret_cast<float4 *>(e) + h,
                          make_float4(wt * d[4 * h], wt * d[4 * h + 1], wt * d[4 * h + 2], wt * d[4 * h + 3]));
        } else if constexpr (F == 2) {
            atomicAdd(reinterpret_cast<float2 *>(e), make_float2(wt * d[0], wt * d[1]));
        } else {
            atomicAdd(e, wt * d[0]);
        }
    }
}
// relative L2 (prediction constant in the denominator): dP = 2 (p - t) / (p^2 + 0.01) / (B O), stored
// 16-bit times `scale` (the FP16 loss scale; 1 for BF16)
__global__ void k_rel_l2_grad(uint32_t B, int O, const float *__restrict__ pred, const float *__restrict__ tgt,
                              uint16_t *__restrict__ dp, float *__restrict__ loss, bool f16, float scale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < B) {
        const float norm = 1.0f / ((float)B * (float)O);
        for (int c = 0; c < kOpad; c++) {
            float g = 0.0f;
            if (c < O) {
                const float p = pred[(size_t)i * kOpad + c], t = tgt[(size_t)i * O + c];
                const float den = p * p + 0.01f;
                l += (p - t) * (p - t) / den;
                g = 2.0f * (p - t) / den * norm;
            }
            dp[(size_t)i * kOpad + c] = to16(g * scale, f16);
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l / ((float)B * (float)O));
}
// FP32 parameters -> 16-bit GEMM operands; the output layer padded to kOpad rows of zeros
__global__ void k_weights16(size_t n_mlp, size_t out_off, int O, int H, const float *__restrict__ w,
                            uint16_t *__restrict__ wb, bool f16) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = out_off + (size_t)kOpad * H;
    if (i >= total) return;
    float v = 0.0f;
    if (i < out_off) v = w[i];
    else if ((i - out_off) / H < (size_t)O) v = w[i];
    wb[i] = to16(v, f16);
    (void)n_mlp;
}
__global__ void k_out_rows(uint64_t n, int O, const float *__restrict__ pad, float *__restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n * (uint64_t)O) out[i] = pad[(i / O) * kOpad + i % O];
}
__device__ __forceinline__ uint32_t mix32(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return (uint32_t)x;
}
// MLP: uniform(+-sqrt(6 / (fan_in + fan_out))); tables: uniform(+-1e-4)
__global__ void k_grid_init(size_t n_mlp, size_t n_total, const int *fan_in, const int *fan_out, const size_t *layer_off,
                            int n_layers, uint64_t seed, float *w) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total) return;
    const float u = (mix32(seed * 0x9e3779b97f4a7c15ull + i) >> 8) * (1.0f / 16777216.0f) * 2.0f - 1.0f;
    if (i >= n_mlp) {
        w[i] = 1e-4f * u;
        return;
    }
    int l = 0;
    while (l + 1 < n_layers && i >= layer_off[l + 1]) l++;
    w[i] = u * sqrtf(6.0f / (float)(fan_in[l] + fan_out[l]));
}
__global__ void k_tab_half(size_t n, const float *__restrict__ t, __half *__restrict__ h) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) h[i] = __float2half_rn(t[i]);
}

// Optimiser step of the grid network: tiny-cuda-nn's Adam (the reference's "Adam" nested in
// "ExponentialDecay", nrc_pt.rs:1195-1213) and the reference's EMA (akari_tcnn.cu:42-83).
//   MLP weights (p < n_mlp): Adam with the global step t (bias corrections bc1 = 1 - b1^t,
//     bc2 = 1 - b2^t).
//   table entries: an entry whose gradient is exactly 0 this step keeps its weight, moments and
//     step count (tiny-cuda-nn's rule for non-matrix parameters); the others advance their own step
//     count t_p and use it in the bias correction. Updated entries refresh their FP16 copy.
//   EMA over every parameter: ema = (ema d (1 - d^(t-1)) + w (1 - d)) / (1 - d^t), with the FP16
//     copy of the EMA tables written in place.
// Four parameters per thread (the MLP block and the tables both start at multiples of 16 floats).
// A table entry's bias correction 1 - b^t for its own step count t is 1 - 2^(t log2 b) with log2 b
// computed once on the host (exp2f: a few instructions, where powf's exact-rounding path took most
// of the kernel's time in the divergent lanes of stepped entries).
__global__ void k_adam_grid(size_t n_mlp, size_t np, float *__restrict__ w, float *__restrict__ m,
                            float *__restrict__ v, const float *__restrict__ g, float *__restrict__ ema,
                            uint32_t *__restrict__ tsteps, __half *__restrict__ tab16, __half *__restrict__ tab16_ema,
                            float lr, float b1, float b2, float eps, float bc1, float bc2, float l2b1, float l2b2,
                            float ema_decay, float ema_old, float ema_new) {
    const size_t p0 = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) * 4;
    if (p0 >= np) return;
    const float4 g4 = *reinterpret_cast<const float4 *>(g + p0);
    float4 w4 = *reinterpret_cast<const float4 *>(w + p0);
    float4 e4 = *reinterpret_cast<const float4 *>(ema + p0);
    const float gr[4] = {g4.x, g4.y, g4.z, g4.w};
    float wn[4] = {w4.x, w4.y, w4.z, w4.w}, en[4] = {e4.x, e4.y, e4.z, e4.w};
    const bool table = p0 >= n_mlp;
    const bool any = !table || gr[0] != 0.0f || gr[1] != 0.0f || gr[2] != 0.0f || gr[3] != 0.0f;
    if (any) {
        float4 m4 = *reinterpret_cast<const float4 *>(m + p0), v4 = *reinterpret_cast<const float4 *>(v + p0);
        float mm[4] = {m4.x, m4.y, m4.z, m4.w}, vv[4] = {v4.x, v4.y, v4.z, v4.w};
        uint4 t4 = make_uint4(0u, 0u, 0u, 0u);
        if (table) t4 = *reinterpret_cast<const uint4 *>(tsteps + (p0 - n_mlp));
        uint32_t tp[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float c1 = bc1, c2 = bc2;
            if (table) {
                if (gr[k] == 0.0f) continue;  // untouched entry: weight, moments and step count stay
                tp[k] += 1u;
                c1 = 1.0f - exp2f((float)tp[k] * l2b1);
                c2 = 1.0f - exp2f((float)tp[k] * l2b2);
            }
            mm[k] = b1 * mm[k] + (1.0f - b1) * gr[k];
            vv[k] = b2 * vv[k] + (1.0f - b2) * gr[k] * gr[k];
            wn[k] -= lr * (mm[k] / c1) / (sqrtf(vv[k] / c2) + eps);
        }
        *reinterpret_cast<float4 *>(m + p0) = make_float4(mm[0], mm[1], mm[2], mm[3]);
        *reinterpret_cast<float4 *>(v + p0) = make_float4(vv[0], vv[1], vv[2], vv[3]);
        *reinterpret_cast<float4 *>(w + p0) = make_float4(wn[0], wn[1], wn[2], wn[3]);
        if (table) {
            *reinterpret_cast<uint4 *>(tsteps + (p0 - n_mlp)) = make_uint4(tp[0], tp[1], tp[2], tp[3]);
            __half2 *t16 = reinterpret_cast<__half2 *>(tab16 + (p0 - n_mlp));
            t16[0] = __floats2half2_rn(wn[0], wn[1]);
            t16[1] = __floats2half2_rn(wn[2], wn[3]);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) en[k] = (en[k] * ema_decay * ema_old + wn[k] * (1.0f - ema_decay)) * ema_new;
    *reinterpret_cast<float4 *>(ema + p0) = make_float4(en[0], en[1], en[2], en[3]);
    if (table) {
        __half2 *e16 = reinterpret_cast<__half2 *>(tab16_ema + (p0 - n_mlp));
        e16[0] = __floats2half2_rn(en[0], en[1]);
        e16[1] = __floats2half2_rn(en[2], en[3]);
    }
}

// ---- tensor-core inference --------------------------------------------------------------------------
// Two launches per chunk of rows:
//   k_grid_tiles   the encoding, written straight into 128-row tile images in the MMA A-operand
//                  layout (K-major core matrices, K = E columns). One thread per (row, unit):
//                  unit v < levels gathers hash-grid level v, unit levels + k writes columns
//                  G + 8k .. G + 8k + 7 (one-blob / identity / zero padding). A gather-bound kernel
//                  wants every warp slot of the SM for loads in flight, so it is kept apart from
//                  the MMA kernel, whose weights fill shared memory.
//   k_grid_mlp_tc  one persistent CTA per SM holding every layer's weights as BF16 operand images
//                  (W_0: H x E, W_1..W_{L-1}: H x H, W_out: 16 x H with rows >= O zero) and one
//                  activation image. Warps 0-7: per layer thread 0 issues K/16 x tcgen05.mma (M=128,
//                  N=H or 16, K=16) and commits to `bar_mma`; the warps wait (bounded), tcgen05.ld
//                  their rows (TMEM lane quarter warp % 4) and column half (warp / 4), apply ReLU,
//                  convert to BF16 and write them back as the next layer's A operand; after the
//                  output layer's MMA the image is released (`bar_free`) and warps 0-3 read the
//                  output columns. Warps 8-15 copy the next tile's image from global memory into
//                  registers while the current tile's layers run, then store it once `bar_free`
//                  completes and arrive on `bar_full`.
// Every wait is bounded: on a timeout the kernel sets STY_DEV_WAIT_TIMEOUT, waits once more for an
// MMA still in flight, frees its TMEM columns and returns.
constexpr int kTM = 128;
constexpr int kEpiThreads = 256;  // two warpgroups: TMEM lane quarter = warp % 4, column half = warp / 4
constexpr int kCopyThreads = 256;
constexpr int kMlpThreads = kEpiThreads + kCopyThreads;
constexpr int kMaxE = 160;  // encoded width the copy warps stage (10 x 16 bytes per thread)
constexpr int kCopyChunks = kTM * kMaxE * 2 / 16 / kCopyThreads;
constexpr int kOutN = 16;
constexpr uint64_t kInferChunk = 1ull << 18;  // rows per encode + MLP launch pair

// byte offset of (row, k) in a K-major no-swizzle image of K columns (core matrices of one 8-row
// group adjacent along K: LBO 128 bytes, SBO K * 16 bytes)
__host__ __device__ __forceinline__ uint32_t kimg_off(uint32_t row, uint32_t k, uint32_t K) {
    return ((row >> 3) * (K >> 3) + (k >> 3)) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}
// element offset of layer l's image (l = L: the output layer)
__host__ __device__ __forceinline__ size_t img_layer(int l, int H, int E) {
    return l == 0 ? 0 : (size_t)H * E + (size_t)(l - 1) * H * H;
}
// FP32 parameters -> the MMA kernel's BF16 weight images; grid (rows * K / 256, L + 1)
__global__ void k_grid_img(int H, int L, int E, int O, const float *__restrict__ w, uint16_t *__restrict__ img) {
    const int l = blockIdx.y;
    const uint32_t K = l == 0 ? (uint32_t)E : (uint32_t)H, R = l == L ? (uint32_t)kOutN : (uint32_t)H;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R * K) return;
    const uint32_t n = i / K, k = i % K;
    const size_t base = img_layer(l, H, E);  // also the layer's offset in the flat parameters
    const float v = (l < L || n < (uint32_t)O) ? w[base + (size_t)n * K + k] : 0.0f;
    img[base + kimg_off(n, k, K) / 2] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

// block = one tile x one unit (blockIdx.x = tile * units + unit, so a tile's units run together
// and its input rows are read while they are cached); rows >= count are written as zeros
// vec_x: every row starts 16-byte aligned (the host checks the pointer and in_dims % 4)
template <int F>
__global__ void __launch_bounds__(kTM) k_grid_tiles(uint64_t count, const float *__restrict__ x, GridGeo g,
                                                    int units, int vec_x, const __half *__restrict__ tab,
                                                    uint8_t *__restrict__ img) {
    const uint32_t m = threadIdx.x;
    const uint64_t tile = blockIdx.x / (uint32_t)units;
    const int v = (int)(blockIdx.x % (uint32_t)units);
    const uint64_t row = tile * kTM + m;
    const bool valid = row < count;
    const uint32_t E = (uint32_t)g.out_w;
    uint8_t *t = img + tile * (uint64_t)(kTM * E * 2u);
    const float *xs = x + (valid ? row : 0) * (uint64_t)g.in_dims;
    if (v < g.levels) {
        float acc[F];
#pragma unroll
        for (int f = 0; f < F; f++) acc[f] = 0.0f;
        if (valid) {
            // the divergent loads are what bound this kernel (L1): the position in one request
            // when rows are 16-byte aligned
            float p0, p1, p2;
            if (vec_x) {
                const float4 p = __ldg(reinterpret_cast<const float4 *>(xs));
                p0 = p.x;
                p1 = p.y;
                p2 = p.z;
            } else {
                p0 = xs[0];
                p1 = xs[1];
                p2 = xs[2];
            }
            gather_level<F>(g, v, p0, p1, p2, tab, acc);
        }
        uint8_t *p = t + kimg_off(m, (uint32_t)(v * F), E);
        if constexpr (F == 1) {
            *reinterpret_cast<unsigned short *>(p) = __bfloat16_as_ushort(__float2bfloat16_rn(acc[0]));
        } else if constexpr (F == 2) {
            *reinterpret_cast<uint32_t *>(p) = pack2_bf16(acc[0], acc[1]);
        } else if constexpr (F == 4) {
            *reinterpret_cast<uint2 *>(p) = make_uint2(pack2_bf16(acc[0], acc[1]), pack2_bf16(acc[2], acc[3]));
        } else {
            *reinterpret_cast<uint4 *>(p) = make_uint4(pack2_bf16(acc[0], acc[1]), pack2_bf16(acc[2], acc[3]),
                                                       pack2_bf16(acc[4], acc[5]), pack2_bf16(acc[6], acc[7]));
        }
        return;
    }
    const int G = g.levels * F, c0 = G + (v - g.levels) * 8;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int c = c0 + i;
        if (c < (int)E) {
            const float val = valid ? extra_column(g, c - G, xs) : 0.0f;
            *reinterpret_cast<unsigned short *>(t + kimg_off(m, (uint32_t)c, E)) =
                __bfloat16_as_ushort(__float2bfloat16_rn(val));
        }
    }
}

struct GridTcArgs {
    int E, H, L, O;
    const uint8_t *enc;  // tile images of the chunk (k_grid_tiles)
    const uint16_t *wimg;
    uint64_t count;
    float *output;
    uint32_t *status;
};

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(kMlpThreads, 1) k_grid_mlp_tc(const GridTcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar_mma, bar_full, bar_free;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int H = a.H, L = a.L, E = a.E;
    const uint32_t wbytes = (uint32_t)(img_layer(L, H, E) + (size_t)kOutN * H) * 2u;
    uint8_t *act = smem + ((wbytes + 1023u) & ~1023u);
    for (uint32_t o = tid * 16u; o < wbytes; o += kMlpThreads * 16u)
        *reinterpret_cast<uint4 *>(smem + o) =
            *reinterpret_cast<const uint4 *>(reinterpret_cast<const uint8_t *>(a.wimg) + o);
    if (tid == 0) {
        mbar_init(&bar_mma, 1);
        mbar_init(&bar_full, kCopyThreads);
        mbar_init(&bar_free, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"((uint32_t)H)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t ntiles = (a.count + kTM - 1) / kTM;

    if (tid < kEpiThreads) {
        // ---- MMA issue + epilogue ----
        const uint32_t t = (uint32_t)(tid & 127), half = (uint32_t)(warp >> 2);
        const uint32_t lane_base = tmem + (((uint32_t)(warp & 3) * 32u) << 16);
        const uint32_t wbase = smem_u32(smem), abase = smem_u32(act);
        const uint32_t hc = (uint32_t)H / 2u, c_lo = half * hc;  // this warp's columns
        uint32_t phase = 0, it = 0;
        bool failed = false, pending = false;
        for (uint64_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x, it++) {
            const bool got = mbar_wait(&bar_full, it & 1u, a.status);
            if (!bar_and_n(1, kEpiThreads, got)) {
                failed = true;
                break;
            }
            const uint64_t row = tile * kTM + t;
            for (int l = 0; l <= L; l++) {
                const bool out_layer = l == L;
                const uint32_t K = l == 0 ? (uint32_t)E : (uint32_t)H;
                if (tid == 0) {
                    fence_after();
                    const uint32_t wl = wbase + (uint32_t)img_layer(l, H, E) * 2u;
                    const uint32_t idesc = out_layer ? idesc_bf16(kTM, kOutN) : idesc_bf16(kTM, (uint32_t)H);
                    for (uint32_t kk = 0; kk < K / 16u; kk++)
                        mma_bf16(tmem, make_desc(abase + kk * 256u, 128u, K * 16u),
                                 make_desc(wl + kk * 256u, 128u, K * 16u), idesc, kk > 0 ? 1u : 0u);
                    mma_commit(&bar_mma);
                }
                pending = true;
                const bool ok = mbar_wait(&bar_mma, phase, a.status);
                if (!bar_and_n(1, kEpiThreads, ok)) {
                    failed = true;
                    break;
                }
                pending = false;
                phase ^= 1u;
                fence_after();
                if (!out_layer) {
                    for (uint32_t c = c_lo; c < c_lo + hc; c += 16u) {
                        float v[16];
                        tmem_ld16(lane_base + c, v);
                        tmem_wait_ld();
#pragma unroll
                        for (int kb = 0; kb < 2; kb++) {
                            const uint4 q = make_uint4(pack2_relu_bf16(v[kb * 8 + 0], v[kb * 8 + 1]),
                                                       pack2_relu_bf16(v[kb * 8 + 2], v[kb * 8 + 3]),
                                                       pack2_relu_bf16(v[kb * 8 + 4], v[kb * 8 + 5]),
                                                       pack2_relu_bf16(v[kb * 8 + 6], v[kb * 8 + 7]));
                            *reinterpret_cast<uint4 *>(act + kimg_off(t, c + kb * 8u, (uint32_t)H)) = q;
                        }
                    }
                    fence_async_smem();
                } else {
                    if (tid == 0) mbar_arrive(&bar_free);  // the output MMA has read the last activations
                    if (half == 0) {
                        float v[16];
                        tmem_ld16(lane_base, v);
                        tmem_wait_ld();
                        if (row < a.count)
                            for (int c = 0; c < a.O; c++) a.output[row * a.O + c] = v[c];
                    }
                }
                fence_before();
                bar_sync_n(1, kEpiThreads);
            }
        }
        if (failed && pending) mbar_wait(&bar_mma, phase, a.status);
    } else {
        // ---- copy warps: the next tile's image through registers ----
        const uint32_t e = (uint32_t)(tid - kEpiThreads);
        const uint32_t chunks = (uint32_t)(kTM * E * 2) / 16u;  // 16-byte chunks per tile image
        uint32_t it = 0;
        for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
            const uint4 *src = reinterpret_cast<const uint4 *>(a.enc + tile * (uint64_t)(kTM * E * 2));
            uint4 r[kCopyChunks];
#pragma unroll
            for (int i = 0; i < kCopyChunks; i++) {
                const uint32_t c = e + (uint32_t)i * kCopyThreads;
                if (c < chunks) r[i] = __ldcs(src + c);  // read once: evict first
            }
            if (!mbar_wait(&bar_free, (it & 1u) ^ 1u, a.status)) break;
#pragma unroll
            for (int i = 0; i < kCopyChunks; i++) {
                const uint32_t c = e + (uint32_t)i * kCopyThreads;
                if (c < chunks) reinterpret_cast<uint4 *>(act)[c] = r[i];
            }
            fence_async_smem();
            mbar_arrive(&bar_full);
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot), "r"((uint32_t)H)
                     : "memory");
}

}  // namespace

struct GridModel {
    sty_nrc_grid_config cfg;
    GridGeo geo;
    int H, L, O, E;
    size_t n_mlp, n_tab, out_off;
    std::vector<size_t> loff;  // FP32 offsets of W_0 .. W_L (W_L = output layer)
    bool f16 = false;          // MLP operands FP16 (else BF16)
    float loss_scale = 1.0f;   // the backward's scale of the loss gradient (FP16: 128)
    uint16_t *wb = nullptr, *wb_ema = nullptr;  // 16-bit weights: W_0 .. W_{L-1}, W_out padded to kOpad rows
    __half *tab16 = nullptr, *tab16_ema = nullptr;  // FP16 copies of the tables the forward reads
    bool tab16_valid = false;     // tab16 == fp16(current tables) (kept by k_adam_grid)
    bool tab16_ema_valid = false; // tab16_ema == fp16(EMA tables) (kept by k_adam_grid)
    uint32_t *tsteps = nullptr;   // per-entry Adam step counts of the tables
    // tensor-core inference (k_grid_tiles + k_grid_mlp_tc): BF16 weight images, the MMA kernel's
    // shared memory, the chunk's tile images
    bool tc = false;
    size_t img_elems = 0, tc_smem = 0;
    uint16_t *img = nullptr, *img_ema = nullptr;
    uint8_t *tiles = nullptr;
    uint64_t tiles_cap = 0;
    // batch scratch: 16-bit encoding and activations, two layer-gradient buffers, FP32 output /
    // encoding gradient, the weight gradients' per-chunk partial sums
    uint64_t cap = 0;
    uint16_t *enc = nullptr, *acts = nullptr, *dp = nullptr, *dp2 = nullptr;
    float *z = nullptr, *dh = nullptr, *parts = nullptr;
    int *d_fan_in = nullptr, *d_fan_out = nullptr;
    size_t *d_loff = nullptr;
};

namespace {

sty_status ensure_cap(GridModel *g, uint64_t B) {
    if (B <= g->cap) return STY_OK;
    void *ptrs[] = {g->enc, g->acts, g->dp, g->dp2, g->z, g->dh, g->parts};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    g->enc = g->acts = g->dp = g->dp2 = nullptr;
    g->z = g->dh = g->parts = nullptr;
    g->cap = 0;
    STY_ARG_CHECK(B < (1ull << 31), "batch of %llu rows too large", (unsigned long long)B);
    const size_t wide = (size_t)std::max({g->H, g->E, kOpad});
    const size_t parts = tc_dw_partials_floats((int)B, std::max({g->H, g->E, kOpad}));
    STY_TRY(check_cuda(cudaMalloc(&g->enc, B * g->E * 2), "alloc encoding"));
    STY_TRY(check_cuda(cudaMalloc(&g->acts, (size_t)g->L * B * g->H * 2), "alloc activations"));
    STY_TRY(check_cuda(cudaMalloc(&g->dp, B * wide * 2), "alloc layer gradient"));
    STY_TRY(check_cuda(cudaMalloc(&g->dp2, B * wide * 2), "alloc layer gradient"));
    STY_TRY(check_cuda(cudaMalloc(&g->z, B * wide * 4), "alloc output"));
    STY_TRY(check_cuda(cudaMalloc(&g->dh, B * wide * 4), "alloc encoding gradient"));
    STY_TRY(check_cuda(cudaMalloc(&g->parts, parts * 4), "alloc weight-gradient partials"));
    g->cap = B;
    return STY_OK;
}

// forward of B rows with the given 16-bit weights and FP16 tables: leaves enc, acts (for the
// backward) and the padded output (B x kOpad, FP32) in g->z
sty_status grid_forward(GridModel *g, uint64_t B, const float *x, const __half *tables, const uint16_t *wb,
                        cudaStream_t st) {
    const uint64_t nl = B * (uint64_t)g->geo.levels;
    const unsigned blocks = (unsigned)((nl + 255) / 256);
    switch (g->geo.feats) {
        case 1: k_grid_enc<1><<<blocks, 256, 0, st>>>(B, x, g->geo, tables, g->enc, g->f16); break;
        case 2: k_grid_enc<2><<<blocks, 256, 0, st>>>(B, x, g->geo, tables, g->enc, g->f16); break;
        case 4: k_grid_enc<4><<<blocks, 256, 0, st>>>(B, x, g->geo, tables, g->enc, g->f16); break;
        default: k_grid_enc<8><<<blocks, 256, 0, st>>>(B, x, g->geo, tables, g->enc, g->f16); break;
    }
    STY_TRY(check_launch("k_grid_enc"));
    const uint64_t nx = B * (uint64_t)(g->E - g->geo.levels * g->geo.feats);
    k_blob_ident<<<(unsigned)((nx + 255) / 256), 256, 0, st>>>(B, x, g->geo, g->enc, g->f16);
    STY_TRY(check_launch("k_blob_ident"));
    const uint16_t *a = g->enc;
    int K = g->E;
    for (int l = 0; l < g->L; l++) {  // z = a W_l^T, ReLU into the next layer's 16-bit input
        uint16_t *nx = g->acts + (size_t)l * B * g->H;
        STY_TRY(tc_gemm_rows(a, K, wb + g->loff[l], (int)B, K, g->H, false, g->f16, kEpiRelu16, nullptr, nx, nullptr,
                             1.0f, st));
        a = nx;
        K = g->H;
    }
    return tc_gemm_rows(a, g->H, wb + g->out_off, (int)B, g->H, kOpad, false, g->f16, kEpiF32, g->z, nullptr, nullptr,
                        1.0f, st);
}

// the two tensor-core launches per chunk of kInferChunk rows (tile images in g->tiles)
sty_status grid_tc_forward(GridModel *g, bool ema, uint64_t count, const float *in, float *out, cudaStream_t st) {
    const uint64_t chunk = std::min<uint64_t>(count, kInferChunk);
    const uint64_t tile_bytes = (uint64_t)kTM * g->E * 2;
    const uint64_t need = (chunk + kTM - 1) / kTM * tile_bytes;
    if (need > g->tiles_cap) {
        if (g->tiles) cudaFree(g->tiles);
        g->tiles = nullptr;
        g->tiles_cap = 0;
        STY_TRY(check_cuda(cudaMalloc(&g->tiles, need), "alloc tile images"));
        g->tiles_cap = need;
    }
    GridTcArgs a;
    a.E = g->E;
    a.H = g->H;
    a.L = g->L;
    a.O = g->O;
    a.enc = g->tiles;
    a.wimg = ema ? g->img_ema : g->img;
    a.status = device_status_ptr();
    if (!a.status) {
        set_error("device status word unavailable");
        return STY_ERR_CUDA;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int smem = (int)g->tc_smem;
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_grid_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                       "attr k_grid_mlp_tc"));
    const int units = g->geo.levels + (g->E - g->geo.levels * g->geo.feats + 7) / 8;
    const __half *tab = ema ? g->tab16_ema : g->tab16;
    for (uint64_t b0 = 0; b0 < count; b0 += chunk) {
        const uint64_t B = std::min<uint64_t>(chunk, count - b0);
        const uint64_t ntiles = (B + kTM - 1) / kTM;
        const float *x = in + b0 * g->geo.in_dims;
        const unsigned blocks = (unsigned)(ntiles * (uint64_t)units);
        const int vx = (g->geo.in_dims % 4 == 0 && reinterpret_cast<uintptr_t>(x) % 16 == 0) ? 1 : 0;
        switch (g->geo.feats) {
            case 1: k_grid_tiles<1><<<blocks, kTM, 0, st>>>(B, x, g->geo, units, vx, tab, g->tiles); break;
            case 2: k_grid_tiles<2><<<blocks, kTM, 0, st>>>(B, x, g->geo, units, vx, tab, g->tiles); break;
            case 4: k_grid_tiles<4><<<blocks, kTM, 0, st>>>(B, x, g->geo, units, vx, tab, g->tiles); break;
            default: k_grid_tiles<8><<<blocks, kTM, 0, st>>>(B, x, g->geo, units, vx, tab, g->tiles); break;
        }
        STY_TRY(check_launch("k_grid_tiles"));
        a.count = B;
        a.output = out + b0 * g->O;
        k_grid_mlp_tc<<<(unsigned)std::min<uint64_t>(ntiles, (uint64_t)sms), kMlpThreads, smem, st>>>(a);
        STY_TRY(check_launch("k_grid_mlp_tc"));
    }
    return STY_OK;
}

}  // namespace

// ---- interface used by nrc.cu ----------------------------------------------------------------------
sty_status grid_create(const sty_nrc_grid_config *c, GridModel **out, size_t *n_params, size_t *n_mlp) {
    STY_ARG_CHECK(c->grid_levels >= 1 && c->grid_levels <= kMaxLevels, "grid_levels must be in [1, %d]", kMaxLevels);
    STY_ARG_CHECK(c->grid_features == 1 || c->grid_features == 2 || c->grid_features == 4 || c->grid_features == 8,
                  "grid_features must be 1, 2, 4 or 8");
    STY_ARG_CHECK(c->log2_table >= 4 && c->log2_table <= 24, "log2_table must be in [4, 24]");
    STY_ARG_CHECK(c->input_dims >= 3 + c->blob_dims && c->input_dims <= 64, "input_dims must cover 3 + blob_dims");
    STY_ARG_CHECK(c->blob_bins >= 1 && c->blob_bins <= 16, "blob_bins must be in [1, 16]");
    STY_ARG_CHECK(c->hidden_units % 16 == 0 && c->hidden_units >= 16 && c->hidden_units <= 256,
                  "hidden_units must be a multiple of 16 in [16, 256]");
    STY_ARG_CHECK(c->hidden_layers >= 1 && c->hidden_layers <= 8, "hidden_layers must be in [1, 8]");
    STY_ARG_CHECK(c->output_dims >= 1 && c->output_dims <= kOpad, "output_dims must be in [1, %d]", kOpad);
    STY_ARG_CHECK((c->flags & ~(STY_NRC_GRID_LAYERED | STY_NRC_GRID_FP16)) == 0, "unknown flags 0x%x", c->flags);
    STY_ARG_CHECK(c->base_resolution >= 2 && c->per_level_scale >= 1.0f, "bad grid resolution");
    GridModel *g = new GridModel();
    g->cfg = *c;
    GridGeo &geo = g->geo;
    geo.in_dims = (int)c->input_dims;
    geo.levels = (int)c->grid_levels;
    geo.feats = (int)c->grid_features;
    geo.blob_dims = (int)c->blob_dims;
    geo.bins = (int)c->blob_bins;
    uint64_t off = 0;
    for (int l = 0; l < geo.levels; l++) {
        // FP32 like tiny-cuda-nn's grid_scale / grid_resolution
        const float scale = std::exp2((float)l * std::log2(c->per_level_scale)) * (float)c->base_resolution - 1.0f;
        STY_ARG_CHECK(std::isfinite(scale) && scale < 2147483648.0f, "grid level %d resolution overflows", l);
        const uint64_t res = (uint64_t)std::ceil(scale) + 1;
        STY_ARG_CHECK(res < (1ull << 31), "grid level %d resolution overflows", l);
        // r^3 exceeds 64 bits at the finest levels of deep grids: compare in double first
        const uint64_t cap = 1ull << c->log2_table;
        const bool fits = (double)res * (double)res * (double)res <= (double)cap;
        const uint64_t size = fits ? std::min<uint64_t>((res * res * res + 7) / 8 * 8, cap) : cap;
        geo.scale[l] = scale;
        geo.res[l] = (uint32_t)res;
        geo.size[l] = (uint32_t)size;
        geo.dense[l] = fits && res * res * res <= size;
        geo.off[l] = (uint32_t)off;
        off += size;
    }
    const int enc = geo.levels * geo.feats + geo.blob_dims * geo.bins + (geo.in_dims - 3 - geo.blob_dims);
    geo.out_w = (enc + 15) / 16 * 16;
    if (geo.out_w > 256) {
        set_error("encoded width %d exceeds 256 (the GEMMs' operand width)", geo.out_w);
        delete g;
        return STY_ERR_ARG;
    }
    g->f16 = (c->flags & STY_NRC_GRID_FP16) != 0;
    g->loss_scale = g->f16 ? kFp16LossScale : 1.0f;
    g->E = geo.out_w;
    g->H = (int)c->hidden_units;
    g->L = (int)c->hidden_layers;
    g->O = (int)c->output_dims;
    size_t o = 0;
    for (int l = 0; l < g->L; l++) {
        g->loff.push_back(o);
        o += (size_t)g->H * (l == 0 ? g->E : g->H);
    }
    g->out_off = o;
    g->loff.push_back(o);
    g->n_mlp = o + (size_t)g->O * g->H;  // a multiple of 16 (H is), as the tables' size is of 8 entries
    g->n_tab = off * geo.feats;
    *n_params = g->n_mlp + g->n_tab;
    *n_mlp = g->n_mlp;
    // the tensor-core path: H in {32, 64, 128} (one TMEM column per unit), E <= kMaxE (what the copy
    // warps stage), weight images + one 128-row activation image within the opt-in shared memory
    int dev = 0, smem_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g->img_elems = img_layer(g->L, g->H, g->E) + (size_t)kOutN * g->H;
    g->tc_smem = ((g->img_elems * 2 + 1023) & ~(size_t)1023) + (size_t)kTM * std::max(g->E, g->H) * 2 + 1024;
    // (BF16 only: FP16 networks infer layer by layer on the same tensor-core GEMMs as training)
    g->tc = !g->f16 && (g->H == 32 || g->H == 64 || g->H == 128) && g->E <= kMaxE &&
            g->tc_smem + 64 <= (size_t)smem_optin;
    sty_status s = check_cuda(cudaMalloc(&g->wb, (g->out_off + (size_t)kOpad * g->H) * 2), "alloc 16-bit weights");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->wb_ema, (g->out_off + (size_t)kOpad * g->H) * 2), "alloc 16-bit ema");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->tab16, g->n_tab * 2), "alloc fp16 tables");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->tab16_ema, g->n_tab * 2), "alloc fp16 ema tables");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->tsteps, g->n_tab * 4), "alloc table step counts");
    if (s == STY_OK) s = check_cuda(cudaMemset(g->tsteps, 0, g->n_tab * 4), "zero table step counts");
    if (s == STY_OK && g->tc) s = check_cuda(cudaMalloc(&g->img, g->img_elems * 2), "alloc weight images");
    if (s == STY_OK && g->tc) s = check_cuda(cudaMalloc(&g->img_ema, g->img_elems * 2), "alloc ema images");
    if (s != STY_OK) {
        grid_destroy(g);
        return s;
    }
    *out = g;
    return STY_OK;
}

void grid_destroy(GridModel *g) {
    if (!g) return;
    void *ptrs[] = {g->wb, g->wb_ema, g->tab16, g->tab16_ema, g->tsteps, g->img, g->img_ema, g->tiles, g->enc,
                    g->acts, g->dp, g->dp2, g->z, g->dh, g->parts, g->d_fan_in, g->d_fan_out, g->d_loff};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete g;
}

sty_status grid_init_params(GridModel *g, uint64_t seed, float *w, cudaStream_t st) {
    std::vector<int> fi, fo;
    for (int l = 0; l <= g->L; l++) {
        fi.push_back(l == 0 ? g->E : g->H);
        fo.push_back(l == g->L ? g->O : g->H);
    }
    if (!g->d_fan_in) {
        STY_TRY(check_cuda(cudaMalloc(&g->d_fan_in, fi.size() * sizeof(int)), "alloc fans"));
        STY_TRY(check_cuda(cudaMalloc(&g->d_fan_out, fo.size() * sizeof(int)), "alloc fans"));
        STY_TRY(check_cuda(cudaMalloc(&g->d_loff, g->loff.size() * sizeof(size_t)), "alloc offsets"));
    }
    STY_TRY(check_cuda(cudaMemcpyAsync(g->d_fan_in, fi.data(), fi.size() * sizeof(int), cudaMemcpyHostToDevice, st),
                       "upload fans"));
    STY_TRY(check_cuda(cudaMemcpyAsync(g->d_fan_out, fo.data(), fo.size() * sizeof(int), cudaMemcpyHostToDevice, st),
                       "upload fans"));
    STY_TRY(check_cuda(cudaMemcpyAsync(g->d_loff, g->loff.data(), g->loff.size() * sizeof(size_t),
                                       cudaMemcpyHostToDevice, st),
                       "upload offsets"));
    const size_t n = g->n_mlp + g->n_tab;
    g->tab16_valid = g->tab16_ema_valid = false;
    k_grid_init<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g->n_mlp, n, g->d_fan_in, g->d_fan_out, g->d_loff,
                                                             g->L + 1, seed, w);
    return check_launch("k_grid_init");
}

sty_status grid_pack(GridModel *g, const float *w, const float *ema, cudaStream_t st) {
    const size_t total = g->out_off + (size_t)kOpad * g->H;
    const unsigned tblocks = (unsigned)((g->n_tab + 255) / 256);
    k_weights16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g->n_mlp, g->out_off, g->O, g->H, w, g->wb, g->f16);
    STY_TRY(check_launch("k_weights16"));
    if (!g->tab16_valid) {
        k_tab_half<<<tblocks, 256, 0, st>>>(g->n_tab, w + g->n_mlp, g->tab16);
        STY_TRY(check_launch("k_tab_half"));
        g->tab16_valid = true;
    }
    if (!ema) return STY_OK;
    // the inference set: EMA copies and the tensor-core weight images of both parameter sets
    k_weights16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g->n_mlp, g->out_off, g->O, g->H, ema, g->wb_ema,
                                                                  g->f16);
    STY_TRY(check_launch("k_weights16"));
    if (!g->tab16_ema_valid) {
        k_tab_half<<<tblocks, 256, 0, st>>>(g->n_tab, ema + g->n_mlp, g->tab16_ema);
        STY_TRY(check_launch("k_tab_half"));
        g->tab16_ema_valid = true;
    }
    if (g->tc) {
        const dim3 grid((unsigned)(((size_t)g->H * std::max(g->E, g->H) + 255) / 256), (unsigned)(g->L + 1));
        k_grid_img<<<grid, 256, 0, st>>>(g->H, g->L, g->E, g->O, w, g->img);
        STY_TRY(check_launch("k_grid_img"));
        k_grid_img<<<grid, 256, 0, st>>>(g->H, g->L, g->E, g->O, ema, g->img_ema);
        STY_TRY(check_launch("k_grid_img"));
    }
    return STY_OK;
}

sty_status grid_infer(GridModel *g, bool ema, bool allow_tc, uint64_t count, const float *in, float *out,
                      cudaStream_t st) {
    if (g->tc && allow_tc) return grid_tc_forward(g, ema, count, in, out, st);
    const uint64_t chunk = 1ull << 18;
    STY_TRY(ensure_cap(g, std::min<uint64_t>(count, chunk)));
    for (uint64_t b0 = 0; b0 < count; b0 += chunk) {
        const uint64_t B = std::min<uint64_t>(chunk, count - b0);
        STY_TRY(grid_forward(g, B, in + b0 * g->geo.in_dims, ema ? g->tab16_ema : g->tab16, ema ? g->wb_ema : g->wb,
                             st));
        k_out_rows<<<(unsigned)((B * g->O + 255) / 256), 256, 0, st>>>(B, g->O, g->z, out + b0 * g->O);
        STY_TRY(check_launch("k_out_rows"));
    }
    return STY_OK;
}

// dW[m][n] (pitch ldd; transposed: dW[n][m]) = scale * P^T Q for P = [B][mp] of any width: the
// tensor-core reduction takes 128 columns of P at a time
sty_status weight_grad(GridModel *g, const uint16_t *P, int mp, const uint16_t *Q, int nq, int B, int n_valid,
                       bool transpose, float scale, float *dst, cudaStream_t st) {
    for (int m0 = 0; m0 < mp; m0 += 128) {
        const int w = std::min(128, mp - m0);
        float *d = transpose ? dst + m0 : dst + (size_t)m0 * nq;
        STY_TRY(tc_gemm_dw(P + m0, mp, w, Q, nq, B, nq, g->f16, g->parts, d, n_valid, transpose, transpose ? mp : nq,
                           scale, st));
    }
    return STY_OK;
}

// loss gradient, backward and the full parameter gradient (MLP weights and tables) of B rows
sty_status grid_gradient(GridModel *g, uint32_t B, const float *x, const float *target, float *grad, float *loss,
                         cudaStream_t st) {
    STY_TRY(ensure_cap(g, B));
    STY_TRY(grid_forward(g, B, x, g->tab16, g->wb, st));
    const float S = g->loss_scale, inv = 1.0f / S;
    const int H = g->H, L = g->L, Bi = (int)B;
    // dP_out = S dLoss/dpred (B x kOpad, 16-bit) in g->dp
    k_rel_l2_grad<<<(B + 255) / 256, 256, 0, st>>>(B, g->O, g->z, target, g->dp, loss, g->f16, S);
    STY_TRY(check_launch("k_rel_l2_grad"));
    const uint16_t *aL = g->acts + (size_t)(L - 1) * B * H;
    // dW_out [O][H] = (A_{L-1}^T dP_out)^T / S
    STY_TRY(weight_grad(g, aL, H, g->dp, kOpad, Bi, g->O, true, inv, grad + g->out_off, st));
    // dP_{L-1} = (dP_out W_out) where A_{L-1} > 0
    STY_TRY(tc_gemm_rows(g->dp, kOpad, g->wb + g->out_off, Bi, kOpad, H, true, g->f16, kEpiMask16, nullptr, g->dp2, aL,
                         1.0f, st));
    uint16_t *dp = g->dp2, *other = g->dp;
    for (int l = L - 1; l >= 0; l--) {
        const uint16_t *al = l == 0 ? g->enc : g->acts + (size_t)(l - 1) * B * H;
        const int K = l == 0 ? g->E : H;
        // dW_l [H][K] = dP_l^T A_{l-1} / S
        STY_TRY(weight_grad(g, dp, H, al, K, Bi, K, false, inv, grad + g->loff[l], st));
        if (l > 0) {  // dP_{l-1} = (dP_l W_l) where A_{l-1} > 0
            STY_TRY(tc_gemm_rows(dp, H, g->wb + g->loff[l], Bi, H, K, true, g->f16, kEpiMask16, nullptr, other, al,
                                 1.0f, st));
            std::swap(dp, other);
        } else {  // dLoss/dencoding = dP_0 W_0 / S (FP32)
            STY_TRY(tc_gemm_rows(dp, H, g->wb + g->loff[0], Bi, H, g->E, true, g->f16, kEpiF32, g->dh, nullptr, nullptr,
                                 inv, st));
        }
    }
    // g->dh now holds dLoss/dencoding (B x E): the tables' gradient
    STY_TRY(check_cuda(cudaMemsetAsync(grad + g->n_mlp, 0, g->n_tab * 4, st), "zero table gradient"));
    const uint64_t nl = (uint64_t)B * g->geo.levels;
    const unsigned blocks = (unsigned)((nl + 255) / 256);
    float *gtab = grad + g->n_mlp;
    switch (g->geo.feats) {
        case 1: k_grid_bwd<1><<<blocks, 256, 0, st>>>(B, x, g->geo, g->dh, gtab); break;
        case 2: k_grid_bwd<2><<<blocks, 256, 0, st>>>(B, x, g->geo, g->dh, gtab); break;
        case 4: k_grid_bwd<4><<<blocks, 256, 0, st>>>(B, x, g->geo, g->dh, gtab); break;
        default: k_grid_bwd<8><<<blocks, 256, 0, st>>>(B, x, g->geo, g->dh, gtab); break;
    }
    return check_launch("k_grid_bwd");
}

void grid_params_changed(GridModel *g) { g->tab16_valid = g->tab16_ema_valid = false; }

sty_status grid_reset_steps(GridModel *g) {
    return check_cuda(cudaMemset(g->tsteps, 0, g->n_tab * 4), "zero table step counts");
}

sty_status grid_adam(GridModel *g, float *w, float *m, float *v, const float *grad, float *ema, float lr, float b1,
                     float b2, float eps, float bc1, float bc2, float ema_decay, float ema_old, float ema_new,
                     cudaStream_t st) {
    const size_t np = g->n_mlp + g->n_tab;  // a multiple of 4: n_mlp of 16, the tables of 8 entries
    const size_t nt = (np + 3) / 4;
    k_adam_grid<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(g->n_mlp, np, w, m, v, grad, ema, g->tsteps, g->tab16,
                                                              g->tab16_ema, lr, b1, b2, eps, bc1, bc2,
                                                              (float)std::log2((double)b1), (float)std::log2((double)b2),
                                                              ema_decay, ema_old, ema_new);
    return check_launch("k_adam_grid");
}

}  // namespace sty
