// nrc.cu -- neural radiance cache: host object, FP32 CUDA-core path, loss, Adam / EMA, sampling.
//
// The object mirrors `struct NRC` of crates/akari_cpp_ext/cpp_ext/akari_tcnn.cu:84-248: it owns the
// weights, the optimiser state and its scratch; the caller owns the input / output / target
// matrices. Unlike the reference, no call synchronises the device unless documented.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fastmod.h"
#include "nrc.cuh"

namespace sty {
namespace {

constexpr int W = kNrcWidth;

// ---- FP32 forward: one thread per sample, all weights in shared memory ----------------------
// acts (optional): [layers+1][count][64] post-activation rows (row 0 = encoded input).
__global__ void __launch_bounds__(128) k_fwd_f32(NrcNet n, const float *__restrict__ wg, uint64_t count,
                                                 const float *__restrict__ input, float *__restrict__ output,
                                                 float *__restrict__ acts) {
    extern __shared__ float ws[];
    const size_t np = nrc_param_count(n);
    for (size_t k = threadIdx.x; k < np; k += blockDim.x) ws[k] = wg[k];
    __syncthreads();
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    float enc[W];
    nrc_encode(n, input + i * n.in_dims, enc);
    float h[W];
#pragma unroll
    for (int k = 0; k < W; k++) h[k] = enc[k];
    if (acts)
#pragma unroll
        for (int k = 0; k < W; k += 4)
            *reinterpret_cast<float4 *>(acts + i * W + k) = make_float4(h[k], h[k + 1], h[k + 2], h[k + 3]);
#pragma unroll 1
    for (int l = 0; l < n.layers; l++) {
        const float *wl = ws + nrc_w_offset(l);
        float z[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < W; k += 4) {
                const float4 w4 = *reinterpret_cast<const float4 *>(wl + j * W + k);
                a = fmaf(w4.x, h[k], a);
                a = fmaf(w4.y, h[k + 1], a);
                a = fmaf(w4.z, h[k + 2], a);
                a = fmaf(w4.w, h[k + 3], a);
            }
            z[j] = a;
        }
#pragma unroll
        for (int j = 0; j < W; j++) h[j] = fmaxf(z[j], 0.0f);
        if (acts) {
            float *dst = acts + ((size_t)(l + 1) * count + i) * W;
#pragma unroll
            for (int k = 0; k < W; k += 4)
                *reinterpret_cast<float4 *>(dst + k) = make_float4(h[k], h[k + 1], h[k + 2], h[k + 3]);
        }
    }
    const float *wo = ws + nrc_w_offset(n.layers);
    for (int c = 0; c < n.out_dims; c++) {
        float a = 0.0f;
#pragma unroll
        for (int k = 0; k < W; k++) a = fmaf(wo[c * W + k], h[k], a);
        output[i * n.out_dims + c] = a;
    }
}

// ---- FP32 forward, register-tiled (the batched and inference path) ---------------------------
// One persistent CTA per SM: every hidden layer's weights transposed into shared memory once
// (wt[l][k][j] = W_l[j][k]), the output layer as stored. Two groups of 256 threads each walk their
// own 128-sample tiles (named barrier per group), each with two activation buffers [64 k][kFP]
// (k-major; a pitch of 132 floats puts consecutive rows 16 bytes apart in bank order). Thread
// (ty, tx) = (t / 16, t % 16) of a group computes samples 8 ty .. 8 ty + 7 x outputs 4 tx .. 4 tx + 3:
// per k two 16-byte activation loads and one 16-byte weight load feed 32 FMAs.
// Every output is summed over k = 0 .. 63 in order with fmaf on the same operands as k_fwd_f32, so
// the two kernels agree bit for bit.
constexpr int kFT = 128;      // samples per tile
constexpr int kFP = kFT + 4;  // activation row pitch (floats)
__host__ __device__ inline size_t fwd_tiled_floats(const NrcNet &n) {
    return (size_t)n.layers * W * W + (size_t)((n.out_dims * W + 3) & ~3) + 4 * (size_t)W * kFP;
}
__global__ void __launch_bounds__(512, 1) k_fwd_f32_tiled(NrcNet n, const float *__restrict__ wg, uint64_t count,
                                                          const float *__restrict__ input,
                                                          float *__restrict__ output, float *__restrict__ acts) {
    extern __shared__ __align__(16) float sm[];
    const int L = n.layers, O = n.out_dims;
    float *wt = sm;
    float *wo = wt + (size_t)L * W * W;
    const int grp = threadIdx.x >> 8, tid = threadIdx.x & 255;
    float *buf0 = wo + ((O * W + 3) & ~3) + (size_t)grp * 2 * W * kFP;
    float *buf1 = buf0 + W * kFP;
    for (int e = threadIdx.x; e < L * W * W; e += 512) {
        const int l = e / (W * W), r = e - l * (W * W), j = r / W, k = r - j * W;
        wt[(size_t)l * W * W + k * W + j] = wg[nrc_w_offset(l) + (size_t)j * W + k];
    }
    for (int e = threadIdx.x; e < O * W; e += 512) wo[e] = wg[nrc_w_offset(L) + e];
    __syncthreads();
    auto group_sync = [&]() { asm volatile("bar.sync %0, 256;" ::"r"(1 + grp) : "memory"); };
    const int ty = tid >> 4, tx = tid & 15;
    const uint64_t ntiles = (count + kFT - 1) / kFT;
    for (uint64_t tile = 2 * (uint64_t)blockIdx.x + grp; tile < ntiles; tile += 2 * (uint64_t)gridDim.x) {
        const uint64_t s0 = tile * kFT;
        if (tid < kFT) {  // encode one sample per thread into buf0[k][sample]
            const uint64_t i = s0 + tid;
            float enc[W];
            if (i < count) {
                nrc_encode(n, input + i * n.in_dims, enc);
            } else {
#pragma unroll
                for (int k = 0; k < W; k++) enc[k] = 0.0f;
            }
#pragma unroll
            for (int k = 0; k < W; k++) buf0[k * kFP + tid] = enc[k];
            if (acts && i < count)
#pragma unroll
                for (int k = 0; k < W; k += 4)
                    *reinterpret_cast<float4 *>(acts + i * W + k) = make_float4(enc[k], enc[k + 1], enc[k + 2], enc[k + 3]);
        }
        group_sync();
        float *cur = buf0, *nxt = buf1;
        for (int l = 0; l < L; l++) {
            const float *w = wt + (size_t)l * W * W + 4 * tx;
            const float *av = cur + 8 * ty;
            float acc[8][4];
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
#pragma unroll 4
            for (int k = 0; k < W; k++) {
                const float4 a0 = *reinterpret_cast<const float4 *>(av + k * kFP);
                const float4 a1 = *reinterpret_cast<const float4 *>(av + k * kFP + 4);
                const float4 w4 = *reinterpret_cast<const float4 *>(w + k * W);
                const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int i = 0; i < 8; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = fmaf(wv[j], a[i], acc[i][j]);
            }
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaxf(acc[i][j], 0.0f);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float *dst = nxt + (4 * tx + j) * kFP + 8 * ty;
                *reinterpret_cast<float4 *>(dst) = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
                *reinterpret_cast<float4 *>(dst + 4) = make_float4(acc[4][j], acc[5][j], acc[6][j], acc[7][j]);
            }
            if (acts) {
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const uint64_t s = s0 + 8 * ty + i;
                    if (s < count)
                        *reinterpret_cast<float4 *>(acts + ((size_t)(l + 1) * count + s) * W + 4 * tx) =
                            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
                }
            }
            group_sync();
            float *t = cur;
            cur = nxt;
            nxt = t;
        }
        if (tid < kFT && s0 + tid < count) {
            for (int c = 0; c < O; c++) {
                float a = 0.0f;
#pragma unroll
                for (int k = 0; k < W; k++) a = fmaf(wo[c * W + k], cur[k * kFP + tid], a);
                output[(s0 + tid) * O + c] = a;
            }
        }
        group_sync();  // the next tile's encoding overwrites buf0
    }
}

// ---- loss gradient + FP32 backward: one thread per sample -----------------------------------
// dpre: [layers+1][B][64]: row l < layers = dL/d(pre-activation of hidden layer l),
// row `layers` = dL/d(output) (first out_dims entries).
__global__ void __launch_bounds__(128) k_bwd_f32(NrcNet n, const float *__restrict__ wg, uint32_t B,
                                                 const float *__restrict__ pred, const float *__restrict__ target,
                                                 const float *__restrict__ acts, float *__restrict__ dpre,
                                                 float *__restrict__ loss_acc) {
    extern __shared__ float ws[];
    __shared__ float red[4];
    const size_t np = nrc_param_count(n);
    for (size_t k = threadIdx.x; k < np; k += blockDim.x) ws[k] = wg[k];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float lsum = 0.0f;
    if (i < B) {
        const float norm = 1.0f / ((float)B * (float)n.out_dims);
        float g[kNrcOutPad];
        for (int c = 0; c < n.out_dims; c++) {
            const float p = pred[(size_t)i * n.out_dims + c], t = target[(size_t)i * n.out_dims + c];
            const float den = p * p + 0.01f;  // relative L2, prediction treated as constant below
            lsum += (p - t) * (p - t) / den;
            g[c] = 2.0f * (p - t) / den * norm;
            dpre[((size_t)n.layers * B + i) * W + c] = g[c];
        }
        // dH = W_out^T g
        float dh[W];
        const float *wo = ws + nrc_w_offset(n.layers);
#pragma unroll
        for (int k = 0; k < W; k++) dh[k] = 0.0f;
        for (int c = 0; c < n.out_dims; c++)
#pragma unroll
            for (int k = 0; k < W; k++) dh[k] = fmaf(wo[c * W + k], g[c], dh[k]);
#pragma unroll 1
        for (int l = n.layers - 1; l >= 0; l--) {
            const float *hl = acts + ((size_t)(l + 1) * B + i) * W;  // post-activation of layer l
            float dp[W];
#pragma unroll
            for (int k = 0; k < W; k += 4) {
                const float4 h4 = *reinterpret_cast<const float4 *>(hl + k);
                dp[k] = h4.x > 0.0f ? dh[k] : 0.0f;
                dp[k + 1] = h4.y > 0.0f ? dh[k + 1] : 0.0f;
                dp[k + 2] = h4.z > 0.0f ? dh[k + 2] : 0.0f;
                dp[k + 3] = h4.w > 0.0f ? dh[k + 3] : 0.0f;
            }
            float *dst = dpre + ((size_t)l * B + i) * W;
#pragma unroll
            for (int k = 0; k < W; k += 4) *reinterpret_cast<float4 *>(dst + k) = make_float4(dp[k], dp[k + 1], dp[k + 2], dp[k + 3]);
            if (l == 0) break;
            const float *wl = ws + nrc_w_offset(l);
#pragma unroll
            for (int k = 0; k < W; k++) dh[k] = 0.0f;
#pragma unroll
            for (int j = 0; j < W; j++) {
                const float dj = dp[j];
#pragma unroll
                for (int k = 0; k < W; k += 4) {
                    const float4 w4 = *reinterpret_cast<const float4 *>(wl + j * W + k);
                    dh[k] = fmaf(w4.x, dj, dh[k]);
                    dh[k + 1] = fmaf(w4.y, dj, dh[k + 1]);
                    dh[k + 2] = fmaf(w4.z, dj, dh[k + 2]);
                    dh[k + 3] = fmaf(w4.w, dj, dh[k + 3]);
                }
            }
        }
    }
    // block-reduce the loss
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
    __syncthreads();
    if (threadIdx.x == 0 && loss_acc) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(loss_acc, t / ((float)B * (float)n.out_dims));
    }
}

// ---- loss gradient + FP32 backward, register-tiled ------------------------------------------
// The same persistent layout as k_fwd_f32_tiled: the weights as stored ([j][k]: for a summed row j
// the outputs k are contiguous), two groups of 256 threads on their own 128-sample tiles, thread
// (ty, tx) holding samples 8 ty .. 8 ty + 7 x units 4 tx .. 4 tx + 3. Per tile: the relative-L2
// gradient g of each sample, dH = W_out^T g, then per hidden layer l (last first) dP_l = dH where
// act_{l+1} > 0 (to dpre and to a k-major buffer) and dH = W_l^T dP_l. Every sum runs over the same
// index in the same order with fmaf on the same operands as k_bwd_f32, so dpre is bit-identical.
__host__ __device__ inline size_t bwd_tiled_floats(const NrcNet &n) {
    return (size_t)n.layers * W * W + (size_t)((n.out_dims * W + 3) & ~3) + 2 * ((size_t)W * kFP + kNrcOutPad * kFT);
}
__global__ void __launch_bounds__(512, 1) k_bwd_f32_tiled(NrcNet n, const float *__restrict__ wg, uint32_t B,
                                                          const float *__restrict__ pred,
                                                          const float *__restrict__ target,
                                                          const float *__restrict__ acts, float *__restrict__ dpre,
                                                          float *__restrict__ loss_acc) {
    extern __shared__ __align__(16) float sm[];
    const int L = n.layers, O = n.out_dims;
    float *ws = sm;                              // [L][64 j][64 k] as stored
    float *wo = ws + (size_t)L * W * W;          // [O][64]
    const int grp = threadIdx.x >> 8, tid = threadIdx.x & 255;
    float *dpb = wo + ((O * W + 3) & ~3) + (size_t)grp * ((size_t)W * kFP + kNrcOutPad * kFT);  // [64 j][kFP]
    float *gb = dpb + W * kFP;                   // [O][128]: the loss gradient, k-major
    for (size_t e = threadIdx.x; e < nrc_param_count(n); e += 512) ws[e] = wg[e];
    __syncthreads();
    auto group_sync = [&]() { asm volatile("bar.sync %0, 256;" ::"r"(1 + grp) : "memory"); };
    const int ty = tid >> 4, tx = tid & 15;
    const float norm = 1.0f / ((float)B * (float)O);
    float lsum = 0.0f;
    const uint32_t ntiles = (B + kFT - 1) / kFT;
    for (uint32_t tile = 2 * blockIdx.x + grp; tile < ntiles; tile += 2 * gridDim.x) {
        const uint32_t s0 = tile * kFT;
        if (tid < kFT) {
            const uint32_t i = s0 + tid;
            for (int c = 0; c < O; c++) {
                float g = 0.0f;
                if (i < B) {
                    const float p = pred[(size_t)i * O + c], t = target[(size_t)i * O + c];
                    const float den = p * p + 0.01f;  // relative L2, prediction treated as constant below
                    lsum += (p - t) * (p - t) / den;
                    g = 2.0f * (p - t) / den * norm;
                    dpre[((size_t)L * B + i) * W + c] = g;
                }
                gb[c * kFT + tid] = g;
            }
        }
        group_sync();
        // dH = W_out^T g
        float acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
        for (int c = 0; c < O; c++) {
            const float4 w4 = *reinterpret_cast<const float4 *>(wo + c * W + 4 * tx);
            const float4 g0 = *reinterpret_cast<const float4 *>(gb + c * kFT + 8 * ty);
            const float4 g1 = *reinterpret_cast<const float4 *>(gb + c * kFT + 8 * ty + 4);
            const float gv[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
            const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(wv[j], gv[i], acc[i][j]);
        }
        for (int l = L - 1; l >= 0; l--) {
            // dP_l = dH where act_{l+1} > 0 -> dpre and dpb[j][sample]
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const uint32_t s = s0 + 8 * ty + i;
                float4 h4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (s < B) h4 = *reinterpret_cast<const float4 *>(acts + ((size_t)(l + 1) * B + s) * W + 4 * tx);
                acc[i][0] = h4.x > 0.0f ? acc[i][0] : 0.0f;
                acc[i][1] = h4.y > 0.0f ? acc[i][1] : 0.0f;
                acc[i][2] = h4.z > 0.0f ? acc[i][2] : 0.0f;
                acc[i][3] = h4.w > 0.0f ? acc[i][3] : 0.0f;
                if (s < B)
                    *reinterpret_cast<float4 *>(dpre + ((size_t)l * B + s) * W + 4 * tx) =
                        make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
            }
            if (l == 0) break;
            group_sync();  // the previous layer's dpb reads are done
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float *dst = dpb + (4 * tx + j) * kFP + 8 * ty;
                *reinterpret_cast<float4 *>(dst) = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
                *reinterpret_cast<float4 *>(dst + 4) = make_float4(acc[4][j], acc[5][j], acc[6][j], acc[7][j]);
            }
            group_sync();
            // dH = W_l^T dP_l: dH[k] = sum_j W_l[j][k] dP_l[j]
            const float *w = ws + nrc_w_offset(l) + 4 * tx;
            const float *dv = dpb + 8 * ty;
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
#pragma unroll 4
            for (int j = 0; j < W; j++) {
                const float4 d0 = *reinterpret_cast<const float4 *>(dv + j * kFP);
                const float4 d1 = *reinterpret_cast<const float4 *>(dv + j * kFP + 4);
                const float4 w4 = *reinterpret_cast<const float4 *>(w + j * W);
                const float dd[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
                const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int i = 0; i < 8; i++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[i][q] = fmaf(wv[q], dd[i], acc[i][q]);
            }
        }
        group_sync();  // the next tile overwrites gb and dpb
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0 && loss_acc && lsum != 0.0f) atomicAdd(loss_acc, lsum / ((float)B * (float)O));
}

// ---- weight gradient: grad_l[j][k] = sum_i dpre_l[i][j] * acts_l[i][k] ----------------------
// grid: (chunks, layers+1); 256 threads; rows R = 64 (hidden) or out_dims (output layer). Each
// chunk of kWgChunk samples stores its partial sums at part + chunk * np; k_sum_chunks adds the
// chunks in order, so the gradient does not depend on scheduling.
constexpr int kWgChunk = 1024;
// Register-tiled: thread (ty, tx) = (t / 16, t % 16) owns outputs j = 4 ty .. 4 ty + 3 x
// k = 4 tx .. 4 tx + 3, so per sample two 16-byte shared-memory loads feed 16 FMAs; the next
// 64-sample tile's rows are loaded into registers while the current one is summed. Every output
// is summed over the chunk's samples in order with fmaf(dpre, act, acc) (padding samples add
// fmaf(0, 0, acc)), as the one-output-row-per-thread version did, so the partials are unchanged.
__global__ void __launch_bounds__(256) k_wgrad_f32(NrcNet n, uint32_t B, const float *__restrict__ acts,
                                                   const float *__restrict__ dpre, size_t np,
                                                   float *__restrict__ part) {
    __shared__ __align__(16) float sd[64][W];  // dpre rows of 64 samples
    __shared__ __align__(16) float sh[64][W];  // activation rows (the input of weight matrix l)
    const int l = blockIdx.y;
    const int rows = l < n.layers ? W : n.out_dims;
    const uint32_t i0 = blockIdx.x * kWgChunk, i1 = min(B, i0 + kWgChunk);
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    const float4 *dl = reinterpret_cast<const float4 *>(dpre + (size_t)l * B * W);
    const float4 *al = reinterpret_cast<const float4 *>(acts + (size_t)l * B * W);
    constexpr int kPer = 64 * W / 4 / 256;  // float4 of each array per thread per tile
    float4 pd[kPer], pa[kPer];
    auto fetch = [&](uint32_t s0) {
#pragma unroll
        for (int u = 0; u < kPer; u++) {
            const int e = threadIdx.x + u * 256, r = e / (W / 4), c4 = e % (W / 4);
            const uint32_t s = s0 + (uint32_t)r;
            const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            pd[u] = s < i1 ? dl[(size_t)s * (W / 4) + c4] : z;
            pa[u] = s < i1 ? al[(size_t)s * (W / 4) + c4] : z;
        }
    };
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[i][c] = 0.0f;
    fetch(i0);
    for (uint32_t s0 = i0; s0 < i1; s0 += 64) {
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kPer; u++) {
            const int e = threadIdx.x + u * 256, r = e / (W / 4), c4 = e % (W / 4);
            reinterpret_cast<float4 *>(&sd[r][0])[c4] = pd[u];
            reinterpret_cast<float4 *>(&sh[r][0])[c4] = pa[u];
        }
        __syncthreads();
        if (s0 + 64 < i1) fetch(s0 + 64);
        if (4 * ty < rows) {
#pragma unroll 4
            for (int r = 0; r < 64; r++) {
                const float4 a4 = *reinterpret_cast<const float4 *>(&sd[r][4 * ty]);
                const float4 b4 = *reinterpret_cast<const float4 *>(&sh[r][4 * tx]);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[i][c] = fmaf(av[i], bv[c], acc[i][c]);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int j = 4 * ty + i;
        if (j < rows)
            *reinterpret_cast<float4 *>(part + blockIdx.x * np + nrc_w_offset(l) + (size_t)j * W + 4 * tx) =
                make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    }
}

// grad[p] = part[0][p] + part[1][p] + ... in chunk order (one sequential FP32 sum per parameter;
// np is a multiple of 64: layers x 64 x 64 + outputs x 64). A block owns kSumP parameters: its 256
// threads stage a slab of up to kSumC chunk rows into shared memory with 16-byte loads, every load of
// the slab issued before the first store (16 in flight per thread), then kSumP threads continue their
// sums over the slab in order. The 152 per-CTA partials of a tensor-core training step are one slab.
constexpr int kSumP = 64, kSumC = 256, kSumLd = kSumC / (256 / (kSumP / 4));
__global__ void __launch_bounds__(256) k_sum_chunks(size_t np, uint32_t chunks, uint32_t slab_rows,
                                                    const float *__restrict__ part, float *__restrict__ grad) {
    extern __shared__ float4 slab4[];  // [slab_rows][kSumP / 4]
    const float *slab = reinterpret_cast<const float *>(slab4);
    const int t = threadIdx.x, c4 = t % (kSumP / 4), r0 = t / (kSumP / 4);
    const size_t p0 = (size_t)blockIdx.x * kSumP;
    const float4 *src = reinterpret_cast<const float4 *>(part + p0) + c4;
    const size_t row4 = np / 4;
    float s = 0.0f;
    for (uint32_t c0 = 0; c0 < chunks; c0 += slab_rows) {
        const uint32_t nc = min(slab_rows, chunks - c0);
        float4 v[kSumLd];
#pragma unroll
        for (int j = 0; j < kSumLd; j++) {
            const uint32_t r = (uint32_t)r0 + (uint32_t)j * (256 / (kSumP / 4));
            if (r < nc) v[j] = src[(size_t)(c0 + r) * row4];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kSumLd; j++) {
            const uint32_t r = (uint32_t)r0 + (uint32_t)j * (256 / (kSumP / 4));
            if (r < nc) slab4[r * (kSumP / 4) + c4] = v[j];
        }
        __syncthreads();
        if (t < kSumP)
            for (uint32_t r = 0; r < nc; r++) s += slab[r * kSumP + t];
    }
    if (t < kSumP && p0 + (size_t)t < np) grad[p0 + t] = s;
}
void sum_chunks(size_t np, uint32_t chunks, const float *part, float *grad, cudaStream_t st) {
    const uint32_t rows = chunks < (uint32_t)kSumC ? (chunks > 0 ? chunks : 1u) : (uint32_t)kSumC;
    const size_t smem = rows * kSumP * sizeof(float);
    if (smem > 48 * 1024)  // beyond the default dynamic shared-memory limit (a check_launch follows)
        cudaFuncSetAttribute(k_sum_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSumC * kSumP * 4));
    k_sum_chunks<<<(unsigned)((np + kSumP - 1) / kSumP), 256, smem, st>>>(np, chunks, rows, part, grad);
}

// ---- batch sampling (collect_batch, akari_tcnn.cu:15-38) -------------------------------------
__device__ __forceinline__ uint32_t pcg_step(uint64_t &state, uint64_t inc) {
    const uint64_t old = state;
    state = old * 0x5851f42d4c957f2dULL + inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}
// count_magic = fastmod_magic(count): the row index r % count without a 64-bit division
__global__ void k_collect(uint32_t B, uint64_t seed, uint64_t step, uint64_t count, uint64_t count_magic, int in_dims,
                          int out_dims, const float *__restrict__ in, const float *__restrict__ tg,
                          float *__restrict__ bin, float *__restrict__ btg) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    uint64_t st = 0, inc = ((step * (uint64_t)B + b) << 1) | 1ull;
    pcg_step(st, inc);
    st += seed;
    pcg_step(st, inc);
    const uint64_t r = ((uint64_t)pcg_step(st, inc) << 32) | pcg_step(st, inc);
    const uint64_t idx = fastmod(r, count, count_magic);
    // the row's loads in batches of 8 before their stores, so the random-row latency is paid once
    // per batch, not once per value
    const float *src = in + idx * in_dims;
    float *dst = bin + (size_t)b * in_dims;
    for (int d0 = 0; d0 < in_dims; d0 += 8) {
        float v[8];
#pragma unroll
        for (int d = 0; d < 8; d++) v[d] = d0 + d < in_dims ? src[d0 + d] : 0.0f;
#pragma unroll
        for (int d = 0; d < 8; d++)
            if (d0 + d < in_dims) dst[d0 + d] = v[d];
    }
    float u[kNrcOutPad];
#pragma unroll
    for (int c = 0; c < kNrcOutPad; c++) u[c] = c < out_dims ? tg[idx * out_dims + c] : 0.0f;
#pragma unroll
    for (int c = 0; c < kNrcOutPad; c++)
        if (c < out_dims) btg[(size_t)b * out_dims + c] = u[c];
}

// ---- Adam + EMA (akari_tcnn.cu:42-83 for the EMA) --------------------------------------------
__global__ void k_adam(size_t np, float *w, float *m, float *v, const float *g, float *ema, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, float ema_decay, float ema_old, float ema_new) {
    const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float gr = g[p];
    const float mm = b1 * m[p] + (1.0f - b1) * gr;
    const float vv = b2 * v[p] + (1.0f - b2) * gr * gr;
    m[p] = mm;
    v[p] = vv;
    const float wn = w[p] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    w[p] = wn;
    ema[p] = (ema[p] * ema_decay * ema_old + wn * (1.0f - ema_decay)) * ema_new;
}

__global__ void k_init_weights(size_t np, NrcNet n, uint64_t seed, float *w) {
    const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    uint64_t st = 0, inc = ((uint64_t)p << 1) | 1ull;
    pcg_step(st, inc);
    st += seed;
    pcg_step(st, inc);
    const float u = (float)pcg_step(st, inc) * (1.0f / 4294967296.0f);
    const size_t hid = (size_t)n.layers * W * W;
    const float fan_out = p < hid ? (float)W : (float)n.out_dims;
    const float s = sqrtf(6.0f / ((float)W + fan_out));  // uniform Xavier
    w[p] = (2.0f * u - 1.0f) * s;
}

}  // namespace
}  // namespace sty

using namespace sty;

struct sty_nrc {
    sty_nrc_config cfg;
    NrcNet net;
    size_t np = 0;
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *ema = nullptr;
    uint16_t *img = nullptr, *img_ema = nullptr;  // BF16 tensor-core images of w / ema
    float *bin = nullptr, *btg = nullptr, *bpred = nullptr, *acts = nullptr, *dpre = nullptr, *loss = nullptr;
    float *gpart = nullptr;  // per-chunk weight-gradient partials
    GridModel *grid = nullptr;  // the composite-encoding network (sty_nrc_create_grid), else null
    bool layered = false;       // grid network: STY_NRC_GRID_LAYERED (no tensor-core inference)
    uint32_t bcap = 0;
    uint64_t step = 0;  // optimiser steps taken (Adam t, EMA iteration)
    float lr = 0.0f;
    bool img_dirty = true;
};

namespace sty {
uint32_t nrc_batch_size(const sty_nrc *nr) { return nr->cfg.batch_size; }
uint32_t nrc_input_dims(const sty_nrc *nr) { return nr->cfg.input_dims; }
}  // namespace sty

namespace {

sty_status ensure_batch(sty_nrc *nr, uint32_t B) {
    if (B <= nr->bcap) return STY_OK;
    void *ptrs[] = {nr->bin, nr->btg, nr->bpred, nr->acts, nr->dpre, nr->gpart};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    nr->bin = nr->btg = nr->bpred = nr->acts = nr->dpre = nr->gpart = nullptr;
    const NrcNet &n = nr->net;
    STY_TRY(check_cuda(cudaMalloc(&nr->bin, (size_t)B * n.in_dims * 4), "alloc batch input"));
    STY_TRY(check_cuda(cudaMalloc(&nr->btg, (size_t)B * n.out_dims * 4), "alloc batch target"));
    STY_TRY(check_cuda(cudaMalloc(&nr->bpred, (size_t)B * n.out_dims * 4), "alloc batch pred"));
    STY_TRY(check_cuda(cudaMalloc(&nr->acts, (size_t)(n.layers + 1) * B * kNrcWidth * 4), "alloc activations"));
    STY_TRY(check_cuda(cudaMalloc(&nr->dpre, (size_t)(n.layers + 1) * B * kNrcWidth * 4), "alloc gradients"));
    if (!nr->grid) {  // the composite-encoding network computes its gradient without partials
        size_t chunks = (B + kWgChunk - 1) / kWgChunk;
        if (nr->cfg.precision == STY_NRC_BF16) chunks = std::max<size_t>(chunks, nrc_tc_train_ctas(B));
        STY_TRY(check_cuda(cudaMalloc(&nr->gpart, chunks * nr->np * 4), "alloc gradient partials"));
    }
    nr->bcap = B;
    return STY_OK;
}

size_t fwd_smem(const sty_nrc *nr) { return nr->np * sizeof(float); }

sty_status fwd_f32(sty_nrc *nr, const float *wts, uint64_t count, const float *in, float *out, float *acts,
                   cudaStream_t st) {
    if (count == 0) return STY_OK;
    int dev = 0, optin = 0, sms = 0;
    STY_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    STY_TRY(check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attr smem"));
    STY_TRY(check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr SMs"));
    const size_t tsmem = fwd_tiled_floats(nr->net) * sizeof(float);
    if (tsmem <= (size_t)optin) {  // register-tiled kernel (bit-identical to k_fwd_f32)
        STY_TRY(check_cuda(cudaFuncSetAttribute(k_fwd_f32_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem),
                           "attr k_fwd_f32_tiled"));
        const uint64_t ntiles = (count + kFT - 1) / kFT;
        const unsigned grid = (unsigned)std::min<uint64_t>((ntiles + 1) / 2, (uint64_t)sms);
        k_fwd_f32_tiled<<<grid, 512, tsmem, st>>>(nr->net, wts, count, in, out, acts);
        return check_launch("k_fwd_f32_tiled");
    }
    const size_t smem = fwd_smem(nr);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_fwd_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "attr k_fwd_f32"));
    k_fwd_f32<<<(unsigned)((count + 127) / 128), 128, smem, st>>>(nr->net, wts, count, in, out, acts);
    return check_launch("k_fwd_f32");
}

// Loss gradient, backward and weight gradient for the batch already forwarded into nr->bpred /
// nr->acts (FP32 CUDA-core path, also used for the BF16 path's weight update).
sty_status backward(sty_nrc *nr, uint32_t B, const float *target, cudaStream_t st) {
    const NrcNet &n = nr->net;
    int dev = 0, optin = 0, sms = 0;
    STY_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    STY_TRY(check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attr smem"));
    STY_TRY(check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr SMs"));
    const size_t tsmem = bwd_tiled_floats(n) * sizeof(float);
    if (B > 0 && n.out_dims <= kNrcOutPad && tsmem <= (size_t)optin) {  // register-tiled (bit-identical dpre)
        STY_TRY(check_cuda(cudaFuncSetAttribute(k_bwd_f32_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem),
                           "attr k_bwd_f32_tiled"));
        const uint32_t ntiles = (B + kFT - 1) / kFT;
        const unsigned grid = std::min<uint32_t>((ntiles + 1) / 2, (uint32_t)sms);
        k_bwd_f32_tiled<<<grid, 512, tsmem, st>>>(n, nr->w, B, nr->bpred, target, nr->acts, nr->dpre, nr->loss);
        STY_TRY(check_launch("k_bwd_f32_tiled"));
    } else {
        const size_t smem = fwd_smem(nr);
        STY_TRY(check_cuda(cudaFuncSetAttribute(k_bwd_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "attr k_bwd_f32"));
        k_bwd_f32<<<(B + 127) / 128, 128, smem, st>>>(n, nr->w, B, nr->bpred, target, nr->acts, nr->dpre, nr->loss);
        STY_TRY(check_launch("k_bwd_f32"));
    }
    const uint32_t chunks = (B + kWgChunk - 1) / kWgChunk;
    dim3 grid(chunks, n.layers + 1);
    k_wgrad_f32<<<grid, 256, 0, st>>>(n, B, nr->acts, nr->dpre, nr->np, nr->gpart);
    STY_TRY(check_launch("k_wgrad_f32"));
    sum_chunks(nr->np, chunks, nr->gpart, nr->g, st);
    return check_launch("k_sum_chunks");
}

sty_status forward_batch(sty_nrc *nr, uint32_t B, const float *in, cudaStream_t st) {
    // training forward (stores the activations the backward pass reads)
    return fwd_f32(nr, nr->w, B, in, nr->bpred, nr->acts, st);
}

bool tc_training(const sty_nrc *nr) {
    return !nr->grid && nr->cfg.precision == STY_NRC_BF16 && nr->net.layers <= kNrcTcTrainMaxLayers;
}

// Weight gradient of one batch into nr->g (loss added to nr->loss): the fused BF16 tensor-core
// step for BF16 caches, else the FP32 forward / backward / weight-gradient kernels.
sty_status batch_gradient(sty_nrc *nr, uint32_t B, const float *in, const float *target, cudaStream_t st) {
    if (nr->grid) {
        STY_TRY(grid_pack(nr->grid, nr->w, nullptr, st));
        nr->img_dirty = true;
        return grid_gradient(nr->grid, B, in, target, nr->g, nr->loss, st);
    }
    if (!tc_training(nr)) {
        STY_TRY(forward_batch(nr, B, in, st));
        return backward(nr, B, target, st);
    }
    STY_TRY(nrc_tc_pack(nr->net, nr->w, nr->img, st));
    nr->img_dirty = true;  // nr->img now holds w, which the optimiser step is about to change
    const uint32_t ctas = nrc_tc_train_ctas(B);
    STY_TRY(nrc_tc_train(nr->net, nr->img, B, in, target, nr->gpart, nr->np, nr->loss, ctas, st));
    sum_chunks(nr->np, ctas, nr->gpart, nr->g, st);
    return check_launch("k_sum_chunks");
}

sty_status refresh_images(sty_nrc *nr, cudaStream_t st) {
    if (nr->grid) {
        if (nr->img_dirty) STY_TRY(grid_pack(nr->grid, nr->w, nr->ema, st));
        nr->img_dirty = false;
        return STY_OK;
    }
    if (nr->cfg.precision != STY_NRC_BF16 || !nr->img_dirty) return STY_OK;
    STY_TRY(nrc_tc_pack(nr->net, nr->w, nr->img, st));
    STY_TRY(nrc_tc_pack(nr->net, nr->ema, nr->img_ema, st));
    nr->img_dirty = false;
    return STY_OK;
}

sty_status infer(sty_nrc *nr, bool ema, uint64_t count, const float *in, float *out, cudaStream_t st) {
    if (count == 0) return STY_OK;
    if (nr->grid) {
        STY_TRY(refresh_images(nr, st));
        return grid_infer(nr->grid, ema, !nr->layered, count, in, out, st);
    }
    if (nr->cfg.precision == STY_NRC_BF16) {
        STY_TRY(refresh_images(nr, st));
        return nrc_tc_forward(nr->net, ema ? nr->img_ema : nr->img, count, in, out, st);
    }
    return fwd_f32(nr, ema ? nr->ema : nr->w, count, in, out, nullptr, st);
}

void free_nrc(sty_nrc *nr) {
    grid_destroy(nr->grid);
    void *ptrs[] = {nr->w, nr->m, nr->v, nr->g, nr->ema, nr->img, nr->img_ema, nr->bin,
                    nr->btg, nr->bpred, nr->acts, nr->dpre, nr->loss, nr->gpart};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete nr;
}

}  // namespace

extern "C" {

sty_status sty_nrc_create(const sty_nrc_config *cfg, sty_nrc **out) {
    clear_error();
    STY_ARG_CHECK(cfg && out, "sty_nrc_create: null argument");
    STY_ARG_CHECK(cfg->input_dims >= 1 && cfg->input_dims <= STY_NRC_MAX_INPUTS, "input_dims must be in [1, 16]");
    STY_ARG_CHECK(cfg->output_dims >= 1 && cfg->output_dims <= (uint32_t)kNrcOutPad, "output_dims must be in [1, 16]");
    STY_ARG_CHECK(cfg->hidden_layers >= 1 && cfg->hidden_layers <= (uint32_t)kNrcMaxLayers,
                  "hidden_layers must be in [1, 8]");
    STY_ARG_CHECK(cfg->batch_size >= 128 && cfg->batch_size % 128 == 0, "batch_size must be a multiple of 128");
    STY_ARG_CHECK(cfg->precision == STY_NRC_FP32 || cfg->precision == STY_NRC_BF16, "unknown precision");
    uint32_t enc = 0;
    for (uint32_t d = 0; d < cfg->input_dims; d++) enc += 2 * cfg->freqs[d];
    STY_ARG_CHECK(enc <= (uint32_t)kNrcWidth, "encoded width %u exceeds 64", enc);
    STY_ARG_CHECK(cfg->decay_interval > 0 && cfg->learning_rate > 0.0f, "decay_interval and learning_rate must be > 0");
    sty_nrc *nr = new sty_nrc();
    nr->cfg = *cfg;
    nr->net.in_dims = (int)cfg->input_dims;
    nr->net.out_dims = (int)cfg->output_dims;
    nr->net.layers = (int)cfg->hidden_layers;
    for (int d = 0; d < STY_NRC_MAX_INPUTS; d++) nr->net.freqs[d] = cfg->freqs[d];
    nr->np = nrc_param_count(nr->net);
    nr->lr = cfg->learning_rate;
    sty_status s = STY_OK;
    auto alloc = [&](void **p, size_t bytes, const char *what) {
        if (s == STY_OK) s = check_cuda(cudaMalloc(p, bytes), what);
    };
    alloc((void **)&nr->w, nr->np * 4, "alloc weights");
    alloc((void **)&nr->m, nr->np * 4, "alloc adam m");
    alloc((void **)&nr->v, nr->np * 4, "alloc adam v");
    alloc((void **)&nr->g, nr->np * 4, "alloc grad");
    alloc((void **)&nr->ema, nr->np * 4, "alloc ema");
    alloc((void **)&nr->loss, 4, "alloc loss");
    if (cfg->precision == STY_NRC_BF16) {
        alloc((void **)&nr->img, nrc_tc_image_elems(nr->net) * 2, "alloc bf16 image");
        alloc((void **)&nr->img_ema, nrc_tc_image_elems(nr->net) * 2, "alloc bf16 ema image");
    }
    if (s == STY_OK) s = ensure_batch(nr, cfg->batch_size);
    if (s == STY_OK) {
        k_init_weights<<<(unsigned)((nr->np + 255) / 256), 256>>>(nr->np, nr->net, cfg->seed, nr->w);
        s = check_launch("k_init_weights");
    }
    if (s == STY_OK) s = check_cuda(cudaMemcpy(nr->ema, nr->w, nr->np * 4, cudaMemcpyDeviceToDevice), "init ema");
    if (s == STY_OK) s = check_cuda(cudaMemset(nr->m, 0, nr->np * 4), "zero m");
    if (s == STY_OK) s = check_cuda(cudaMemset(nr->v, 0, nr->np * 4), "zero v");
    if (s == STY_OK) s = check_cuda(cudaDeviceSynchronize(), "sty_nrc_create");
    if (s != STY_OK) {
        free_nrc(nr);
        return s;
    }
    *out = nr;
    return STY_OK;
}

sty_status sty_nrc_create_grid(const sty_nrc_grid_config *gc, sty_nrc **out) {
    clear_error();
    STY_ARG_CHECK(gc && out, "sty_nrc_create_grid: null argument");
    STY_ARG_CHECK(gc->batch_size >= 128 && gc->batch_size % 128 == 0, "batch_size must be a multiple of 128");
    STY_ARG_CHECK(gc->decay_interval > 0 && gc->learning_rate > 0.0f, "decay_interval and learning_rate must be > 0");
    STY_ARG_CHECK((gc->flags & ~(STY_NRC_GRID_LAYERED | STY_NRC_GRID_FP16)) == 0, "unknown flags 0x%x", gc->flags);
    sty_nrc *nr = new sty_nrc();
    nr->layered = (gc->flags & STY_NRC_GRID_LAYERED) != 0;
    size_t np = 0, n_mlp = 0;
    sty_status s = grid_create(gc, &nr->grid, &np, &n_mlp);
    if (s != STY_OK) {
        delete nr;
        return s;
    }
    // the fields the shared training loop reads (batch sampling, Adam, decay, EMA)
    sty_nrc_config &c = nr->cfg;
    std::memset(&c, 0, sizeof(c));
    c.input_dims = gc->input_dims;
    c.output_dims = gc->output_dims;
    c.batch_size = gc->batch_size;
    c.hidden_layers = gc->hidden_layers;
    c.precision = STY_NRC_BF16;
    c.learning_rate = gc->learning_rate;
    c.beta1 = gc->beta1;
    c.beta2 = gc->beta2;
    c.epsilon = gc->epsilon;
    c.ema_decay = gc->ema_decay;
    c.decay_base = gc->decay_base;
    c.decay_interval = gc->decay_interval;
    c.seed = gc->seed;
    nr->net.in_dims = (int)gc->input_dims;
    nr->net.out_dims = (int)gc->output_dims;
    nr->net.layers = 1;
    nr->np = np;
    nr->lr = gc->learning_rate;
    auto alloc = [&](void **p, size_t bytes, const char *what) {
        if (s == STY_OK) s = check_cuda(cudaMalloc(p, bytes), what);
    };
    alloc((void **)&nr->w, np * 4, "alloc parameters");
    alloc((void **)&nr->m, np * 4, "alloc adam m");
    alloc((void **)&nr->v, np * 4, "alloc adam v");
    alloc((void **)&nr->g, np * 4, "alloc grad");
    alloc((void **)&nr->ema, np * 4, "alloc ema");
    alloc((void **)&nr->loss, 4, "alloc loss");
    if (s == STY_OK) s = ensure_batch(nr, gc->batch_size);
    if (s == STY_OK) s = grid_init_params(nr->grid, gc->seed, nr->w, nullptr);
    if (s == STY_OK) s = check_cuda(cudaMemcpy(nr->ema, nr->w, np * 4, cudaMemcpyDeviceToDevice), "init ema");
    if (s == STY_OK) s = check_cuda(cudaMemset(nr->m, 0, np * 4), "zero m");
    if (s == STY_OK) s = check_cuda(cudaMemset(nr->v, 0, np * 4), "zero v");
    if (s == STY_OK) s = check_cuda(cudaDeviceSynchronize(), "sty_nrc_create_grid");
    if (s != STY_OK) {
        free_nrc(nr);
        return s;
    }
    *out = nr;
    return STY_OK;
}

sty_status sty_nrc_destroy(sty_nrc *nr) {
    clear_error();
    if (!nr) return STY_OK;
    cudaDeviceSynchronize();
    free_nrc(nr);
    return STY_OK;
}

sty_status sty_nrc_param_count(sty_nrc *nr, uint64_t *count) {
    clear_error();
    STY_ARG_CHECK(nr && count, "sty_nrc_param_count: null argument");
    *count = nr->np;
    return STY_OK;
}

sty_status sty_nrc_save_params(sty_nrc *nr, float *host) {
    clear_error();
    STY_ARG_CHECK(nr && host, "sty_nrc_save_params: null argument");
    STY_TRY(check_cuda(cudaDeviceSynchronize(), "sync before save"));
    return check_cuda(cudaMemcpy(host, nr->w, nr->np * 4, cudaMemcpyDeviceToHost), "save params");
}

sty_status sty_nrc_load_params(sty_nrc *nr, const float *host) {
    clear_error();
    STY_ARG_CHECK(nr && host, "sty_nrc_load_params: null argument");
    STY_TRY(check_cuda(cudaDeviceSynchronize(), "sync before load"));
    STY_TRY(check_cuda(cudaMemcpy(nr->w, host, nr->np * 4, cudaMemcpyHostToDevice), "load params"));
    STY_TRY(check_cuda(cudaMemcpy(nr->ema, host, nr->np * 4, cudaMemcpyHostToDevice), "load ema"));
    nr->img_dirty = true;
    if (nr->grid) grid_params_changed(nr->grid);
    return STY_OK;
}

sty_status sty_nrc_set_learning_rate(sty_nrc *nr, float lr) {
    clear_error();
    STY_ARG_CHECK(nr && lr > 0.0f, "sty_nrc_set_learning_rate: bad argument");
    nr->lr = lr;
    return STY_OK;
}

sty_status sty_nrc_get_learning_rate(sty_nrc *nr, float *lr) {
    clear_error();
    STY_ARG_CHECK(nr && lr, "sty_nrc_get_learning_rate: null argument");
    *lr = nr->lr;
    return STY_OK;
}

sty_status sty_nrc_reset_optimizer(sty_nrc *nr) {
    clear_error();
    STY_ARG_CHECK(nr, "sty_nrc_reset_optimizer: null nrc");
    STY_TRY(check_cuda(cudaMemset(nr->m, 0, nr->np * 4), "zero m"));
    STY_TRY(check_cuda(cudaMemset(nr->v, 0, nr->np * 4), "zero v"));
    if (nr->grid) STY_TRY(grid_reset_steps(nr->grid));
    nr->step = 0;
    return STY_OK;
}

sty_status sty_nrc_inference(sty_nrc *nr, uint64_t count, const float *in, float *out, void *stream) {
    clear_error();
    STY_ARG_CHECK(nr && (count == 0 || (in && out)), "sty_nrc_inference: null argument");
    return infer(nr, true, count, in, out, as_stream(stream));
}

sty_status sty_nrc_train_inference(sty_nrc *nr, uint64_t count, const float *in, float *out, void *stream) {
    clear_error();
    STY_ARG_CHECK(nr && (count == 0 || (in && out)), "sty_nrc_train_inference: null argument");
    return infer(nr, false, count, in, out, as_stream(stream));
}

sty_status sty_nrc_gradient(sty_nrc *nr, uint32_t B, const float *in, const float *target, float *grad,
                            float *loss_out, void *stream) {
    clear_error();
    STY_ARG_CHECK(nr && in && target && grad && B > 0, "sty_nrc_gradient: bad argument");
    cudaStream_t st = as_stream(stream);
    STY_TRY(ensure_batch(nr, B));
    STY_TRY(check_cuda(cudaMemsetAsync(nr->loss, 0, 4, st), "zero loss"));
    STY_TRY(batch_gradient(nr, B, in, target, st));
    STY_TRY(check_cuda(cudaMemcpyAsync(grad, nr->g, nr->np * 4, cudaMemcpyDeviceToDevice, st), "copy grad"));
    if (loss_out) {
        STY_TRY(check_cuda(cudaMemcpyAsync(loss_out, nr->loss, 4, cudaMemcpyDeviceToHost, st), "read loss"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync loss"));
    }
    return STY_OK;
}

sty_status sty_nrc_train(sty_nrc *nr, uint64_t count, uint64_t n_iters, const float *in, const float *target,
                         float *loss_out, void *stream) {
    clear_error();
    STY_ARG_CHECK(nr && in && target && count > 0, "sty_nrc_train: bad argument");
    cudaStream_t st = as_stream(stream);
    const sty_nrc_config &c = nr->cfg;
    const uint32_t B = c.batch_size;
    STY_TRY(check_cuda(cudaMemsetAsync(nr->loss, 0, 4, st), "zero loss"));
    for (uint64_t it = 0; it < n_iters; it++) {
        k_collect<<<(B + 255) / 256, 256, 0, st>>>(B, c.seed, nr->step, count, fastmod_magic(count), nr->net.in_dims,
                                                   nr->net.out_dims, in, target, nr->bin, nr->btg);
        STY_TRY(check_launch("k_collect"));
        STY_TRY(batch_gradient(nr, B, nr->bin, nr->btg, st));
        nr->step++;
        const double t = (double)nr->step;
        const float lr_t = nr->lr * (float)std::pow((double)c.decay_base, std::floor((t - 1.0) / c.decay_interval));
        const float bc1 = (float)(1.0 - std::pow((double)c.beta1, t));
        const float bc2 = (float)(1.0 - std::pow((double)c.beta2, t));
        const float ema_old = (float)(1.0 - std::pow((double)c.ema_decay, t - 1.0));
        const float ema_new = (float)(1.0 / (1.0 - std::pow((double)c.ema_decay, t)));
        if (nr->grid) {
            STY_TRY(grid_adam(nr->grid, nr->w, nr->m, nr->v, nr->g, nr->ema, lr_t, c.beta1, c.beta2, c.epsilon, bc1,
                              bc2, c.ema_decay, ema_old, ema_new, st));
        } else {
            k_adam<<<(unsigned)((nr->np + 255) / 256), 256, 0, st>>>(nr->np, nr->w, nr->m, nr->v, nr->g, nr->ema,
                                                                     lr_t, c.beta1, c.beta2, c.epsilon, bc1, bc2,
                                                                     c.ema_decay, ema_old, ema_new);
            STY_TRY(check_launch("k_adam"));
        }
        nr->img_dirty = true;
    }
    if (loss_out) {
        float l = 0.0f;
        STY_TRY(check_cuda(cudaMemcpyAsync(&l, nr->loss, 4, cudaMemcpyDeviceToHost, st), "read loss"));
        STY_TRY(check_cuda(cudaStreamSynchronize(st), "sync loss"));
        *loss_out = n_iters ? l / (float)n_iters : 0.0f;
    }
    return STY_OK;
}

}  // extern "C"
