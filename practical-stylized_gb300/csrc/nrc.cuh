// nrc.cuh -- neural radiance cache: shared definitions of the FP32 and BF16 (tcgen05) paths.
#pragma once

#include "common.cuh"

namespace sty {

constexpr int kNrcWidth = 64;      // hidden width and encoded input width
constexpr int kNrcMaxLayers = 8;   // hidden layers supported
constexpr int kNrcOutPad = 16;     // output rows padded to one MMA N tile

struct NrcNet {
    int in_dims, out_dims, layers;     // layers = hidden layers; weight matrices = layers + 1
    uint32_t freqs[STY_NRC_MAX_INPUTS];
};

// offsets (floats) of the weight matrices in the flat FP32 parameter vector:
// layer l < layers: [64 out][64 in]; output layer: [out_dims][64]
__host__ __device__ inline size_t nrc_w_offset(int l) { return (size_t)l * kNrcWidth * kNrcWidth; }
__host__ __device__ inline size_t nrc_param_count(const NrcNet &n) {
    return (size_t)n.layers * kNrcWidth * kNrcWidth + (size_t)n.out_dims * kNrcWidth;
}

// Frequency encoding of one sample: dim d contributes sin(2^k pi x), cos(2^k pi x), k < freqs[d],
// in order (d, k, sin, cos); the tail up to 64 is zero. One sincosf per dim, higher octaves by the
// double-angle identities sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a.
__device__ __forceinline__ void nrc_encode(const NrcNet &n, const float *x, float enc[kNrcWidth]) {
    int o = 0;
#pragma unroll 1
    for (int d = 0; d < n.in_dims; d++) {
        float s, c;
        sincospif(x[d], &s, &c);
        for (uint32_t k = 0; k < n.freqs[d]; k++) {
            enc[o] = s;
            enc[o + 1] = c;
            o += 2;
            const float s2 = 2.0f * s * c;
            c = fmaf(-2.0f * s, s, 1.0f);
            s = s2;
        }
    }
    for (; o < kNrcWidth; o++) enc[o] = 0.0f;
}

// BF16 tensor-core path (nrc_tc.cu)
struct NrcTcWeights;  // device buffers in the UMMA shared-memory image layout
sty_status nrc_tc_pack(const NrcNet &n, const float *w_fp32, uint16_t *w_img, cudaStream_t st);
size_t nrc_tc_image_elems(const NrcNet &n);
sty_status nrc_tc_forward(const NrcNet &n, const uint16_t *w_img, uint64_t count, const float *input, float *output,
                          cudaStream_t st);
// Fused BF16 training step (forward, relative-L2 gradient, backward, weight gradient) over a batch
// of B samples on `ctas` CTAs (nrc_tc_train_ctas); per-CTA gradient sums go to part[ctas][np].
constexpr int kNrcTcTrainMaxLayers = 6;
uint32_t nrc_tc_train_ctas(uint32_t B);
sty_status nrc_tc_train(const NrcNet &n, const uint16_t *w_img, uint32_t B, const float *input, const float *target,
                        float *part, size_t np, float *loss, uint32_t ctas, cudaStream_t st);

// The reference's composite-encoding network (nrc_grid.cu)
struct GridModel;
sty_status grid_create(const sty_nrc_grid_config *c, GridModel **out, size_t *n_params, size_t *n_mlp);
void grid_destroy(GridModel *g);
sty_status grid_init_params(GridModel *g, uint64_t seed, float *w, cudaStream_t st);
sty_status grid_pack(GridModel *g, const float *w, const float *ema, cudaStream_t st);
// inference with the EMA or the current parameters (packed by grid_pack with both sets); the
// tensor-core path (tile encoder + MMA kernel) when the network fits it and allow_tc, else the
// layer-by-layer path on the tcgen05 row GEMMs (gemm_tc.cu)
sty_status grid_infer(GridModel *g, bool ema, bool allow_tc, uint64_t count, const float *in, float *out,
                      cudaStream_t st);
// the optimiser step (tiny-cuda-nn's Adam: sparse over the tables, per-entry step counts) and the EMA;
// keeps the FP16 table copy current
sty_status grid_adam(GridModel *g, float *w, float *m, float *v, const float *grad, float *ema, float lr, float b1,
                     float b2, float eps, float bc1, float bc2, float ema_decay, float ema_old, float ema_new,
                     cudaStream_t st);
// the parameters were overwritten outside the optimiser (load): the FP16 table copy is stale
void grid_params_changed(GridModel *g);
// zero the tables' per-entry Adam step counts (optimiser reset)
sty_status grid_reset_steps(GridModel *g);
// loss and full parameter gradient of B rows with the current parameters (packed by grid_pack)
sty_status grid_gradient(GridModel *g, uint32_t B, const float *x, const float *target, float *grad, float *loss,
                         cudaStream_t st);

}  // namespace sty
