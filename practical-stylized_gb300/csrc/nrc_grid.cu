// nrc_grid.cu -- the reference's NL-NRC network (crates/akari_integrator/src/nrc_pt.rs:1159-1352):
// a Composite encoding of the 20 + max_depth inputs -- multiresolution hash grid on the position,
// one-blob on the next `blob_dims` inputs, identity on the rest -- and a ReLU MLP of width H without
// biases, linear output, relative L2, Adam + exponential decay, EMA weights for inference.
//
// Encoding (definitions restated from the published papers: tiny-cuda-nn is not available):
//   hash grid: level l: s_l = N_min b^l - 1, r_l = ceil(s_l) + 1, u = clamp(x, 0, 1) s_l + 0.5,
//     trilinear over the 8 corners of floor(u); table T_l = min(roundup8(r_l^3), 2^log2T) entries
//     of F features, dense index when r_l^3 <= T_l else (c.x ^ c.y 2654435761 ^ c.z 805459861) in
//     32-bit arithmetic, both mod T_l. One thread per (sample, level); the backward scatters
//     w * dL/dfeature into the FP32 table gradient with atomics.
//   one-blob: bin k of B gets the mass of N(x, (1/B)^2) over [k/B, (k+1)/B] (erf).
// MLP layers are plain BF16 GEMMs with FP32 accumulation (cuBLAS); ReLU, the ReLU mask, the loss
// gradient and the BF16 packing are the kernels below. Activations are kept in BF16 for the
// backward. Layout: rows are samples; encoded width padded to a multiple of 16, output padded to 8.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "nrc.cuh"

namespace sty {
namespace {

constexpr int kMaxLevels = 32;
constexpr int kOpad = 8;

struct GridGeo {
    int in_dims, levels, feats, blob_dims, bins, out_w;
    float scale[kMaxLevels];
    uint32_t res[kMaxLevels], size[kMaxLevels], off[kMaxLevels];
    int dense[kMaxLevels];
};

__device__ __forceinline__ uint32_t grid_index(const GridGeo &g, int l, uint32_t cx, uint32_t cy, uint32_t cz) {
    uint32_t h;
    if (g.dense[l]) h = cx + cy * g.res[l] + cz * g.res[l] * g.res[l];
    else h = cx ^ (cy * 2654435761u) ^ (cz * 805459861u);
    return g.off[l] + h % g.size[l];
}

// one thread per (sample, level): the level's F features into enc[s][l F ..]
__global__ void k_grid_enc(uint64_t n, const float *__restrict__ x, GridGeo g, const float *__restrict__ tab,
                           __nv_bfloat16 *__restrict__ enc) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n * (uint64_t)g.levels) return;
    const uint64_t s = t / g.levels;
    const int l = (int)(t % g.levels);
    const float *xs = x + s * g.in_dims;
    float u[3], w[3];
    uint32_t c[3];
    for (int a = 0; a < 3; a++) {
        u[a] = fminf(fmaxf(xs[a], 0.0f), 1.0f) * g.scale[l] + 0.5f;
        const float f = floorf(u[a]);
        c[a] = (uint32_t)f;
        w[a] = u[a] - f;
    }
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 8; k++) {
        const uint32_t ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
        const float wt = (ox ? w[0] : 1.0f - w[0]) * (oy ? w[1] : 1.0f - w[1]) * (oz ? w[2] : 1.0f - w[2]);
        const float *e = tab + (size_t)grid_index(g, l, c[0] + ox, c[1] + oy, c[2] + oz) * g.feats;
        for (int f = 0; f < g.feats; f++) acc[f] = fmaf(wt, e[f], acc[f]);
    }
    __nv_bfloat16 *o = enc + s * g.out_w + (size_t)l * g.feats;
    for (int f = 0; f < g.feats; f++) o[f] = __float2bfloat16_rn(acc[f]);
}
// one thread per sample: one-blob bins, identity dims, zero padding
__global__ void k_blob_ident(uint64_t n, const float *__restrict__ x, GridGeo g, __nv_bfloat16 *__restrict__ enc) {
    const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float *xs = x + s * g.in_dims;
    __nv_bfloat16 *o = enc + s * g.out_w;
    int k = g.levels * g.feats;
    const float inv = 1.0f / ((1.0f / g.bins) * 1.41421356237f);
    for (int d = 0; d < g.blob_dims; d++) {
        const float v = xs[3 + d];
        float prev = 0.5f * (1.0f + erff((0.0f - v) * inv));
        for (int b = 0; b < g.bins; b++) {
            const float cdf = 0.5f * (1.0f + erff(((float)(b + 1) / g.bins - v) * inv));
            o[k++] = __float2bfloat16_rn(cdf - prev);
            prev = cdf;
        }
    }
    for (int d = 3 + g.blob_dims; d < g.in_dims; d++) o[k++] = __float2bfloat16_rn(xs[d]);
    for (; k < g.out_w; k++) o[k] = __float2bfloat16_rn(0.0f);
}
// the hash-grid part of the backward: gtab[entry][f] += w * denc[s][l F + f]
__global__ void k_grid_bwd(uint64_t n, const float *__restrict__ x, GridGeo g, const float *__restrict__ denc,
                           float *__restrict__ gtab) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n * (uint64_t)g.levels) return;
    const uint64_t s = t / g.levels;
    const int l = (int)(t % g.levels);
    const float *xs = x + s * g.in_dims;
    float w[3];
    uint32_t c[3];
    for (int a = 0; a < 3; a++) {
        const float u = fminf(fmaxf(xs[a], 0.0f), 1.0f) * g.scale[l] + 0.5f;
        const float f = floorf(u);
        c[a] = (uint32_t)f;
        w[a] = u - f;
    }
    const float *d = denc + s * g.out_w + (size_t)l * g.feats;
    for (int k = 0; k < 8; k++) {
        const uint32_t ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
        const float wt = (ox ? w[0] : 1.0f - w[0]) * (oy ? w[1] : 1.0f - w[1]) * (oz ? w[2] : 1.0f - w[2]);
        float *e = gtab + (size_t)grid_index(g, l, c[0] + ox, c[1] + oy, c[2] + oz) * g.feats;
        for (int f = 0; f < g.feats; f++) atomicAdd(e + f, wt * d[f]);
    }
}
__global__ void k_relu_bf16(size_t n, const float *__restrict__ z, __nv_bfloat16 *__restrict__ a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = __float2bfloat16_rn(fmaxf(z[i], 0.0f));
}
__global__ void k_mask_bf16(size_t n, const float *__restrict__ dh, const __nv_bfloat16 *__restrict__ act,
                            __nv_bfloat16 *__restrict__ dp) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dp[i] = __float2bfloat16_rn(__bfloat162float(act[i]) > 0.0f ? dh[i] : 0.0f);
}
// relative L2 (prediction constant in the denominator): dP = 2 (p - t) / (p^2 + 0.01) / (B O)
__global__ void k_rel_l2_grad(uint32_t B, int O, const float *__restrict__ pred, const float *__restrict__ tgt,
                              __nv_bfloat16 *__restrict__ dp, float *__restrict__ loss) {
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
            dp[(size_t)i * kOpad + c] = __float2bfloat16_rn(g);
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l / ((float)B * (float)O));
}
// FP32 parameters -> BF16 GEMM operands; the output layer padded to kOpad rows of zeros
__global__ void k_weights_bf16(size_t n_mlp, size_t out_off, int O, int H, const float *__restrict__ w,
                               __nv_bfloat16 *__restrict__ wb) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = out_off + (size_t)kOpad * H;
    if (i >= total) return;
    float v = 0.0f;
    if (i < out_off) v = w[i];
    else if ((i - out_off) / H < (size_t)O) v = w[i];
    wb[i] = __float2bfloat16_rn(v);
    (void)n_mlp;
}
__global__ void k_out_rows(uint64_t n, int O, const float *__restrict__ pad, float *__restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n * (uint64_t)O) out[i] = pad[(i / O) * kOpad + i % O];
}
__global__ void k_copy_rows(size_t rows, size_t cols, size_t ld_src, const float *__restrict__ src, float *__restrict__ dst) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows * cols) dst[i] = src[(i / cols) * ld_src + i % cols];
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

}  // namespace

struct GridModel {
    sty_nrc_grid_config cfg;
    GridGeo geo;
    int H, L, O, E;
    size_t n_mlp, n_tab, out_off;
    std::vector<size_t> loff;  // FP32 offsets of W_0 .. W_L (W_L = output layer)
    __nv_bfloat16 *wb = nullptr, *wb_ema = nullptr;
    bool wb_dirty = true;
    cublasHandle_t h = nullptr;
    // batch scratch
    uint64_t cap = 0;
    __nv_bfloat16 *enc = nullptr, *acts = nullptr, *dp = nullptr;
    float *z = nullptr, *dh = nullptr;
    int *d_fan_in = nullptr, *d_fan_out = nullptr;
    size_t *d_loff = nullptr;
};

namespace {

sty_status cublas_ok(cublasStatus_t s, const char *what) {
    if (s == CUBLAS_STATUS_SUCCESS) return STY_OK;
    set_error("%s: cuBLAS status %d", what, (int)s);
    return STY_ERR_CUDA;
}
// row-major Y[B][N] (fp32) = X[B][K] (bf16) . W[N][K]^T (bf16)
sty_status gemm_fwd(GridModel *g, int B, int N, int K, const __nv_bfloat16 *X, const __nv_bfloat16 *W, float *Y) {
    const float one = 1.0f, zero = 0.0f;
    return cublas_ok(cublasGemmEx(g->h, CUBLAS_OP_T, CUBLAS_OP_N, N, B, K, &one, W, CUDA_R_16BF, K, X, CUDA_R_16BF, K,
                                  &zero, Y, CUDA_R_32F, N, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT),
                     "gemm forward");
}
// row-major dX[B][K] (fp32) = dY[B][N] (bf16) . W[N][K] (bf16)
sty_status gemm_dx(GridModel *g, int B, int N, int K, const __nv_bfloat16 *dY, const __nv_bfloat16 *W, float *dX) {
    const float one = 1.0f, zero = 0.0f;
    return cublas_ok(cublasGemmEx(g->h, CUBLAS_OP_N, CUBLAS_OP_N, K, B, N, &one, W, CUDA_R_16BF, K, dY, CUDA_R_16BF, N,
                                  &zero, dX, CUDA_R_32F, K, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT),
                     "gemm input gradient");
}
// row-major dW[N][K] (fp32) = dY[B][N]^T (bf16) . X[B][K] (bf16)
sty_status gemm_dw(GridModel *g, int B, int N, int K, const __nv_bfloat16 *dY, const __nv_bfloat16 *X, float *dW) {
    const float one = 1.0f, zero = 0.0f;
    return cublas_ok(cublasGemmEx(g->h, CUBLAS_OP_N, CUBLAS_OP_T, K, N, B, &one, X, CUDA_R_16BF, K, dY, CUDA_R_16BF, N,
                                  &zero, dW, CUDA_R_32F, K, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT),
                     "gemm weight gradient");
}

sty_status ensure_cap(GridModel *g, uint64_t B) {
    if (B <= g->cap) return STY_OK;
    void *ptrs[] = {g->enc, g->acts, g->dp, g->z, g->dh};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    g->enc = g->acts = g->dp = nullptr;
    g->z = g->dh = nullptr;
    const size_t wide = (size_t)std::max(g->H, g->E);
    STY_TRY(check_cuda(cudaMalloc(&g->enc, B * g->E * 2), "alloc encoding"));
    STY_TRY(check_cuda(cudaMalloc(&g->acts, (size_t)g->L * B * g->H * 2), "alloc activations"));
    STY_TRY(check_cuda(cudaMalloc(&g->dp, B * wide * 2), "alloc layer gradient"));
    STY_TRY(check_cuda(cudaMalloc(&g->z, B * wide * 4), "alloc pre-activations"));
    STY_TRY(check_cuda(cudaMalloc(&g->dh, B * wide * 4), "alloc input gradient"));
    g->cap = B;
    return STY_OK;
}

// forward of B rows with the given BF16 weights and FP32 tables: leaves enc, acts (for the backward)
// and the padded output (B x kOpad) in g->z
sty_status grid_forward(GridModel *g, uint64_t B, const float *x, const float *tables, const __nv_bfloat16 *wb,
                        cudaStream_t st) {
    STY_TRY(cublas_ok(cublasSetStream(g->h, st), "cublasSetStream"));
    const uint64_t nl = B * (uint64_t)g->geo.levels;
    k_grid_enc<<<(unsigned)((nl + 255) / 256), 256, 0, st>>>(B, x, g->geo, tables, g->enc);
    STY_TRY(check_launch("k_grid_enc"));
    k_blob_ident<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(B, x, g->geo, g->enc);
    STY_TRY(check_launch("k_blob_ident"));
    const __nv_bfloat16 *a = g->enc;
    int K = g->E;
    for (int l = 0; l < g->L; l++) {
        STY_TRY(gemm_fwd(g, (int)B, g->H, K, a, wb + g->loff[l], g->z));
        count_launch();
        __nv_bfloat16 *nx = g->acts + (size_t)l * B * g->H;
        k_relu_bf16<<<(unsigned)((B * g->H + 255) / 256), 256, 0, st>>>(B * g->H, g->z, nx);
        STY_TRY(check_launch("k_relu_bf16"));
        a = nx;
        K = g->H;
    }
    STY_TRY(gemm_fwd(g, (int)B, kOpad, g->H, a, wb + g->out_off, g->z));
    count_launch();
    return STY_OK;
}

}  // namespace

// ---- interface used by nrc.cu ----------------------------------------------------------------------
sty_status grid_create(const sty_nrc_grid_config *c, GridModel **out, size_t *n_params, size_t *n_mlp) {
    STY_ARG_CHECK(c->grid_levels >= 1 && c->grid_levels <= kMaxLevels, "grid_levels must be in [1, %d]", kMaxLevels);
    STY_ARG_CHECK(c->grid_features >= 1 && c->grid_features <= 8, "grid_features must be in [1, 8]");
    STY_ARG_CHECK(c->log2_table >= 4 && c->log2_table <= 24, "log2_table must be in [4, 24]");
    STY_ARG_CHECK(c->input_dims >= 3 + c->blob_dims && c->input_dims <= 64, "input_dims must cover 3 + blob_dims");
    STY_ARG_CHECK(c->blob_bins >= 1 && c->blob_bins <= 16, "blob_bins must be in [1, 16]");
    STY_ARG_CHECK(c->hidden_units % 16 == 0 && c->hidden_units >= 16 && c->hidden_units <= 256,
                  "hidden_units must be a multiple of 16 in [16, 256]");
    STY_ARG_CHECK(c->hidden_layers >= 1 && c->hidden_layers <= 8, "hidden_layers must be in [1, 8]");
    STY_ARG_CHECK(c->output_dims >= 1 && c->output_dims <= kOpad, "output_dims must be in [1, %d]", kOpad);
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
        const double scale = (double)c->base_resolution * std::pow((double)c->per_level_scale, l) - 1.0;
        const uint64_t res = (uint64_t)std::ceil(scale) + 1;
        STY_ARG_CHECK(res < (1ull << 31), "grid level %d resolution overflows", l);
        // r^3 exceeds 64 bits at the finest levels of deep grids: compare in double first
        const uint64_t cap = 1ull << c->log2_table;
        const bool fits = (double)res * (double)res * (double)res <= (double)cap;
        const uint64_t size = fits ? std::min<uint64_t>((res * res * res + 7) / 8 * 8, cap) : cap;
        geo.scale[l] = (float)scale;
        geo.res[l] = (uint32_t)res;
        geo.size[l] = (uint32_t)size;
        geo.dense[l] = fits && res * res * res <= size;
        geo.off[l] = (uint32_t)off;
        off += size;
    }
    const int enc = geo.levels * geo.feats + geo.blob_dims * geo.bins + (geo.in_dims - 3 - geo.blob_dims);
    geo.out_w = (enc + 15) / 16 * 16;
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
    g->n_mlp = o + (size_t)g->O * g->H;
    g->n_tab = off * geo.feats;
    *n_params = g->n_mlp + g->n_tab;
    *n_mlp = g->n_mlp;
    sty_status s = cublas_ok(cublasCreate(&g->h), "cublasCreate");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->wb, (g->out_off + (size_t)kOpad * g->H) * 2), "alloc bf16 weights");
    if (s == STY_OK) s = check_cuda(cudaMalloc(&g->wb_ema, (g->out_off + (size_t)kOpad * g->H) * 2), "alloc bf16 ema");
    if (s != STY_OK) {
        grid_destroy(g);
        return s;
    }
    *out = g;
    return STY_OK;
}

void grid_destroy(GridModel *g) {
    if (!g) return;
    void *ptrs[] = {g->wb, g->wb_ema, g->enc, g->acts, g->dp, g->z, g->dh, g->d_fan_in, g->d_fan_out, g->d_loff};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (g->h) cublasDestroy(g->h);
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
    k_grid_init<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g->n_mlp, n, g->d_fan_in, g->d_fan_out, g->d_loff,
                                                             g->L + 1, seed, w);
    return check_launch("k_grid_init");
}

sty_status grid_pack(GridModel *g, const float *w, const float *ema, cudaStream_t st) {
    const size_t total = g->out_off + (size_t)kOpad * g->H;
    k_weights_bf16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g->n_mlp, g->out_off, g->O, g->H, w, g->wb);
    STY_TRY(check_launch("k_weights_bf16"));
    if (ema) {
        k_weights_bf16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g->n_mlp, g->out_off, g->O, g->H, ema,
                                                                         g->wb_ema);
        STY_TRY(check_launch("k_weights_bf16"));
    }
    return STY_OK;
}

sty_status grid_infer(GridModel *g, bool ema, const float *params, uint64_t count, const float *in, float *out,
                      cudaStream_t st) {
    const uint64_t chunk = 1ull << 18;
    STY_TRY(ensure_cap(g, std::min<uint64_t>(count, chunk)));
    const float *tables = params + g->n_mlp;
    for (uint64_t b0 = 0; b0 < count; b0 += chunk) {
        const uint64_t B = std::min<uint64_t>(chunk, count - b0);
        STY_TRY(grid_forward(g, B, in + b0 * g->geo.in_dims, tables, ema ? g->wb_ema : g->wb, st));
        k_out_rows<<<(unsigned)((B * g->O + 255) / 256), 256, 0, st>>>(B, g->O, g->z, out + b0 * g->O);
        STY_TRY(check_launch("k_out_rows"));
    }
    return STY_OK;
}

// loss gradient, backward and the full parameter gradient (MLP weights and tables) of B rows
sty_status grid_gradient(GridModel *g, uint32_t B, const float *x, const float *target, const float *params,
                         float *grad, float *loss, cudaStream_t st) {
    STY_TRY(ensure_cap(g, B));
    STY_TRY(grid_forward(g, B, x, params + g->n_mlp, g->wb, st));
    // dP_out = dLoss/dpred (B x kOpad) in g->dp
    k_rel_l2_grad<<<(B + 255) / 256, 256, 0, st>>>(B, g->O, g->z, target, g->dp, loss);
    STY_TRY(check_launch("k_rel_l2_grad"));
    const __nv_bfloat16 *aL = g->acts + (size_t)(g->L - 1) * B * g->H;
    // dW_out (kOpad x H) into scratch, first O rows into the gradient
    STY_TRY(gemm_dw(g, (int)B, kOpad, g->H, g->dp, aL, g->dh));
    count_launch();
    k_copy_rows<<<(unsigned)(((size_t)g->O * g->H + 255) / 256), 256, 0, st>>>(g->O, g->H, g->H, g->dh,
                                                                                grad + g->out_off);
    STY_TRY(check_launch("k_copy_rows"));
    // dH_{L-1} = dP_out W_out, masked by act_{L-1} > 0
    STY_TRY(gemm_dx(g, (int)B, kOpad, g->H, g->dp, g->wb + g->out_off, g->dh));
    count_launch();
    __nv_bfloat16 *dp = g->dp;
    k_mask_bf16<<<(unsigned)(((size_t)B * g->H + 255) / 256), 256, 0, st>>>((size_t)B * g->H, g->dh, aL, dp);
    STY_TRY(check_launch("k_mask_bf16"));
    for (int l = g->L - 1; l >= 0; l--) {
        const __nv_bfloat16 *al = l == 0 ? g->enc : g->acts + (size_t)(l - 1) * B * g->H;
        const int K = l == 0 ? g->E : g->H;
        STY_TRY(gemm_dw(g, (int)B, g->H, K, dp, al, grad + g->loff[l]));
        count_launch();
        STY_TRY(gemm_dx(g, (int)B, g->H, K, dp, g->wb + g->loff[l], g->dh));
        count_launch();
        if (l > 0) {
            k_mask_bf16<<<(unsigned)(((size_t)B * g->H + 255) / 256), 256, 0, st>>>((size_t)B * g->H, g->dh, al, dp);
            STY_TRY(check_launch("k_mask_bf16"));
        }
    }
    // g->dh now holds dLoss/dencoding (B x E): the tables' gradient
    STY_TRY(check_cuda(cudaMemsetAsync(grad + g->n_mlp, 0, g->n_tab * 4, st), "zero table gradient"));
    const uint64_t nl = (uint64_t)B * g->geo.levels;
    k_grid_bwd<<<(unsigned)((nl + 255) / 256), 256, 0, st>>>(B, x, g->geo, g->dh, grad + g->n_mlp);
    return check_launch("k_grid_bwd");
}

}  // namespace sty
