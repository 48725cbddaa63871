// gemm_tc.cuh -- row-major 16-bit GEMMs on the tcgen05 tensor cores (gemm_tc.cu), the layer
// products of the grid network's layer-by-layer path (training and layered inference).
#pragma once

#include "common.cuh"

namespace sty {

// epilogues of tc_gemm_rows
constexpr int kEpiF32 = 0;     // out32[r][c] = scale * acc
constexpr int kEpiRelu16 = 1;  // out16[r][c] = 16-bit(max(scale * acc, 0))
constexpr int kEpiMask16 = 2;  // out16[r][c] = act[r][c] > 0 ? 16-bit(scale * acc) : 0

// Y[rows][n] = A[rows][ka] . W^T with W = [n][ka] (w_mn = false) or Y = A . W with W = [ka][n]
// (w_mn = true), all row-major 16-bit (f16: FP16, else BF16), FP32 accumulation, then the epilogue.
// ka and n are multiples of 16 (n <= 256, ka <= 256); leading dimensions are the widths (lda >= ka).
sty_status tc_gemm_rows(const uint16_t *a, int lda, const uint16_t *w, int rows, int ka, int n, bool w_mn, bool f16,
                        int epi, float *out32, uint16_t *out16, const uint16_t *act, float scale, cudaStream_t st);

// D[mp][nq] = P^T Q over `rows` rows, P = [rows][mp] (mp <= 128) and Q = [rows][nq] row-major
// 16-bit, FP32 accumulation: each CTA reduces a chunk of rows into partials[chunk][128][nq]
// (`partials` holds at least tc_dw_partials_floats(rows, nq) floats), then one kernel sums the
// chunks in order (the result does not depend on scheduling) and writes scale * D: dst[m][n]
// (n < n_valid, row pitch ldd), or transposed dst[n][m] (n < n_valid, row pitch ldd).
size_t tc_dw_partials_floats(int rows, int nq);
sty_status tc_gemm_dw(const uint16_t *p, int ldp, int mp, const uint16_t *q, int ldq, int rows, int nq, bool f16,
                      float *partials, float *dst, int n_valid, bool transpose, int ldd, float scale, cudaStream_t st);

// 16-bit storage helpers shared with the network's kernels
__device__ __forceinline__ uint16_t to16(float v, bool f16) {
    uint16_t r;
    if (f16)
        asm("cvt.rn.f16.f32 %0, %1;" : "=h"(r) : "f"(v));
    else
        asm("cvt.rn.bf16.f32 %0, %1;" : "=h"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float from16(uint16_t v, bool f16) {
    float r;
    if (f16)
        asm("cvt.f32.f16 %0, %1;" : "=f"(r) : "h"(v));
    else
        r = __uint_as_float((uint32_t)v << 16);
    return r;
}

}  // namespace sty
