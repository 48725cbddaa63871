// gemm_tc.cu -- the grid network's layer products on the tcgen05 tensor cores.
//
// Both kernels run one warpgroup per CTA (thread t = TMEM lane t = output row t of a tile), stage
// their operands from row-major global memory into shared memory as no-swizzle core-matrix images
// and issue tcgen05.mma (kind::f16, BF16 or FP16 operands, FP32 accumulator in TMEM) from one
// thread, completion signalled through an mbarrier (bounded waits: a wait that runs out sets the
// device status word and the kernel returns).
//
// Operand images. A row-major R x C tile is stored as core matrices of 8 rows x 16 bytes, 16-byte
// chunk (r, c8) at byte ((r / 8) * (C / 8) + c8) * 128 + (r % 8) * 16. The MMA reads it
//   K-major (C is the reduction dimension): leading offset 128 (next 8 columns along K), stride
//     offset (C / 8) * 128 (next 8 rows), a K step of 16 advances the start by 256 bytes;
//   MN-major (R is the reduction dimension, C the M or N dimension): leading offset (C / 8) * 128
//     (next 8 rows along K), stride offset 128 (next 8 columns along MN), a K step of 16 rows
//     advances the start by 2 (C / 8) 128 bytes.
// So one staging routine serves every operand; the descriptor picks the reading.
//
//   k_gemm_rows: a 128-row tile of A (K-major) times the whole weight matrix (kept in shared
//     memory for the CTA's tiles; K-major for Y = A W^T, MN-major for Y = A W), fused epilogue:
//     FP32 store, ReLU to 16 bits (the next layer's input), or the ReLU mask of the layer below
//     (dL/dz of that layer, 16 bits).
//   k_gemm_dw: the weight gradient P^T Q: both operands MN-major, the reduction runs over a chunk
//     of batch rows in steps of 64 (two staging buffers: the next step's rows are staged while the
//     current MMAs run), the 128 x nq accumulator stays in TMEM across the chunk; k_dw_reduce then
//     adds the chunks' partial sums in a fixed order.
#include <algorithm>

#include "gemm_tc.cuh"
#include "tc.cuh"

namespace sty {
namespace {
using namespace tc;

constexpr int TM = 128;
constexpr int kThreads = 128;
constexpr int kDwStep = 64;                // batch rows per weight-gradient MMA step
constexpr size_t kMinSmem = 100 * 1024;    // at most 2 CTAs per SM: their TMEM (<= 256 columns each) fits

__host__ __device__ constexpr uint32_t idesc16(uint32_t m, uint32_t n, uint32_t a_mn, uint32_t b_mn, uint32_t f16) {
    // D FP32 (bit 4), A / B type (bits 7-9 / 10-12: 0 = FP16, 1 = BF16), A / B MN-major (bits 15 / 16),
    // N >> 3 (bits 17-22), M >> 4 (bits 24-28)
    const uint32_t t = f16 ? 0u : 1u;
    return (1u << 4) | (t << 7) | (t << 10) | (a_mn << 15) | (b_mn << 16) | ((n >> 3) << 17) | ((m >> 4) << 24);
}
__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

// rows [r0, r0 + R) x C columns of a row-major 16-bit matrix (leading dimension ld) into a
// core-matrix image, as asynchronous 16-byte copies (cp.async: every copy of the thread in flight at
// once; the caller commits and waits); slot q holds core matrix q / 8, row q % 8, so consecutive
// threads fill consecutive 16-byte slots; rows at or past `rows` and columns at or past `cvalid`
// are zero-filled (source size 0, the source address then unread)
__device__ __forceinline__ void stage(uint8_t *img, const uint16_t *src, int ld, int r0, int R, int C, int rows,
                                      int tid, int cvalid = 1 << 30) {
    const int ncb = C >> 3, nq = R * ncb;
    const uint32_t dst0 = smem_u32(img);
    for (int q = tid; q < nq; q += kThreads) {
        const int g = q >> 3, rr = q & 7;
        const int rb = g / ncb, cb = g - rb * ncb;
        const int r = r0 + rb * 8 + rr;
        const bool ok = r < rows && cb * 8 < cvalid;
        const uint16_t *p = ok ? src + (size_t)r * ld + cb * 8 : src;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst0 + (uint32_t)q * 16u), "l"(p),
                     "r"(ok ? 16 : 0)
                     : "memory");
    }
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols) : "memory");
}
__device__ __forceinline__ uint32_t pack2_16(float lo, float hi, bool f16, bool relu) {
    uint32_t r;
    if (f16) {
        if (relu) asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
        else asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    } else {
        r = relu ? pack2_relu_bf16(lo, hi) : pack2_bf16(lo, hi);
    }
    return r;
}
// v where the 16-bit value (BF16 or FP16: sign bit 15, zero = +-0) is > 0, else 0
__device__ __forceinline__ float pos_sel(uint32_t h, float v) { return (h & 0x8000u) == 0u && (h & 0x7fffu) != 0u ? v : 0.0f; }

struct RowArgs {
    const uint16_t *a, *w;
    const uint16_t *act;
    float *out32;
    uint16_t *out16;
    uint32_t *status;
    int lda, rows, ka, n, w_mn, f16, epi;
    float scale;
};

__global__ void __launch_bounds__(kThreads) k_gemm_rows(const RowArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t cols = tmem_cols(a.n);
    const uint32_t wbytes = (uint32_t)a.n * a.ka * 2u, abytes = (uint32_t)TM * a.ka * 2u;
    uint8_t *wimg = smem;
    uint8_t *aimgs[2] = {smem + ((wbytes + 1023u) & ~1023u), smem + ((wbytes + 1023u) & ~1023u) + ((abytes + 1023u) & ~1023u)};
    const int ntiles = (a.rows + TM - 1) / TM;
    // the weights and the first tile in one copy group
    if (a.w_mn) stage(wimg, a.w, a.n, 0, a.ka, a.n, a.ka, tid);  // W [ka][n]
    else stage(wimg, a.w, a.ka, 0, a.n, a.ka, a.n, tid);         // W [n][ka]
    if ((int)blockIdx.x < ntiles) stage(aimgs[0], a.a, a.lda, (int)blockIdx.x * TM, TM, a.ka, a.rows, tid);
    cp_commit();
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&tmem_slot, cols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t lane_base = tmem + (((uint32_t)warp * 32u) << 16);
    const uint32_t wbase = smem_u32(wimg);
    const uint32_t sbo_k = (uint32_t)(a.ka / 8) * 128u, nstride = (uint32_t)(a.n / 8) * 128u;
    const uint32_t idesc = idesc16(TM, (uint32_t)a.n, 0u, (uint32_t)a.w_mn, (uint32_t)a.f16);
    const bool f16 = a.f16 != 0;
    uint32_t phase = 0;
    bool failed = false;
    int k = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, k++) {
        const int r0 = tile * TM;
        // prefetch the next tile into the other buffer (its last reader, the previous tile's MMA, has
        // completed: its commit was waited for before that tile's epilogue)
        const int next = tile + (int)gridDim.x;
        if (next < ntiles) {
            stage(aimgs[(k + 1) & 1], a.a, a.lda, next * TM, TM, a.ka, a.rows, tid);
            cp_commit();
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        const uint32_t abase = smem_u32(aimgs[k & 1]);
        if (tid == 0) {
            fence_after();
            for (int ks = 0; ks < a.ka / 16; ks++) {
                const uint64_t ad = make_desc(abase + (uint32_t)ks * 256u, 128u, sbo_k);
                const uint64_t bd = a.w_mn ? make_desc(wbase + (uint32_t)ks * 2u * nstride, nstride, 128u)
                                           : make_desc(wbase + (uint32_t)ks * 256u, 128u, sbo_k);
                mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
            mma_commit(&bar);
        }
        const bool got = mbar_wait(&bar, phase, a.status);
        if (!__syncthreads_and(got)) {
            failed = true;
            break;
        }
        phase ^= 1u;
        fence_after();
        const int row = r0 + tid;
        for (int c0 = 0; c0 < a.n; c0 += 16) {
            float v[16];
            tmem_ld16(lane_base + (uint32_t)c0, v);
            tmem_wait_ld();
            if (row >= a.rows) continue;
#pragma unroll
            for (int i = 0; i < 16; i++) v[i] *= a.scale;
            const size_t o = (size_t)row * a.n + c0;
            if (a.epi == kEpiF32) {
                float4 *d = reinterpret_cast<float4 *>(a.out32 + o);
#pragma unroll
                for (int j = 0; j < 4; j++) d[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            } else {
                if (a.epi == kEpiMask16) {
                    const uint4 *ap = reinterpret_cast<const uint4 *>(a.act + o);
#pragma unroll
                    for (int j = 0; j < 2; j++) {
                        const uint4 h = ap[j];
                        const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            v[8 * j + 2 * k] = pos_sel(hw[k] & 0xffffu, v[8 * j + 2 * k]);
                            v[8 * j + 2 * k + 1] = pos_sel(hw[k] >> 16, v[8 * j + 2 * k + 1]);
                        }
                    }
                }
                const bool relu = a.epi == kEpiRelu16;
                uint4 *d = reinterpret_cast<uint4 *>(a.out16 + o);
#pragma unroll
                for (int j = 0; j < 2; j++)
                    d[j] = make_uint4(pack2_16(v[8 * j], v[8 * j + 1], f16, relu),
                                      pack2_16(v[8 * j + 2], v[8 * j + 3], f16, relu),
                                      pack2_16(v[8 * j + 4], v[8 * j + 5], f16, relu),
                                      pack2_16(v[8 * j + 6], v[8 * j + 7], f16, relu));
            }
        }
        fence_before();
        __syncthreads();
    }
    cp_wait<0>();  // no copy into shared memory outlives the loop
    if (failed) mbar_wait(&bar, phase, a.status);  // the MMAs may still run: one more bounded wait
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_free(tmem, cols);
}

struct DwArgs {
    const uint16_t *p, *q;
    float *partials;
    uint32_t *status;
    int ldp, ldq, rows, mp, nq, chunk, f16;
};

__global__ void __launch_bounds__(kThreads) k_gemm_dw(const DwArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t cols = tmem_cols(a.nq);
    const uint32_t pbytes = kDwStep * TM * 2u, qbytes = (uint32_t)kDwStep * a.nq * 2u;
    const uint32_t bufbytes = ((pbytes + qbytes) + 1023u) & ~1023u;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&tmem_slot, cols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t lane_base = tmem + (((uint32_t)warp * 32u) << 16);
    const int b0 = blockIdx.x * a.chunk, b1 = min(a.rows, b0 + a.chunk);
    const int steps = b1 > b0 ? (b1 - b0 + kDwStep - 1) / kDwStep : 0;
    const uint32_t pstride = (TM / 8) * 128u, qstride = (uint32_t)(a.nq / 8) * 128u;
    const uint32_t idesc = idesc16(TM, (uint32_t)a.nq, 1u, 1u, (uint32_t)a.f16);
    bool failed = false;
    auto issue = [&](int s) {  // step s's rows into buffer s & 1 (P's columns past mp are zero)
        uint8_t *pimg = smem + (size_t)(s & 1) * bufbytes, *qimg = pimg + pbytes;
        const int r0 = b0 + s * kDwStep;
        stage(pimg, a.p, a.ldp, r0, kDwStep, TM, b1, tid, a.mp);
        stage(qimg, a.q, a.ldq, r0, kDwStep, a.nq, b1, tid);
        cp_commit();
    };
    if (steps > 0) issue(0);
    for (int s = 0; s < steps; s++) {
        const int buf = s & 1;
        if (s + 1 < steps) {
            // buffer (s + 1) & 1 was last read by step s - 1's MMAs
            if (s >= 1) {
                const bool got = mbar_wait(&bars[(s + 1) & 1], (uint32_t)((s - 1) >> 1) & 1u, a.status);
                if (!__syncthreads_and(got)) {
                    failed = true;
                    break;
                }
            }
            issue(s + 1);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        uint8_t *pimg = smem + (size_t)buf * bufbytes, *qimg = pimg + pbytes;
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            const uint32_t pb = smem_u32(pimg), qb = smem_u32(qimg);
            for (int ks = 0; ks < kDwStep / 16; ks++)
                mma_bf16(tmem, make_desc(pb + (uint32_t)ks * 2u * pstride, pstride, 128u),
                         make_desc(qb + (uint32_t)ks * 2u * qstride, qstride, 128u), idesc, (s > 0 || ks > 0) ? 1u : 0u);
            mma_commit(&bars[buf]);
        }
    }
    cp_wait<0>();
    if (!failed) {
        bool got = true;
        for (int s = steps >= 2 ? steps - 2 : 0; s < steps; s++)
            got = mbar_wait(&bars[s & 1], (uint32_t)(s >> 1) & 1u, a.status) && got;
        failed = !__syncthreads_and(got);
    } else {
        for (int s = steps >= 2 ? steps - 2 : 0; s < steps; s++) mbar_wait(&bars[s & 1], (uint32_t)(s >> 1) & 1u, a.status);
    }
    fence_after();
    float *dst = a.partials + ((size_t)blockIdx.x * TM + tid) * a.nq;
    for (int c0 = 0; c0 < a.nq; c0 += 16) {
        float v[16];
        tmem_ld16(lane_base + (uint32_t)c0, v);
        tmem_wait_ld();
        const float nan = __int_as_float(0x7fc00000);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float4 o = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            if (steps == 0) o = make_float4(0.f, 0.f, 0.f, 0.f);
            if (failed) o = make_float4(nan, nan, nan, nan);
            reinterpret_cast<float4 *>(dst + c0)[j] = o;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_free(tmem, cols);
}

// 32 consecutive outputs per block, 8 thread groups: group j sums chunks j, j + 8, j + 16, ... in
// order (for one chunk the block reads 32 consecutive floats), then thread j = 0 adds the 8 group
// sums in order -- a fixed summation order for every output
constexpr int kRedOut = 32, kRedGroups = 8;
__global__ void __launch_bounds__(kRedOut * kRedGroups) k_dw_reduce(const float *__restrict__ partials, int nchunks,
                                                                  int mp, int nq, int n_valid, int transpose, int ldd,
                                                                  float scale, float *__restrict__ dst) {
    __shared__ float part[kRedGroups][kRedOut];
    const int o = threadIdx.x % kRedOut, j = threadIdx.x / kRedOut;
    const int i = blockIdx.x * kRedOut + o;
    const size_t stride = (size_t)TM * nq;
    float s = 0.0f;
    if (i < mp * nq)
        for (int c = j; c < nchunks; c += kRedGroups) s += partials[(size_t)c * stride + i];
    part[j][o] = s;
    __syncthreads();
    if (j != 0 || i >= mp * nq) return;
    float t = 0.0f;
#pragma unroll
    for (int k = 0; k < kRedGroups; k++) t += part[k][o];
    const int m = i / nq, n = i - m * nq;
    if (n >= n_valid) return;
    if (transpose) dst[(size_t)n * ldd + m] = t * scale;
    else dst[(size_t)m * ldd + n] = t * scale;
}

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}
// rows per weight-gradient chunk: about one chunk per SM, a multiple of the MMA step
int dw_chunk_rows(int rows) {
    const int sms = sm_count();
    int chunk = (rows + sms - 1) / sms;
    chunk = (chunk + kDwStep - 1) / kDwStep * kDwStep;
    return chunk < kDwStep ? kDwStep : chunk;
}
int dw_chunks(int rows) { return (rows + dw_chunk_rows(rows) - 1) / dw_chunk_rows(rows); }

}  // namespace

sty_status tc_gemm_rows(const uint16_t *a, int lda, const uint16_t *w, int rows, int ka, int n, bool w_mn, bool f16,
                        int epi, float *out32, uint16_t *out16, const uint16_t *act, float scale, cudaStream_t st) {
    STY_ARG_CHECK(ka % 16 == 0 && ka >= 16 && ka <= 256 && n % 16 == 0 && n >= 16 && n <= 256 && lda >= ka &&
                      lda % 8 == 0,
                  "tc_gemm_rows: bad shape ka %d n %d lda %d", ka, n, lda);
    STY_ARG_CHECK(epi == kEpiF32 ? out32 != nullptr : out16 != nullptr, "tc_gemm_rows: null output");
    STY_ARG_CHECK(epi != kEpiMask16 || act, "tc_gemm_rows: null activation");
    if (rows <= 0) return STY_OK;
    RowArgs g;
    g.a = a;
    g.w = w;
    g.act = act;
    g.out32 = out32;
    g.out16 = out16;
    g.status = device_status_ptr();
    STY_ARG_CHECK(g.status, "device status word unavailable");
    g.lda = lda;
    g.rows = rows;
    g.ka = ka;
    g.n = n;
    g.w_mn = w_mn ? 1 : 0;
    g.f16 = f16 ? 1 : 0;
    g.epi = epi;
    g.scale = scale;
    const size_t wb = ((size_t)n * ka * 2 + 1023) & ~(size_t)1023;
    const size_t smem = std::max(kMinSmem, wb + 2 * (((size_t)TM * ka * 2 + 1023) & ~(size_t)1023));
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_gemm_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_gemm_rows)"));
    const int ntiles = (rows + TM - 1) / TM;
    k_gemm_rows<<<std::min(ntiles, 2 * sm_count()), kThreads, smem, st>>>(g);
    return check_launch("k_gemm_rows");
}

size_t tc_dw_partials_floats(int rows, int nq) { return (size_t)dw_chunks(std::max(rows, 1)) * TM * nq; }

sty_status tc_gemm_dw(const uint16_t *p, int ldp, int mp, const uint16_t *q, int ldq, int rows, int nq, bool f16,
                      float *partials, float *dst, int n_valid, bool transpose, int ldd, float scale, cudaStream_t st) {
    STY_ARG_CHECK(nq % 16 == 0 && nq >= 16 && nq <= 256 && mp % 8 == 0 && mp >= 8 && mp <= TM && ldp >= mp &&
                      ldq >= nq && ldp % 8 == 0 && ldq % 8 == 0,
                  "tc_gemm_dw: bad shape mp %d nq %d ldp %d ldq %d", mp, nq, ldp, ldq);
    STY_ARG_CHECK(n_valid >= 0 && n_valid <= nq, "tc_gemm_dw: bad n_valid");
    const int nchunks = dw_chunks(std::max(rows, 1));
    DwArgs g;
    g.p = p;
    g.q = q;
    g.partials = partials;
    g.status = device_status_ptr();
    STY_ARG_CHECK(g.status, "device status word unavailable");
    g.ldp = ldp;
    g.ldq = ldq;
    g.rows = std::max(rows, 0);
    g.mp = mp;
    g.nq = nq;
    g.chunk = dw_chunk_rows(std::max(rows, 1));
    g.f16 = f16 ? 1 : 0;
    const size_t buf = (((size_t)kDwStep * TM * 2 + (size_t)kDwStep * nq * 2) + 1023) & ~(size_t)1023;
    const size_t smem = std::max(kMinSmem, 2 * buf);
    STY_TRY(check_cuda(cudaFuncSetAttribute(k_gemm_dw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "cudaFuncSetAttribute(k_gemm_dw)"));
    k_gemm_dw<<<nchunks, kThreads, smem, st>>>(g);
    STY_TRY(check_launch("k_gemm_dw"));
    k_dw_reduce<<<(mp * nq + kRedOut - 1) / kRedOut, kRedOut * kRedGroups, 0, st>>>(
        partials, nchunks, mp, nq, n_valid, transpose ? 1 : 0, ldd, scale, dst);
    return check_launch("k_dw_reduce");
}

}  // namespace sty
