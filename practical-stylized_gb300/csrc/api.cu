// api.cu -- status/error plumbing and the small element-wise entry points of the C ABI:
// style application, Pcg32 streams, hash-grid cells and the FP64 film accumulation.
#include <cstdarg>
#include <cmath>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "rng.cuh"
#include "style.cuh"

namespace sty {

static thread_local char g_last_error[512] = {0};
static std::atomic<uint64_t> g_launches{0};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}
void clear_error() { g_last_error[0] = 0; }
void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

sty_status check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return STY_OK;
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    if (e == cudaErrorMemoryAllocation) return STY_ERR_OOM;
    return STY_ERR_CUDA;
}
sty_status check_launch(const char *what) {
    count_launch();
    return check_cuda(cudaGetLastError(), what);
}

bool style_program_valid(const sty_style_program *p) {
    if (!p) return true;
    if (p->n_nodes < 0 || p->n_nodes > STY_STYLE_MAX_NODES) return false;
    for (int i = 0; i < p->n_nodes; i++) {
        const sty_style_node &n = p->nodes[i];
        switch (n.kind) {
            case STY_STYLE_NONE:
            case STY_STYLE_TOON:
            case STY_STYLE_SAT_ADJUST:
            case STY_STYLE_SAT_REX:
            case STY_STYLE_EIGHT_BIT:
                break;
            case STY_STYLE_PALETTE:
                if (n.n < 0 || n.n > 19) return false;
                break;
            case STY_STYLE_TOON_STEPS:
            case STY_STYLE_RAMP_SMOOTH:
                if (n.n < 1 || n.n > 8) return false;
                break;
            case STY_STYLE_HALF_TONE:  // the dot spacing divides the mapped point
                if (!(n.p[3] > 0.0f) || !std::isfinite(n.p[3])) return false;
                break;
            default:
                return false;
        }
    }
    return true;
}

// Unique id of the calling thread's current CUDA context (0 if there is none or the driver does not
// say). A device address looked up for a module symbol is valid only while the context that loaded
// the module lives: cudaDeviceReset destroys the primary context and the next use reloads the
// module, possibly at another address, so such caches are keyed on this id.
uint64_t current_context_id() {
    using GetCurrent = int (*)(void **);                  // CUresult cuCtxGetCurrent(CUcontext *)
    using GetId = int (*)(void *, unsigned long long *);  // CUresult cuCtxGetId(CUcontext, unsigned long long *)
    static GetCurrent get_cur = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    if (!get_cur || !get_id) return 0;
    void *ctx = nullptr;
    if (get_cur(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    if (get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device status word: one per device (a __device__ variable exists once per device context).
static __device__ uint32_t g_device_status = 0;

uint32_t *device_status_ptr() {
    struct Entry {
        uint32_t *ptr = nullptr;
        uint64_t ctx = 0;
    };
    static Entry cache[64];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    const uint64_t ctx = current_context_id();
    if (!cache[dev].ptr || ctx == 0 || cache[dev].ctx != ctx) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_status) != cudaSuccess) return nullptr;
        cache[dev].ptr = static_cast<uint32_t *>(p);
        cache[dev].ctx = current_context_id();
    }
    return cache[dev].ptr;
}

// ---- kernels ------------------------------------------------------------------------------
// A wait on an mbarrier whose phase nothing completes, bounded by %globaltimer (and by an
// iteration cap, so the loop ends even if the timer stalled): the timeout path of every bounded
// wait in the library, in isolation.
__global__ void k_wait_timeout_probe(unsigned long long limit_ns, uint32_t *status) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(&bar));
    if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    __syncthreads();
    if (threadIdx.x != 0) return;
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (uint32_t it = 0; it < (1u << 26); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a)
            : "memory");
        if (done) return;
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) break;
    }
    atomicOr(status, (uint32_t)STY_DEV_WAIT_TIMEOUT);
}

__global__ void k_style_apply(sty_style_program prog, uint32_t depth, const float *in, const float *pos, float *out,
                              uint64_t n) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 c = {in[3 * i], in[3 * i + 1], in[3 * i + 2]};
    const f3 p = pos ? f3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]} : f3{0.0f, 0.0f, 0.0f};
    c = style_apply(prog, depth, c, p);
    out[3 * i] = c.x;
    out[3 * i + 1] = c.y;
    out[3 * i + 2] = c.z;
}

__device__ __forceinline__ uint32_t pcg_next(sty_pcg32 &g) {
    uint64_t old = g.state;
    g.state = old * 0x5851f42d4c957f2dULL + g.inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
}

// Pcg32::new_seq_offset + gen_u32 (crates/akari_render/src/sampler/mod.rs:94-123).
__global__ void k_pcg32_streams(const uint64_t *seeds, uint64_t first_seq, uint64_t n, uint32_t draws,
                                uint32_t *out, sty_pcg32 *states) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    sty_pcg32 g;
    g.state = 0;
    g.inc = ((first_seq + i) << 1) | 1ull;
    pcg_next(g);
    g.state += seeds[i];
    pcg_next(g);
    if (out)
        for (uint32_t k = 0; k < draws; k++) out[i * draws + k] = pcg_next(g);
    else
        for (uint32_t k = 0; k < draws; k++) pcg_next(g);
    if (states) states[i] = g;
}

struct RngKey {
    uint32_t k[8];
};
// gen::<u64>() outputs first .. first + n - 1 of StdRng::seed_from_u64 (rng.cuh)
__global__ void k_std_rng_u64(RngKey key, uint64_t first, uint64_t n, uint64_t *out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = std_rng_u64(key.k, first + i);
}

struct GridDesc {
    float pmin[3], pmax[3];
    uint32_t res[3];
    uint32_t table_size;
};

// HashGridVar::get_cell + cell_pos_to_index (lm_path_filtering.rs:20-59).
__global__ void k_hash_cells(const float *pts, uint64_t n, GridDesc g, uint32_t *cell_xyz,
                             uint32_t *cell_index) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float p = __fdiv_rn(pts[3 * i + a] - g.pmin[a], g.pmax[a] - g.pmin[a]);
        p = fminf(fmaxf(p, 0.0f), 1.0f);
        p = __fmul_rn(p, (float)g.res[a]);
        uint32_t u = (uint32_t)p;
        c[a] = min(u, g.res[a] - 1u);
        if (cell_xyz) cell_xyz[3 * i + a] = c[a];
    }
    uint64_t h = ((uint64_t)c[0] * 73856093ull) ^ ((uint64_t)c[1] * 19349663ull) ^ ((uint64_t)c[2] * 83492791ull);
    if (cell_index) cell_index[i] = (uint32_t)(h % (uint64_t)g.table_size);
}

// Pixel mean of the depth-0 outputs over spp, accumulated in FP64 (kernel_splat +
// kernel_update_film, lm_path_filtering.rs:429-506).
__global__ void k_film_accumulate(const float *out0, int32_t npix, int32_t spp, double weight, double *film) {
    int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const size_t N = (size_t)npix * spp;
    for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int k = 0; k < spp; k++) s += (double)out0[c * N + (size_t)p * spp + k];
        film[3 * (size_t)p + c] += weight * (s / spp);
    }
}

}  // namespace sty

using namespace sty;

extern "C" {

int32_t sty_version(void) { return 100; }

const char *sty_status_string(sty_status s) {
    switch (s) {
        case STY_OK: return "STY_OK";
        case STY_ERR_ARG: return "STY_ERR_ARG";
        case STY_ERR_OOM: return "STY_ERR_OOM";
        case STY_ERR_CUDA: return "STY_ERR_CUDA";
        case STY_ERR_ITER_LIMIT: return "STY_ERR_ITER_LIMIT";
        case STY_ERR_NAN: return "STY_ERR_NAN";
        case STY_ERR_UNSUPPORTED: return "STY_ERR_UNSUPPORTED";
        default: return "STY_ERR_UNKNOWN";
    }
}

const char *sty_last_error(void) { return g_last_error; }

uint64_t sty_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

uint64_t sty_struct_size(const char *name) {
    if (!name) return 0;
    if (!strcmp(name, "sty_pcg32")) return sizeof(sty_pcg32);
    if (!strcmp(name, "sty_style_node")) return sizeof(sty_style_node);
    if (!strcmp(name, "sty_style_program")) return sizeof(sty_style_program);
    if (!strcmp(name, "sty_pf_records")) return sizeof(sty_pf_records);
    if (!strcmp(name, "sty_pf_screen_params")) return sizeof(sty_pf_screen_params);
    if (!strcmp(name, "sty_pf_material")) return sizeof(sty_pf_material);
    if (!strcmp(name, "sty_pf_vertices")) return sizeof(sty_pf_vertices);
    if (!strcmp(name, "sty_pf_ref_params")) return sizeof(sty_pf_ref_params);
    if (!strcmp(name, "sty_nrc_config")) return sizeof(sty_nrc_config);
    if (!strcmp(name, "sty_nrc_grid_config")) return sizeof(sty_nrc_grid_config);
    if (!strcmp(name, "sty_scene_material")) return sizeof(sty_scene_material);
    if (!strcmp(name, "sty_camera")) return sizeof(sty_camera);
    if (!strcmp(name, "sty_pf_render_config")) return sizeof(sty_pf_render_config);
    if (!strcmp(name, "sty_nrc_render_config")) return sizeof(sty_nrc_render_config);
    if (!strcmp(name, "sty_nrc_render_stats")) return sizeof(sty_nrc_render_stats);
    if (!strcmp(name, "sty_brpt_config")) return sizeof(sty_brpt_config);
    if (!strcmp(name, "sty_brpt_stats")) return sizeof(sty_brpt_stats);
    if (!strcmp(name, "sty_pf_records_out")) return sizeof(sty_pf_records_out);
    if (!strcmp(name, "sty_pf_nrc_config")) return sizeof(sty_pf_nrc_config);
    return 0;
}

sty_status sty_device_status(uint32_t *status_out, int32_t clear) {
    clear_error();
    STY_ARG_CHECK(status_out, "sty_device_status: null status_out");
    STY_TRY(check_cuda(cudaMemcpyFromSymbol(status_out, g_device_status, sizeof(uint32_t)), "read device status"));
    if (clear) {
        const uint32_t zero = 0;
        STY_TRY(check_cuda(cudaMemcpyToSymbol(g_device_status, &zero, sizeof(uint32_t)), "clear device status"));
    }
    return STY_OK;
}

sty_status sty_wait_timeout_probe(uint32_t limit_us, void *stream) {
    clear_error();
    STY_ARG_CHECK(limit_us >= 1 && limit_us <= 2000000u, "sty_wait_timeout_probe: limit_us must be in [1, 2e6]");
    uint32_t *st = device_status_ptr();
    if (!st) {
        set_error("sty_wait_timeout_probe: device status word unavailable");
        return STY_ERR_CUDA;
    }
    k_wait_timeout_probe<<<1, 32, 0, as_stream(stream)>>>((unsigned long long)limit_us * 1000ull, st);
    return check_launch("k_wait_timeout_probe");
}

sty_status sty_style_apply(const sty_style_program *program, uint32_t depth, const float *rgb_in,
                           float *rgb_out, uint64_t n, void *stream) {
    clear_error();
    STY_ARG_CHECK(program && rgb_in && rgb_out, "sty_style_apply: null argument");
    STY_ARG_CHECK(style_program_valid(program), "sty_style_apply: invalid style program");
    if (n == 0) return STY_OK;
    const int bs = 256;
    k_style_apply<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(*program, depth, rgb_in, nullptr,
                                                                             rgb_out, n);
    return check_launch("sty_style_apply");
}

sty_status sty_style_apply_at(const sty_style_program *program, uint32_t depth, const float *rgb_in, const float *pos,
                              float *rgb_out, uint64_t n, void *stream) {
    clear_error();
    STY_ARG_CHECK(program && rgb_in && rgb_out, "sty_style_apply_at: null argument");
    STY_ARG_CHECK(style_program_valid(program), "sty_style_apply_at: invalid style program");
    if (n == 0) return STY_OK;
    const int bs = 256;
    k_style_apply<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(*program, depth, rgb_in, pos, rgb_out,
                                                                             n);
    return check_launch("sty_style_apply_at");
}

sty_status sty_pcg32_streams(const uint64_t *seeds, uint64_t first_seq, uint64_t n, uint32_t draws,
                             uint32_t *out, sty_pcg32 *states, void *stream) {
    clear_error();
    STY_ARG_CHECK(seeds, "sty_pcg32_streams: null seeds");
    STY_ARG_CHECK(out || states, "sty_pcg32_streams: nothing to write");
    if (n == 0) return STY_OK;
    const int bs = 256;
    k_pcg32_streams<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(seeds, first_seq, n, draws, out, states);
    return check_launch("sty_pcg32_streams");
}

sty_status sty_std_rng_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t *out, void *stream) {
    clear_error();
    STY_ARG_CHECK(out, "sty_std_rng_u64: null out");
    STY_ARG_CHECK(n < (1ull << 40), "sty_std_rng_u64: n too large");
    if (n == 0) return STY_OK;
    RngKey key;
    std_rng_key(seed, key.k);
    const int bs = 256;
    k_std_rng_u64<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(key, first, n, out);
    return check_launch("sty_std_rng_u64");
}

sty_status sty_hash_cells(const float *points, uint64_t n, const float pmin[3], const float pmax[3],
                          const uint32_t res[3], uint32_t table_size, uint32_t *cell_xyz,
                          uint32_t *cell_index, void *stream) {
    clear_error();
    STY_ARG_CHECK(points && pmin && pmax && res, "sty_hash_cells: null argument");
    STY_ARG_CHECK(table_size > 0 && res[0] > 0 && res[1] > 0 && res[2] > 0, "sty_hash_cells: empty grid");
    STY_ARG_CHECK(cell_xyz || cell_index, "sty_hash_cells: nothing to write");
    if (n == 0) return STY_OK;
    GridDesc g;
    for (int a = 0; a < 3; a++) {
        g.pmin[a] = pmin[a];
        g.pmax[a] = pmax[a];
        g.res[a] = res[a];
    }
    g.table_size = table_size;
    const int bs = 256;
    k_hash_cells<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(points, n, g, cell_xyz, cell_index);
    return check_launch("sty_hash_cells");
}

sty_status sty_film_accumulate(const float *out0, int32_t width, int32_t height, int32_t spp, double weight,
                               double *film, void *stream) {
    clear_error();
    STY_ARG_CHECK(out0 && film, "sty_film_accumulate: null argument");
    STY_ARG_CHECK(width > 0 && height > 0 && spp > 0, "sty_film_accumulate: bad size %dx%dx%d", width, height, spp);
    const int npix = width * height;
    const int bs = 256;
    k_film_accumulate<<<(npix + bs - 1) / bs, bs, 0, as_stream(stream)>>>(out0, npix, spp, weight, film);
    return check_launch("sty_film_accumulate");
}

}  // extern "C"
