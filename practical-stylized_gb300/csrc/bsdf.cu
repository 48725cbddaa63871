// bsdf.cu -- the principled BSDF's albedo table (one per device) and the entry points that expose
// the device BSDF for checking against the oracle.
//
// The table ggx_dielectric_s (precompute.rs:100-145): cell (x, y, z) of 16^3 holds the mean of
// f/pdf of a unit-colour GGX reflection with dielectric Fresnel, at roughness = x/15, mu = y/15 and
// ior = ior_from_f0((z/15)^4) (each coordinate clamped to [1e-4, 0.9999]), over the
// visible-normal sample (u0, u1). The reference estimates it by Monte Carlo (2^20 samples per
// cell); here it is the same integral over (u0, u1) by a 256 x 256 midpoint rule, summed in a fixed
// order (deterministic).
#include <map>
#include <mutex>

#include "bsdf.cuh"
#include "common.cuh"

namespace sty {
namespace {

constexpr int kQuad = 256;

__global__ void k_ggx_table(float *t) {
    const int cell = blockIdx.x;
    const int xi = cell % bsdf::kTabN, yi = (cell / bsdf::kTabN) % bsdf::kTabN, zi = cell / (bsdf::kTabN * bsdf::kTabN);
    auto coord = [](int i) { return fminf(fmaxf((float)i / (float)(bsdf::kTabN - 1), 1e-4f), 0.9999f); };
    const float rough = coord(xi), mu = coord(yi), z = coord(zi);
    const float ior = bsdf::ior_from_f0(z * z * z * z);
    float sum = 0.0f;
    for (int k = threadIdx.x; k < kQuad * kQuad; k += blockDim.x) {
        const float u0 = ((float)(k % kQuad) + 0.5f) / kQuad, u1 = ((float)(k / kQuad) + 0.5f) / kQuad;
        sum += bsdf::ggx_albedo_sample(rough, mu, ior, u0, u1);
    }
    __shared__ float red[256];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) t[cell] = red[0] / (float)(kQuad * kQuad);
}

template <class M>
__device__ __forceinline__ bsdf::B3 ld3(const float *a, uint64_t i) {
    return bsdf::b3(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
}
__global__ void k_bsdf_eval(sty_scene_material m, const float *tab, uint64_t n, const float *wo, const float *wi,
                            float *f, float *pdf) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bsdf::PClosure c = bsdf::make_closure(m);
    float fv[3];
    pdf[i] = bsdf::eval(c, tab, ld3<int>(wo, i), ld3<int>(wi, i), fv);
    for (int k = 0; k < 3; k++) f[3 * i + k] = fv[k];
}
__global__ void k_bsdf_sample(sty_scene_material m, const float *tab, uint64_t n, const float *wo, const float *u,
                              float *wi, float *f, float *pdf) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bsdf::PClosure c = bsdf::make_closure(m);
    const bsdf::B3 o = ld3<int>(wo, i);
    bsdf::B3 w = bsdf::b3(0.0f, 0.0f, 0.0f);
    float fv[3] = {0.0f, 0.0f, 0.0f}, p = 0.0f;
    if (bsdf::sample(c, tab, o, u[3 * i], u[3 * i + 1], u[3 * i + 2], &w)) p = bsdf::eval(c, tab, o, w, fv);
    if (!(p > 0.0f)) {
        p = 0.0f;
        fv[0] = fv[1] = fv[2] = 0.0f;
    }
    wi[3 * i] = w.x;
    wi[3 * i + 1] = w.y;
    wi[3 * i + 2] = w.z;
    for (int k = 0; k < 3; k++) f[3 * i + k] = fv[k];
    pdf[i] = p;
}

}  // namespace

const float *principled_table() {
    static std::mutex mu;
    static std::map<int, float *> tables;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    auto it = tables.find(dev);
    if (it != tables.end()) return it->second;
    float *t = nullptr;
    const int cells = bsdf::kTabN * bsdf::kTabN * bsdf::kTabN;
    if (cudaMalloc(&t, cells * sizeof(float)) != cudaSuccess) return nullptr;
    k_ggx_table<<<cells, 256>>>(t);
    count_launch();
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaFree(t);
        return nullptr;
    }
    tables[dev] = t;
    return t;
}

}  // namespace sty

using namespace sty;

sty_status sty_principled_table(float *host_table) {
    clear_error();
    STY_ARG_CHECK(host_table, "sty_principled_table: null argument");
    const float *t = principled_table();
    if (!t) {
        set_error("principled albedo table: %s", cudaGetErrorString(cudaGetLastError()));
        return STY_ERR_CUDA;
    }
    return check_cuda(cudaMemcpy(host_table, t, bsdf::kTabN * bsdf::kTabN * bsdf::kTabN * sizeof(float),
                                 cudaMemcpyDeviceToHost),
                      "read table");
}

sty_status sty_bsdf_eval(const sty_scene_material *material, uint64_t n, const float *wo, const float *wi, float *f,
                         float *pdf, void *stream) {
    clear_error();
    STY_ARG_CHECK(material && (n == 0 || (wo && wi && f && pdf)), "sty_bsdf_eval: null argument");
    STY_ARG_CHECK(bsdf::closure_kind(material->kind), "sty_bsdf_eval: only STY_MAT_PRINCIPLED and STY_MAT_GLASS are exposed");
    if (n == 0) return STY_OK;
    const float *t = principled_table();
    if (!t) {
        set_error("principled albedo table unavailable");
        return STY_ERR_CUDA;
    }
    k_bsdf_eval<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(*material, t, n, wo, wi, f, pdf);
    return check_launch("k_bsdf_eval");
}

sty_status sty_bsdf_sample(const sty_scene_material *material, uint64_t n, const float *wo, const float *u, float *wi,
                           float *f, float *pdf, void *stream) {
    clear_error();
    STY_ARG_CHECK(material && (n == 0 || (wo && u && wi && f && pdf)), "sty_bsdf_sample: null argument");
    STY_ARG_CHECK(bsdf::closure_kind(material->kind), "sty_bsdf_sample: only STY_MAT_PRINCIPLED and STY_MAT_GLASS are exposed");
    if (n == 0) return STY_OK;
    const float *t = principled_table();
    if (!t) {
        set_error("principled albedo table unavailable");
        return STY_ERR_CUDA;
    }
    k_bsdf_sample<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(*material, t, n, wo, u, wi, f, pdf);
    return check_launch("k_bsdf_sample");
}
