// common.cuh -- status handling, launch accounting and small device helpers shared by every
// translation unit of libsty_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <string>

#include "sty_gb300.h"

namespace sty {

// Last error message of the calling host thread.
void set_error(const char *fmt, ...);
void clear_error();
// Counts kernel launches issued by this library.
void count_launch(uint64_t n = 1);

// Device status word of the current device (bits STY_DEV_*); kernels OR failure bits into it.
uint32_t *device_status_ptr();
// Unique id of the calling thread's current CUDA context, 0 if unknown: keys caches of device
// addresses of module symbols (a device reset reloads the module).
uint64_t current_context_id();

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Checks the launch that was just issued; returns STY_ERR_CUDA with the CUDA message on failure.
sty_status check_launch(const char *what);
sty_status check_cuda(cudaError_t e, const char *what);

#define STY_ARG_CHECK(cond, ...)              \
    do {                                      \
        if (!(cond)) {                        \
            ::sty::set_error(__VA_ARGS__);    \
            return STY_ERR_ARG;               \
        }                                     \
    } while (0)

#define STY_TRY(expr)                         \
    do {                                      \
        sty_status _s = (expr);               \
        if (_s != STY_OK) return _s;          \
    } while (0)

// ---- device helpers ------------------------------------------------------------------------
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Packed FP32: d = a * b + c on both lanes (fma.rn.f32x2; each lane rounds exactly like fmaf),
// one issue slot for two FMAs.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

struct KahanF {
    float s, c;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

}  // namespace sty
