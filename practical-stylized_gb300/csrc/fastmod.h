// fastmod.h -- exact 64-bit remainder by a divisor fixed for a launch (Barrett reduction).
//
// With m = floor((2^64 - 1) / d) for d >= 1 and any r < 2^64, q = floor(r * m / 2^64) is either
// floor(r / d) or one less:  r*m/2^64 > r/d - 1 (since m >= (2^64 - d) / d and r < 2^64) and
// r*m/2^64 < r/d (since m < 2^64 / d). So r - q*d lies in [0, 2d) and one conditional subtraction
// gives r % d exactly: a 64 x 64 -> high-64 multiply instead of the long software routine of a
// 64-bit `%` on the GPU. Plain C++ as well, so the host can check it against `%`.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define STY_FASTMOD_HD __host__ __device__
#else
#define STY_FASTMOD_HD
#endif

namespace sty {

inline uint64_t fastmod_magic(uint64_t d) { return UINT64_MAX / d; }  // d >= 1

STY_FASTMOD_HD inline uint64_t fastmod_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

STY_FASTMOD_HD inline uint64_t fastmod(uint64_t r, uint64_t d, uint64_t m) {
    const uint64_t q = fastmod_mulhi(r, m);
    uint64_t rem = r - q * d;
    if (rem >= d) rem -= d;
    return rem;
}

}  // namespace sty
