// pf_screen.cuh -- arguments shared by the screen-space NL-PF kernels.
#pragma once

#include "common.cuh"

namespace sty {

struct ScreenArgs {
    const float *pos[3];
    const float *nrm[3];
    const float *rad[3];
    const float *thr[3];
    const int32_t *valid;
    const float *out_next;
    float *out;
    float *filtered;
    int32_t W, H, R;
    uint32_t depth;
    float pscale;  // sqrt(log2 e / (2 sigma_pos^2))
    float nscale;  // log2 e / sigma_nrm^2
    float pix2;    // log2 e / (2 sigma_pixel^2), 0 if disabled
    uint32_t *status;  // device status word (STY_DEV_* bits)
};

// Warp-specialised kernels for 4 and 16 spp (pf_screen4.cu), and the largest radius they serve
// with `optin` bytes of shared memory per block.
sty_status launch_screen_s4(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st);
sty_status launch_screen_s16(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st);
int screen_ws_max_radius(int spp, size_t optin);

// tcgen05 split-TF32 kernel (pf_screen_tc.cu): 4 spp, radius 15 or 16, 16-byte aligned planes
bool screen_tc_supports(const ScreenArgs &a, int spp);
sty_status launch_screen_tc(const ScreenArgs &a, const sty_style_program &style, cudaStream_t st);

}  // namespace sty
