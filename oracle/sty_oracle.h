/*
 * sty_oracle.h -- CPU restatement of the reference's NL-PF / style / RNG arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and by nothing else.
 * The product library (libsty_gb300.so) never links or calls it.
 *
 * Parity status: the reference ships no golden vectors, known-answer tests or fixtures for this
 * path and cannot be built here (Rust + LuisaCompute JIT, no toolchain). Every function below
 * restates the cited reference lines; the known-answer vectors under tests/golden/ were derived
 * by hand from those lines (see tests/golden/make_golden.py). Parity of the screen-space filter
 * is against this restatement only ("parity unpinned" against a reference binary).
 *
 * All functions take HOST pointers. Real-valued work is done in double ("_f64") unless the name
 * ends in "_f32" (the FP32 restatement used as the timed CPU baseline).
 */
#ifndef STY_ORACLE_H
#define STY_ORACLE_H
#include <stdint.h>
#include "../include/sty_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int32_t orc_num_threads(void);
void orc_set_num_threads(int32_t n);

/* Style program on n interleaved rgb triples (double). */
void orc_style_apply_at_f64(const sty_style_program *prog, uint32_t depth, const double *rgb_in, const double *pos,
                            double *rgb_out, uint64_t n);
void orc_style_apply_f64(const sty_style_program *prog, uint32_t depth, const double *rgb_in,
                         double *rgb_out, uint64_t n);

/* Screen-space NL-PF, one depth, FP64. Same contract as sty_pf_screen_filter_depth but host
 * pointers, and out_next / out / filtered are double planes. */
void orc_pf_screen_filter_depth_f64(const sty_pf_records *rec, uint32_t depth,
                                    const sty_pf_screen_params *params,
                                    const sty_style_program *style, const double *out_next,
                                    double *out, double *filtered);
/* Same on float planes, FP32 arithmetic with compensated sums (CPU baseline). Processes only
 * query rows [y0, y1) so a bounded sample can be timed. */
void orc_pf_screen_filter_records_f64(const sty_pf_records *rec, uint32_t depth, const sty_pf_screen_params *params,
                                      const sty_style_program *style, const double *out_next, const uint64_t *idx,
                                      uint64_t n_idx, double *out, double *filtered);
void orc_pf_screen_filter_depth_f32(const sty_pf_records *rec, uint32_t depth,
                                    const sty_pf_screen_params *params,
                                    const sty_style_program *style, const float *out_next,
                                    float *out, float *filtered, int32_t y0, int32_t y1);

/* Pcg32 (sampler/mod.rs:82-137): new_seq_offset(first_seq+i, seeds[i]) then `draws` draws. */
void orc_pcg32_streams(const uint64_t *seeds, uint64_t first_seq, uint64_t n, uint32_t draws,
                       uint32_t *out, sty_pcg32 *states);

/* ChaCha block function (out = rounds of `in` + in; 16 words each). */
void orc_chacha_block(const uint32_t *in, uint32_t *out, int32_t rounds);
/* rand_core 0.6.4 seed_from_u64 key of a ChaCha12Rng (8 words). */
void orc_std_rng_key(uint64_t seed, uint32_t *key);
/* gen::<u64>() outputs first .. first+n-1 of StdRng::seed_from_u64(seed) (sampler/mod.rs:157-173). */
void orc_std_rng_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t *out);
/* Depth-0 camera rays of every path slot (as sty_scene_camera_rays). */
void orc_camera_rays(const sty_camera *cam, uint32_t branch, uint64_t seed, float *rays);

/* Hash-grid cell (lm_path_filtering.rs:20-59), float arithmetic as in the reference. */
void orc_hash_cells(const float *points, uint64_t n, const float pmin[3], const float pmax[3],
                    const uint32_t res[3], uint32_t table_size, uint32_t *cell_xyz,
                    uint32_t *cell_index);

#ifdef __cplusplus
}
#endif
#endif
