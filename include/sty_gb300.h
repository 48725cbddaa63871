/*
 * sty_gb300.h -- C ABI of the GB300-native stylized nonlinear rendering hot path.
 *
 * Plain C, bindgen-clean: opaque handles, plain pointers and sizes, int32 status codes.
 * No call aborts the process; every entry point returns a sty_status and leaves a
 * human-readable message for sty_last_error().
 *
 * Memory: every pointer argument documented as "device" must point into CUDA device memory of
 * the current device (or managed memory); the caller owns it. Streams are plain cudaStream_t
 * values passed as void* (NULL = the legacy default stream). No entry point performs a
 * device-wide synchronisation unless documented.
 *
 * Record layout of the screen-space path-vertex buffers (sty_pf_records): every field is a
 * separate array of `depths * height * width * spp` elements indexed as
 *     i = ((d * height + y) * width + x) * spp + s
 * i.e. the spp samples of one pixel are adjacent, then pixels in a row, rows, depths.
 *
 * Reference interfaces this ABI replaces (paths relative to the reference project):
 *   - crates/akari_integrator/src/lm_path_filtering.rs:758-1060 (evaluate_filtered_radiance,
 *     kernel_filter) and :974-998 (kernel_propagate): the NL-PF per-depth filter pass.
 *   - crates/akari_render/src/svm/surface/mod.rs:492-1346 (the sty_* style nodes applied by
 *     Surface::apply_stylization).
 *   - crates/akari_integrator/src/lm_path_filtering.rs:20-59 (hash, get_cell, cell index).
 *   - crates/akari_render/src/sampler/mod.rs:82-137 (Pcg32).
 */
#ifndef STY_GB300_H
#define STY_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define STY_API __attribute__((visibility("default")))
#else
#define STY_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------------------------
 * Status codes
 * -------------------------------------------------------------------------------------- */
typedef int32_t sty_status;
#define STY_OK 0
#define STY_ERR_ARG 1         /* invalid argument (null pointer, bad size, bad enum)        */
#define STY_ERR_OOM 2         /* a device allocation failed                                  */
#define STY_ERR_CUDA 3        /* a CUDA runtime call failed (message in sty_last_error())    */
#define STY_ERR_ITER_LIMIT 4  /* a bounded device loop hit its iteration cap                 */
#define STY_ERR_NAN 5         /* a non-finite value was detected where it is not allowed     */
#define STY_ERR_UNSUPPORTED 6 /* the request is valid but the library as compiled or the device cannot serve it */

/* Pcg32 generator state (crates/akari_render/src/sampler/mod.rs:82-88). */
typedef struct sty_pcg32 {
    uint64_t state;
    uint64_t inc;
} sty_pcg32;

/* Version of this ABI: major * 10000 + minor * 100 + patch. */
STY_API int32_t sty_version(void);
/* Static string naming a status code. */
STY_API const char *sty_status_string(sty_status status);
/* Message of the last failing call on the calling host thread ("" if none). */
STY_API const char *sty_last_error(void);
/* Number of kernels this library launched since load (all threads, all devices). Used by
 * benchmarks to count launches inside a timed region. */
STY_API uint64_t sty_launch_count(void);
/* sizeof of the struct this header names `name` (e.g. "sty_brpt_config") as the library was
 * compiled, 0 for an unknown name: lets a binding check its struct layouts against the library. */
STY_API uint64_t sty_struct_size(const char *name);

/* Device status word of the current device: kernels that hit a bounded wait (instead of
 * hanging) OR a STY_DEV_* bit into it and return. Reading synchronises the device;
 * clear != 0 resets the word to 0 after reading. */
#define STY_DEV_WAIT_TIMEOUT 1u
STY_API sty_status sty_device_status(uint32_t *status_out, int32_t clear);
/* Exercises the bounded-wait failure path without a fault: one block waits on an mbarrier that
 * nothing completes; after `limit_us` microseconds (1 .. 2 000 000) of %globaltimer the wait gives
 * up, ORs STY_DEV_WAIT_TIMEOUT into the device status word and the kernel returns, leaving the
 * context usable. No counterpart in the reference (its kernels have no bounded waits). */
STY_API sty_status sty_wait_timeout_probe(uint32_t limit_us, void *stream);

/* ----------------------------------------------------------------------------------------
 * Style programs: the nonlinear "svm/surface" style nodes
 *
 * A program is a chain of up to STY_STYLE_MAX_NODES nodes applied innermost first, exactly as
 * the reference applies `inner.apply_stylization` before its own operation
 * (crates/akari_render/src/svm/surface/mod.rs:573-610 and siblings). Node i runs at path depth
 * d only if bit min(d,31) of nodes[i].depth_mask is set.
 *
 * Parameter layout per kind (p[] = node.p, n = node.n):
 *   STY_STYLE_TOON        reference sty_toon (mod.rs:573-610):        p[0] = color_band_width
 *   STY_STYLE_PALETTE     reference sty_color_palette (mod.rs:697-735): p[0] = indirect_scale,
 *                         p[1] = gamma, n = palette length (<= 19), p[2+3k .. 4+3k] = colour k
 *   STY_STYLE_SAT_ADJUST  reference sty_saturation_adjust (mod.rs:821-851): p[0] = power,
 *                         p[1] = indirect_scale
 *   STY_STYLE_SAT_REX     reference sty_saturation_adjust_rex (mod.rs:1060-1089): p[0] = blend
 *   STY_STYLE_EIGHT_BIT   reference sty_8bit (mod.rs:1316-1345): p[0] = indirect_scale
 *   STY_STYLE_TOON_STEPS  hard threshold toon on Rec.709 luminance, hue preserving:
 *                         n thresholds (1..8) p[0..n-1] ascending, n+1 output luminance levels
 *                         p[8..8+n]; out = rgb / lum * level(#{t_k <= lum})
 *   STY_STYLE_RAMP_SMOOTH smoothed colour ramp on Rec.709 luminance (differentiable):
 *                         n steps (1..8), p[0] = sharpness s, p[1..8] = thresholds t_k,
 *                         p[9+3k .. 11+3k] = colour c_k;
 *                         out = sum_k sigmoid(s * (lum - t_k)) * (c_k - c_{k-1}), c_{-1} = 0
 *   STY_STYLE_HALF_TONE   reference sty_half_tone (mod.rs:1091-1233), a world-space dot screen:
 *                         p[0] = indirect_scale, p[1] = radius_scale, p[2] = radius,
 *                         p[3] = grid_distance d, p[4] = max_depth, p[5] = blend,
 *                         p[6..8] = dark_tone, p[9..11] = light_tone, p[12..23] = the node's TRS as
 *                         a 3 x 4 row-major affine map. At depth <= max_depth with
 *                         lum = (r + g + b) / 3 != 0: r' = 1 - clamp(lum / radius_scale (depth 0) or
 *                         round(lum / indirect_scale) / radius_scale, 0, 1), dot radius
 *                         r' d radius / 2; the nearest of the 8 corners q of
 *                         floor(affine(p) / d) d (distance |q - p|, p untransformed, as the
 *                         reference computes it) picks dark_tone (inside) or light_tone; out =
 *                         lerp(li, tone * li, blend). Needs the shaded point p: calls without one
 *                         (sty_style_apply, the screen-space filter) use p = 0.
 * -------------------------------------------------------------------------------------- */
#define STY_STYLE_NONE 0
#define STY_STYLE_TOON 1
#define STY_STYLE_PALETTE 2
#define STY_STYLE_SAT_ADJUST 3
#define STY_STYLE_SAT_REX 4
#define STY_STYLE_EIGHT_BIT 5
#define STY_STYLE_TOON_STEPS 7
#define STY_STYLE_RAMP_SMOOTH 8
#define STY_STYLE_HALF_TONE 9

#define STY_STYLE_MAX_NODES 4
#define STY_STYLE_MAX_PARAMS 60

typedef struct sty_style_node {
    int32_t kind;
    uint32_t depth_mask;
    int32_t n;
    int32_t reserved;
    float p[STY_STYLE_MAX_PARAMS];
} sty_style_node;

typedef struct sty_style_program {
    int32_t n_nodes;
    int32_t reserved[3];
    sty_style_node nodes[STY_STYLE_MAX_NODES];
} sty_style_program;

/* Apply a style program to `n` RGB triples (device, interleaved rgb, in-place allowed) at path
 * depth `depth`. Replaces Surface::apply_stylization for one material
 * (crates/akari_render/src/svm/surface/mod.rs:262-285). */
STY_API sty_status sty_style_apply(const sty_style_program *program, uint32_t depth, const float *rgb_in,
                           float *rgb_out, uint64_t n, void *stream);
/* sty_style_apply with the shaded point of each colour (device, 3 floats per item), which
 * STY_STYLE_HALF_TONE reads (si.p in HalfToneSurface::apply_stylization, svm/surface/mod.rs:1180-1232); a null `pos` is the point 0 for every item (sty_style_apply). */
STY_API sty_status sty_style_apply_at(const sty_style_program *program, uint32_t depth, const float *rgb_in,
                                      const float *pos, float *rgb_out, uint64_t n, void *stream);

/* ----------------------------------------------------------------------------------------
 * Screen-space NL-PF filter
 *
 * Per depth d (processed from the deepest to 0, like the reference's backward loop
 * lm_path_filtering.rs:1673-1774), for every valid record i = (d, y, x, s):
 *   in_d(j)  = rad(d, j) + thr(d, j) * out_{d+1}(j)          (out_{D} = 0)
 *   f_d(i)   = sum_j w_ij in_d(j) / sum_j w_ij,   j over valid records (d, y', x', s') with
 *              |x'-x| <= radius, |y'-y| <= radius, inside the image, any s'
 *   w_ij     = exp(-((x'-x)^2 + (y'-y)^2) / (2 sigma_pixel^2)
 *                  - |pos_i - pos_j|^2 / (2 sigma_pos^2) - (1 - nrm_i . nrm_j) / sigma_nrm^2)
 *   out_d(i) = style(d, f_d(i))                              (0 for invalid records)
 * The inner sums are FP32 with compensated (Kahan) accumulation. sigma_pixel <= 0 drops the
 * pixel-distance term. The throughput product thr(d-1) * out_d is the "indirect" term that
 * lm_path_filtering.rs:864-885 forms as f * L * mis / pdf.
 * -------------------------------------------------------------------------------------- */
typedef struct sty_pf_records {
    const float *pos[3];  /* device, world-space vertex position                     */
    const float *nrm[3];  /* device, unit shading normal                             */
    const float *rad[3];  /* device, radiance leaving the vertex without the next bounce */
    const float *thr[3];  /* device, throughput from this vertex to the next one     */
    const int32_t *valid; /* device, nonzero if the record holds a vertex            */
    int32_t width, height, spp, depths;
} sty_pf_records;

typedef struct sty_pf_screen_params {
    int32_t radius;    /* half window in pixels, 0..32 */
    float sigma_pixel; /* pixels; <= 0 disables the pixel-distance term */
    float sigma_pos;   /* world units, > 0 */
    float sigma_nrm;   /* > 0 */
} sty_pf_screen_params;

/* spp must be 1, 2, 4, 8 or 16; radius up to 32 (up to 24 at 4 spp for the fastest kernel). */

/* Filter one depth. `out_next` (device, 3 planes of width*height*spp floats: r plane, g plane,
 * b plane) holds out_{d+1} or is NULL at the deepest depth. `out` receives out_d with the same
 * layout. `filtered` (optional, same layout) receives f_d before the style node. */
STY_API sty_status sty_pf_screen_filter_depth(const sty_pf_records *rec, uint32_t depth,
                                      const sty_pf_screen_params *params,
                                      const sty_style_program *style, const float *out_next,
                                      float *out, float *filtered, void *stream);

/* Which kernel serves the screen filter (process-wide; every sty_pf_screen_filter* call and SCREEN
 * render after it). Returns STY_ERR_ARG for an unknown value.
 *   STY_SCREEN_KERNEL_AUTO    the fastest kernel that serves the records' spp and radius
 *   STY_SCREEN_KERNEL_FP32    the CUDA-core kernels (packed FP32 FMAs) at every spp and radius
 *   STY_SCREEN_KERNEL_TENSOR  the tcgen05 kernel where it serves the configuration (4 spp, radius
 *                             15 or 16: logits and weighted sums as split-TF32 products with FP32
 *                             accumulation), the CUDA-core kernels elsewhere */
#define STY_SCREEN_KERNEL_AUTO 0
#define STY_SCREEN_KERNEL_FP32 1
#define STY_SCREEN_KERNEL_TENSOR 2
STY_API sty_status sty_pf_screen_set_kernel(int32_t kernel);

/* Filter all depths, deepest first. `out` (device) holds 3 * depths planes laid out as
 * [depth][channel][height*width*spp]; on return out[d] = out_d for every depth. */
STY_API sty_status sty_pf_screen_filter(const sty_pf_records *rec, const sty_pf_screen_params *params,
                                const sty_style_program *style, float *out, void *stream);

/* Average the depth-0 outputs of each pixel over its spp samples and add them into an FP64
 * progressive film (device, width*height*3 doubles, interleaved rgb):
 *   film[p] += weight * mean_s out_0(p, s)
 * Replaces kernel_splat + kernel_update_film (lm_path_filtering.rs:429-506); FP64 is used only
 * for this accumulation across iterations. */
STY_API sty_status sty_film_accumulate(const float *out0, int32_t width, int32_t height, int32_t spp,
                               double weight, double *film, void *stream);

/* ----------------------------------------------------------------------------------------
 * Reference-mode NL-PF (world-space hash grid + SMIS), one path depth per call
 *
 * Restates lm_path_filtering.rs with a fixed evaluation order:
 *   grid     HashGrid (:20-255): cell = clamp((p-pmin)/(pmax-pmin),0,1)*res, res = floor(extent/r),
 *            bucket = hash(cell) mod table_size; the 27-cell walk (:61-123, dz outer, dx inner).
 *            The reference's buckets are CAS-built linked lists (order = thread timing); here each
 *            bucket lists its points in ascending path index.
 *   cluster  kernel_init_cluster / kernel_cluster (:533-623, loop :1675-1710) with deterministic
 *            claims: per round every unclustered vertex's bucket elects its lowest-index vertex as
 *            a centre; every other unclustered vertex proposes to the first centre (walk order) within
 *            r that had room at the start of the round; each centre accepts proposals in walk order
 *            while it has room (cluster_size < reuse). Rounds repeat until every vertex is clustered.
 *   filter   evaluate_filtered_radiance (:758-972): neighbours = active vertices within r of the query
 *            point (own position, or the cluster centre's), same cluster, same flags; reservoir of
 *            `reuse` slots fed by the path's Pcg32 (gen_u32 % (cnt+1)); direct term with balance MIS;
 *            indirect term with SMIS (sum of the kept neighbours' BSDF pdfs) or 1/(pdf*k); then the
 *            material's style program (skipped at depth 0 if no_first_hit_stylization, and when the
 *            vertex's flags have bit 0 "stylization disabled" set).
 * All per-vertex arrays below are device arrays of `n` elements indexed by path slot.
 * -------------------------------------------------------------------------------------- */
#define STY_MAT_DIFFUSE 0 /* Lambert: f = albedo/pi |cos|, pdf = |cos|/pi (diffuse.rs:17-48)       */
#define STY_MAT_GGX 1     /* microfacet reflection, Trowbridge-Reitz alpha, unit Fresnel,
                             visible-normal pdf (mod.rs:1877-1910, microfacet.rs:44-206)           */
#define STY_MAT_PRINCIPLED 2 /* the reference's principled BSDF (svm/surface/principled.rs:118-330):
                             diffuse, dielectric reflection / transmission, a tinted specular layer
                             weighted by the ggx_dielectric_s albedo table, a conductor
                             (Gulbrandsen) and a clear coat; albedo = base colour, the
                             roughness / metallic / ior / transmission / specular / coat fields
                             below. Flat shading (normal maps are not supported). */
#define STY_MAT_GLASS 3      /* the reference's glass node (svm/surface/glass.rs:13-44, compiled from
                             the scene's "glass" node at svm/compiler.rs:249-263): rough dielectric
                             reflection + transmission, both tinted by albedo, added with the
                             Fresnel term of cos(wo) as the lobe-choice weight; reads `ior` and
                             `roughness` (alpha = max(roughness^2, 1e-4)). */

typedef struct sty_pf_material {
    int32_t kind;        /* STY_MAT_* */
    float albedo[3];
    float alpha;         /* GGX roughness alpha (>= 1e-4) */
    int32_t style[4];    /* style program per style index 0..3 (flags bits 1..3), -1 = none */
    /* STY_MAT_PRINCIPLED parameters (ignored by the other kinds) */
    float roughness, metallic, ior, transmission, specular_ior_level;
    float specular_tint[3];
    float coat_weight, coat_roughness, coat_ior;
    float coat_tint[3];
} sty_pf_material;

typedef struct sty_pf_vertices {
    const int32_t *active;      /* nonzero: the path has a vertex at this depth              */
    const float *p[3];          /* hit position                                              */
    const float *wo[3];         /* outgoing direction (towards the previous vertex)         */
    const float *ns[3];         /* shading normal                                            */
    const float *ng[3];         /* geometric normal                                          */
    const float *le[3];         /* emitted radiance at the vertex                            */
    const float *mis;           /* MIS weight of the emission (1 if not an emitter)          */
    const float *dir_wi[3];     /* NEE record: direction, stylised irradiance, light pdf     */
    const float *dir_l[3];
    const float *dir_pdf;       /*   (0 = no record)                                         */
    const float *ind_wi[3];     /* direction to the next vertex (-wo of it); 0 = no record   */
    const float *ind_mis;       /* that vertex's emission MIS weight (record.mis)            */
    const uint32_t *flags;      /* new_flags: bit0 disabled, bits1..3 use_style_2..4          */
    const uint32_t *material;   /* index into the material table                             */
    uint64_t n;
} sty_pf_vertices;

typedef struct sty_pf_ref_params {
    uint32_t depth;
    float radius;               /* world-space filter radius                                 */
    uint32_t reuse;             /* reservoir size (reuse[d])                                 */
    int32_t smis;
    int32_t cluster;
    int32_t disable_flag_check;
    int32_t no_first_hit_stylization;
    uint32_t table_size;        /* hash table size (the reference uses 2^26)                 */
    float pmin[3], pmax[3];     /* grid bounds (scene AABB or config scene_bounds)           */
    uint32_t max_cluster_rounds;/* cap on clustering rounds (STY_ERR_ITER_LIMIT beyond)      */
} sty_pf_ref_params;

typedef struct sty_pf_ref_ctx sty_pf_ref_ctx;

/* Create / destroy a reference-mode context owning the scratch for up to `max_vertices` path
 * slots (grid keys, sorted point lists, bucket ranges for `table_size` buckets, cluster state). */
STY_API sty_status sty_pf_ref_create(uint64_t max_vertices, uint32_t table_size, sty_pf_ref_ctx **out);
STY_API sty_status sty_pf_ref_destroy(sty_pf_ref_ctx *ctx);

/* One depth of the reference-mode filter. `in_next` (device, 3 planes of n floats) is the
 * styled result of the next depth for the same path slots (the record kernel_propagate copies,
 * :974-998; its pdf field is never read by the filter), NULL at the deepest depth. `rng` (device,
 * n Pcg32 states) is advanced by the reservoir draws.
 * `materials` (<= 256) and `programs` (<= 64) are HOST arrays, copied on the stream per call.
 * Outputs: `out` (device, 3 planes of n) = styled filtered radiance (0 for inactive slots);
 * optional `neighbours` (device, n) = neighbour count before the reservoir cap, `cluster_id`
 * (device, n; written only when params->cluster) = cluster centre slot (UINT32_MAX inactive). */
STY_API sty_status sty_pf_ref_filter(sty_pf_ref_ctx *ctx, const sty_pf_vertices *v, const float *in_next, const sty_pf_ref_params *params,
                                     const sty_pf_material *materials, uint32_t n_materials,
                                     const sty_style_program *programs, uint32_t n_programs,
                                     sty_pcg32 *rng, float *out, uint32_t *neighbours,
                                     uint32_t *cluster_id, void *stream);

/* ----------------------------------------------------------------------------------------
 * Adjoint of the screen-space NL-PF filter + smoothed ramp style node (one depth)
 *
 * Forward (as sty_pf_screen_filter_depth with a single STY_STYLE_RAMP_SMOOTH node applied at this
 * depth): f_i = sum_j w_ij in_j / sum_j w_ij, out_i = ramp(f_i); image = per-pixel mean over spp of
 * out (invalid records count as 0); loss = sum over pixels and channels of (image - target)^2.
 * Parameters (36 floats, this order): [0] sharpness s, [1..8] thresholds t_k, [9..32] colours
 * c_k (rgb), [33] sigma_pixel, [34] sigma_pos, [35] sigma_nrm. `n_steps` (1..8) ramp steps are used;
 * gradients of unused thresholds / colours are 0. The backward recomputes the neighbourhood
 * weights (two sweeps per query) instead of storing them.
 * `target` (device, width*height*3 floats, interleaved rgb); `grad` (device, 36 floats);
 * `loss_out` (host, optional; synchronises). `in_next` as in sty_pf_screen_filter_depth.
 * -------------------------------------------------------------------------------------- */
STY_API sty_status sty_pf_adjoint(const sty_pf_records *rec, uint32_t depth, int32_t radius, const float params[36],
                                  uint32_t n_steps, const float *in_next, const float *target, float *grad,
                                  float *loss_out, void *stream);

/* Allocation-free variant of sty_pf_adjoint (no counterpart in the reference). For callers that
 * cannot allocate device memory -- a host integrator whose device memory is owned and budgeted by
 * another runtime, or a render loop that must not fail on an allocation mid-frame -- the scratch
 * lives in one fixed device array of 4.31 MiB that every device holds from the library's first use
 * on it until the process exits. Same arguments and results as sty_pf_adjoint; limits: at most
 * 2^18 records per depth (width * height * spp), 2^16 pixels and 4096 32x8 tiles, larger inputs
 * are rejected with STY_ERR_ARG. It calls no cudaMalloc / cudaFree. Its first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device current, and looks
 * it up again if the device's context was replaced (cudaDeviceReset); make that first call before
 * any stream capture. A non-null loss_out is read back with a stream synchronisation, as in
 * sty_pf_adjoint. All calls share the one array, which keeps the last call's contents (every
 * region is fully written before it is read): calls whose work overlaps on the GPU (other
 * streams, other host threads) race and must be serialised by the caller. */
STY_API sty_status sty_pf_adjoint_noalloc(const sty_pf_records *rec, uint32_t depth, int32_t radius,
                                          const float params[36], uint32_t n_steps, const float *in_next,
                                          const float *target, float *grad, float *loss_out, void *stream);

/* ----------------------------------------------------------------------------------------
 * Neural radiance cache (NL-NRC): one-to-one with the reference's tiny-cuda-nn wrapper
 * (crates/akari_cpp_ext/cpp_ext/akari_nrc.h:1-17, akari_tcnn.cu:84-292).
 *
 * Network: frequency encoding of `input_dims` raw inputs (dim d gets freqs[d] pairs
 * sin(2^k pi x), cos(2^k pi x), k < freqs[d]; sum 2*freqs = 64), then `hidden_layers` ReLU layers
 * of width 64 and a linear output layer of `output_dims` (<= 16); no biases. Weights are FP32
 * masters; precision STY_NRC_BF16 runs the MLP on the tcgen05 tensor cores (BF16 operands, FP32
 * accumulation in TMEM), STY_NRC_FP32 runs it in FP32 on the CUDA cores.
 * Loss: relative L2, (pred - target)^2 / (pred^2 + 0.01) with pred treated as constant in the
 * denominator, averaged over the batch and channels. Optimiser: Adam (beta1, beta2, eps) with
 * learning rate lr * decay_base^(step / decay_interval) (tcnn ExponentialDecay, nrc_pt.rs:1199-1216);
 * inference uses EMA weights with the debiased update of akari_tcnn.cu:42-83.
 * Matrices are sample-major: input[i * input_dims + d], output[i * output_dims + c] (tcnn's
 * column-major [dims x count]). All pointers are device pointers unless stated.
 * -------------------------------------------------------------------------------------- */
#define STY_NRC_FP32 0
#define STY_NRC_BF16 1
#define STY_NRC_MAX_INPUTS 16

typedef struct sty_nrc_config {
    uint32_t input_dims;     /* raw input dims (<= 16) */
    uint32_t output_dims;    /* <= 16 */
    uint32_t batch_size;     /* training samples per step, multiple of 128 */
    uint32_t hidden_layers;  /* >= 1 (width fixed at 64) */
    uint32_t precision;      /* STY_NRC_FP32 or STY_NRC_BF16 */
    uint32_t freqs[STY_NRC_MAX_INPUTS];
    float learning_rate, beta1, beta2, epsilon;
    float ema_decay;
    float decay_base;
    uint32_t decay_interval;
    uint64_t seed;
} sty_nrc_config;

typedef struct sty_nrc sty_nrc;

STY_API sty_status sty_nrc_create(const sty_nrc_config *config, sty_nrc **out);       /* akr_create_nrc */

/* The reference's own NL-NRC network (akr_create_nrc with the tiny-cuda-nn JSON of nrc_pt.rs:
 * 1159-1352): a Composite encoding of `input_dims` = 20 + max_depth inputs in the
 * STY_NRC_ROWS_REF layout -- multiresolution hash grid on inputs 0..2 (`grid_levels` levels of
 * `grid_features` features, tables of at most 2^log2_table entries, base resolution
 * `base_resolution`, `per_level_scale` growth; the reference uses 22 x 4, 2^19, 16, 2.0),
 * one-blob (`blob_bins` bins) on the next `blob_dims` inputs (7 / 4), identity on the rest -- and
 * a ReLU MLP of `hidden_units` (128) x `hidden_layers` (5) without biases, linear output. BF16
 * GEMM operands (FP16 with STY_NRC_GRID_FP16, tiny-cuda-nn's precision, its backward scaled by
 * the loss scale 128) with FP32 accumulation on the tensor cores, FP32 master parameters (MLP
 * weights, then the tables), relative L2, Adam + exponential decay, EMA for inference. The
 * encoded width is at most 256. The handle works with every other
 * sty_nrc_* call; param_count covers the tables. Table gradients are accumulated with atomics,
 * so training on this network is not bit-deterministic. No counterpart of the encodings' exact
 * numerics exists here (tiny-cuda-nn is not vendored): they follow the published definitions.
 * The forward reads FP16 copies of the tables (as tiny-cuda-nn's half-precision forward does).
 * Inference runs on the tensor cores in two launches per chunk -- the encoding written as 128-row
 * MMA operand tiles, then one kernel running every layer on chip -- when hidden_units is 32, 64 or
 * 128, the encoded width is at most 160, the weights fit in shared memory (the reference's
 * 144 -> 128 x 5 -> 3 network does) and the operands are BF16; otherwise, or with
 * STY_NRC_GRID_LAYERED in `flags`, it runs the layer-by-layer path (one tensor-core GEMM per
 * layer, as training does). */
#define STY_NRC_GRID_LAYERED 1u
#define STY_NRC_GRID_FP16 2u
typedef struct sty_nrc_grid_config {
    uint32_t input_dims, output_dims, batch_size;
    uint32_t hidden_layers, hidden_units;
    uint32_t grid_levels, grid_features, log2_table, base_resolution;
    float per_level_scale;
    uint32_t blob_dims, blob_bins;
    float learning_rate, beta1, beta2, epsilon;
    float ema_decay;
    float decay_base;
    uint32_t decay_interval;
    uint32_t flags;        /* STY_NRC_GRID_* bits */
    uint64_t seed;
} sty_nrc_grid_config;
STY_API sty_status sty_nrc_create_grid(const sty_nrc_grid_config *config, sty_nrc **out);
STY_API sty_status sty_nrc_destroy(sty_nrc *nrc);                                      /* akr_destroy_nrc */
STY_API sty_status sty_nrc_param_count(sty_nrc *nrc, uint64_t *count);                 /* akr_nrc_param_count */
/* FP32 master weights to / from a HOST array of param_count floats (akr_nrc_save/load_params);
 * loading also resets the EMA copy to the loaded weights. Synchronous. */
STY_API sty_status sty_nrc_save_params(sty_nrc *nrc, float *host_params);
STY_API sty_status sty_nrc_load_params(sty_nrc *nrc, const float *host_params);
STY_API sty_status sty_nrc_set_learning_rate(sty_nrc *nrc, float lr);                  /* akr_nrc_set_learning_rate */
STY_API sty_status sty_nrc_get_learning_rate(sty_nrc *nrc, float *lr);                 /* akr_nrc_get_learning_rate */
STY_API sty_status sty_nrc_reset_optimizer(sty_nrc *nrc);                              /* akr_nrc_reset_optimizer */
/* Inference with the EMA weights (akr_nrc_inference) / the training weights
 * (akr_nrc_train_inference). Asynchronous on `stream`. */
STY_API sty_status sty_nrc_inference(sty_nrc *nrc, uint64_t count, const float *input, float *output, void *stream);
STY_API sty_status sty_nrc_train_inference(sty_nrc *nrc, uint64_t count, const float *input, float *output,
                                           void *stream);
/* n_iters training steps, each on batch_size samples drawn uniformly (Pcg32) from the `count`
 * rows of input/target (akr_nrc_train / collect_batch, akari_tcnn.cu:15-38,136-168). If loss_out is
 * non-NULL it receives the mean loss over the steps (synchronises the stream). */
STY_API sty_status sty_nrc_train(sty_nrc *nrc, uint64_t count, uint64_t n_iters, const float *input,
                                 const float *target, float *loss_out, void *stream);
/* Gradient of the batch loss w.r.t. the FP32 master weights for an explicit batch (rows
 * input[0..batch), no sampling, no optimiser step): `grad` (device, param_count floats). Used to
 * check the backward pass. */
STY_API sty_status sty_nrc_gradient(sty_nrc *nrc, uint32_t batch, const float *input, const float *target,
                                    float *grad, float *loss_out, void *stream);
/* Which tcgen05 kernel runs the BF16 training step of the 64-wide network (process-wide; every
 * later sty_nrc_train / sty_nrc_gradient call). Both give the same weight gradients bit for bit.
 * Returns STY_ERR_ARG for an unknown value.
 *   STY_NRC_TRAIN_KERNEL_AUTO       two 128-sample tiles in flight per SM (two epilogue warpgroups
 *                                   and an MMA-issuing warp) for networks of at most 5 hidden
 *                                   layers, one tile at a time for 6
 *   STY_NRC_TRAIN_KERNEL_ONE_TILE   one warpgroup per SM walking its tiles in sequence */
#define STY_NRC_TRAIN_KERNEL_AUTO 0
#define STY_NRC_TRAIN_KERNEL_ONE_TILE 1
STY_API sty_status sty_nrc_set_train_kernel(int32_t kernel);

/* ----------------------------------------------------------------------------------------
 * Scene, wavefront tracer and the end-to-end NL-PF render
 *
 * Replaces the reference's forward wavefront (kernel_mk_trace, lm_path_filtering.rs:1063-1218,
 * NEE sample_light :1261-1316, emitter MIS handle_surface_light :388-426) and its render driver
 * (:1319-1799), with its own BVH (binned SAH, built on the host) and a hand-written traversal
 * kernel instead of the LuisaCompute/OptiX accel. Intersection is the watertight ray/triangle test
 * of Woop, Benthin and Wald (2013) in explicitly rounded f32; equal distances resolve to the lowest
 * triangle id. Flat shading (shading normal = geometric normal).
 * -------------------------------------------------------------------------------------- */
typedef struct sty_scene_material {
    int32_t kind;        /* STY_MAT_* */
    float albedo[3];
    float alpha;         /* GGX alpha */
    float emission[3];   /* radiance leaving the front (geometric-normal) side; 0 = not a light */
    int32_t style[4];    /* style program per style index, -1 = none (applied by the filter) */
    int32_t set_style;   /* -1: hits keep the path's flags; k >= 0: hits set style index k (sty_set_idx) */
    /* STY_MAT_PRINCIPLED parameters (Blender's Principled BSDF inputs as the reference reads them;
     * ignored by the other kinds) */
    float roughness, metallic, ior, transmission, specular_ior_level;
    float specular_tint[3];
    float coat_weight, coat_roughness, coat_ior;
    float coat_tint[3];
} sty_scene_material;

/* The principled BSDF's pieces, for checking them against the oracle (shading frame: z = normal;
 * device arrays of n 3-vectors). sty_bsdf_eval: f * |cos_i| (rgb) and pdf of `material` for (wo, wi)
 * (Surface::evaluate). sty_bsdf_sample: SurfaceClosure::sample with u = (u_select, u0, u1) per
 * sample: wi, f * |cos_i| and pdf at wi (pdf 0 = invalid sample). sty_principled_table: the 16^3
 * ggx_dielectric_s albedo table of the current device (HOST output, x = roughness fastest, then
 * mu, then z = sqrt(|ior - 1| / (ior + 1))). */
STY_API sty_status sty_bsdf_eval(const sty_scene_material *material, uint64_t n, const float *wo, const float *wi,
                                 float *f, float *pdf, void *stream);
STY_API sty_status sty_bsdf_sample(const sty_scene_material *material, uint64_t n, const float *wo, const float *u,
                                   float *wi, float *f, float *pdf, void *stream);
STY_API sty_status sty_principled_table(float *host_table);

/* Pixel filters (PixelFilter, crates/akari_render/src/film.rs:20-48): the film-plane offset of a
 * camera ray from the sampler draw (u0, u1).
 *   STY_FILTER_BOX       (u - 0.5) * radius per axis
 *   STY_FILTER_GAUSSIAN  Box-Muller: sqrt(-2 ln u0) * (cos 2 pi u1, sin 2 pi u1) * radius / 3, each
 *                        axis clamped to [-radius, radius] (the reference's default, radius 1.5,
 *                        and the filter of every teaser config). */
#define STY_FILTER_BOX 0
#define STY_FILTER_GAUSSIAN 1

typedef struct sty_camera {
    float eye[3], target[3], up[3];
    float fov_y;         /* degrees */
    uint32_t width, height;
    float filter_radius; /* pixel filter radius in pixels */
    int32_t filter;      /* STY_FILTER_BOX or STY_FILTER_GAUSSIAN */
} sty_camera;

typedef struct sty_scene sty_scene;

/* Build a scene from HOST triangle soup: positions (9 floats per triangle: v0, v1, v2), one
 * material index per triangle, the material table and the camera. Builds the BVH on the host and
 * uploads everything. Replaces the reference's scene upload and acceleration-structure build
 * (crates/akari_render/src/load.rs:481-700, LuisaCompute's Accel): the mesh lights are the
 * triangles of emissive materials (load.rs:95-128). */
STY_API sty_status sty_scene_create(const float *tri_positions, const uint32_t *tri_material, uint32_t n_tris,
                                    const sty_scene_material *materials, uint32_t n_materials,
                                    const sty_camera *camera, sty_scene **out);
STY_API sty_status sty_scene_destroy(sty_scene *scene);
/* Closest hit of n rays (device, 8 floats per ray: origin, direction, tmin, tmax). Outputs
 * (device): prim (UINT32_MAX on a miss), t, bary (2 per ray: weights of v1 and v2). The ray query
 * the reference's integrators issue through LuisaCompute (`accel.intersect`), exposed for
 * checking the traversal against a brute-force closest hit. */
STY_API sty_status sty_scene_closest_hit(sty_scene *scene, const float *rays, uint64_t n, uint32_t *prim, float *t,
                                         float *bary, void *stream);

#define STY_PF_MODE_REF 0    /* the reference's world-space hash-grid filter (sty_pf_ref_filter) */
#define STY_PF_MODE_SCREEN 1 /* the screen-space bilateral filter (sty_pf_screen_filter) */

typedef struct sty_pf_render_config {
    uint32_t max_depth;             /* vertex depths 0..max_depth */
    uint32_t branch;                /* paths per pixel */
    uint32_t repeats;
    float radius_scale[16];         /* per depth; depths beyond n_radius_scale use the last entry */
    uint32_t n_radius_scale;
    uint32_t reuse[16];
    uint32_t n_reuse;
    int32_t smis, cluster, disable_flag_check, no_first_hit_stylization;
    int32_t has_scene_bounds;
    float scene_bounds[6];          /* min xyz, max xyz (else the scene AABB) */
    uint64_t seed;                  /* path slot i of pixel px and branch b (i = b * width * height + px)
                                       starts from Pcg32::new_seq_offset(i, seed_i), seed_i the i-th
                                       gen::<u64>() of StdRng::seed_from_u64(seed) (ChaCha12; the
                                       reference renders with seed 0, sampler/mod.rs:157-173) */
    int32_t mode;                   /* STY_PF_MODE_REF (0) or STY_PF_MODE_SCREEN */
    int32_t screen_style;           /* SCREEN: index into `programs` of the filter's style program
                                       (applied per depth by its nodes' depth masks), -1 = none */
    sty_pf_screen_params screen;    /* SCREEN: the bilateral filter's window and bandwidths */
} sty_pf_render_config;

/* Full NL-PF render (lm_path_filtering.rs:1629-1793): per repeat, trace every depth, filter the
 * depths backwards, splat the depth-0 result and add (1/repeats) of the pixel values into `film`
 * (device, width*height*3 doubles, interleaved rgb; the caller zeroes it). `programs` is a HOST
 * array. Optional `vertex_count` (host) receives the number of path vertices traced.
 *   STY_PF_MODE_REF: the reference-mode filter (sty_pf_ref_filter) at every depth; the splat
 *     applies each hit material's style program at the first hit (kernel_splat :480-506).
 *   STY_PF_MODE_SCREEN: the tracer writes every depth's vertices as screen-space records
 *     (sty_pf_records, spp = branch: pos = hit point, nrm = shading normal, rad = emitted radiance
 *     with its MIS weight + the light sample with balance MIS, thr = f |cos| / pdf of the sampled
 *     continuation times the MIS weight of the emission found there, valid = hit), and
 *     sty_pf_screen_filter filters them from max_depth down to 0 with `screen` and the program
 *     `screen_style`; the film receives the mean over the branch samples of the depth-0 output
 *     (sty_film_accumulate). branch must be 1, 2, 4, 8 or 16. */
STY_API sty_status sty_pf_render(sty_scene *scene, const sty_pf_render_config *config,
                                 const sty_style_program *programs, uint32_t n_programs, double *film,
                                 uint64_t *vertex_count, void *stream);

/* Writable record planes: each of the 13 planes holds (max_depth + 1) * height * width * branch
 * elements in the sty_pf_records order; `prim` (optional) receives the hit triangle id of each
 * record (UINT32_MAX where the record is invalid). */
typedef struct sty_pf_records_out {
    float *pos[3];
    float *nrm[3];
    float *rad[3];
    float *thr[3];
    int32_t *valid;
    uint32_t *prim;
} sty_pf_records_out;

/* The screen-space records of the first repeat of a STY_PF_MODE_SCREEN render of `config`
 * (device planes owned by the caller): sty_pf_render with repeats = 1 equals
 * sty_pf_screen_filter on these records followed by sty_film_accumulate, bit for bit. Lets a
 * caller dump the traced buffers the filter sees. */
STY_API sty_status sty_pf_trace_records(sty_scene *scene, const sty_pf_render_config *config,
                                        const sty_style_program *programs, uint32_t n_programs,
                                        const sty_pf_records_out *records, uint64_t *vertex_count, void *stream);

/* The depth-0 camera rays of every path slot of a render with `branch` paths per pixel and seed
 * `seed` (device output, 8 floats per slot: origin, direction, tmin = 0, tmax = 1e20; slot
 * i = b * width * height + px): PerspectiveCamera::generate_ray (camera/mod.rs:73-126) with the
 * scene camera's pixel filter, fed by the slot's Pcg32 stream exactly as sty_pf_render and
 * sty_nrc_render feed it. */
STY_API sty_status sty_scene_camera_rays(sty_scene *scene, uint32_t branch, uint64_t seed, float *rays, void *stream);

/* NL-NRC samples generated by the tracer (nrc_pt.rs:231-434 tracing, write_nrc_inputs :583-663,
 * training targets :723-776).
 * layout STY_NRC_ROWS_REF: rows of 20 + max_depth floats as the reference writes them: position
 *   normalised to the scene bounds (3), shading normal * 0.5 + 0.5 (3), outgoing direction * 0.5 +
 *   0.5 (3), roughness (1 for diffuse, alpha for GGX), albedo (3), [stylization disabled, enabled]
 *   (2), one-hot style index (4), one-hot depth (max_depth + 1).
 * layout STY_NRC_ROWS_SPHERICAL: rows of 11 floats for the frequency-encoded cache: normalised
 *   position (3), shading normal and outgoing direction as (theta / pi, (phi + pi) / 2pi)
 *   (xyz_to_spherical_normalized, geometry.rs:342-346; 2 + 2), roughness (1), albedo (3).
 * mode STY_NRC_SAMPLES_TRAIN: `spp` paths per pixel are traced to `max_depth`; every vertex gives
 *   one row whose target is that vertex's radiance estimate from the traced suffix (emission + NEE
 *   with MIS + BSDF-sampled continuation, the estimator of sty_pf_render with only the vertex itself
 *   reused; no style nodes). The reference instead bootstraps the suffix from the cache's own
 *   prediction at the next vertex; a traced suffix is its unbiased limit.
 * mode STY_NRC_SAMPLES_QUERY: the first hit of `spp` camera rays per pixel, row order
 *   sample-major (index = s * width * height + pixel), depth one-hot 0; rows of camera rays that
 *   miss are zeros and their target (the emission seen at the hit) is 0.
 * inputs / targets are device arrays of `capacity` rows; *count_out (host) receives the rows
 * written (training rows beyond the capacity are dropped). */
#define STY_NRC_SAMPLES_TRAIN 0
#define STY_NRC_SAMPLES_QUERY 1
#define STY_NRC_ROWS_REF 0
#define STY_NRC_ROWS_SPHERICAL 1
STY_API sty_status sty_nrc_samples(sty_scene *scene, uint32_t mode, uint32_t layout, uint32_t spp,
                                   uint32_t max_depth, uint64_t seed, float *inputs, float *targets,
                                   uint64_t capacity, uint64_t *count_out, void *stream);

/* The NL-NRC render (NRCPathTracer::render, nrc_pt.rs:1519-1690) on the scene and a cache made by
 * sty_nrc_create with 11 inputs (rows in STY_NRC_ROWS_SPHERICAL) or by sty_nrc_create_grid with
 * 20 + max_depth inputs (rows in STY_NRC_ROWS_REF, the reference's own network).
 * Training, `training_iters` times: `training_paths` paths (0: batches_per_iter x the cache's batch
 * size / (max_depth + 1), clamped to the pixel count, :1126-1128), each from a pixel drawn from its
 * own Pcg32 stream (:1394), traced to max_depth; the cache (training weights) predicts the
 * radiance leaving every vertex of depth >= 1 (:667-703); each vertex of depth >= training_level
 * gets the target Le + NEE (balance MIS) + f * L_next * mis_next / pdf with L_next the prediction
 * at the next vertex, styled at that depth unless learn_stylized_radiance (:704-842); then
 * sty_nrc_train(rows, batches_per_iter). With per_level_training > 0 the training level starts at
 * max_depth and drops by one every per_level_training iterations (:1538-1545), else it is 0.
 * Rendering, `repeats` times, added with weight 1/repeats to `film` (device, width*height*3
 * doubles, rgb; the caller zeroes it):
 *   final_gather == 0: one first hit per pixel, the cache's EMA prediction there, styled at depth 0
 *     unless no_first_hit_stylization (:844-965);
 *   final_gather > 0: each pixel's path continues through vertices of roughness <= 0.05 up to
 *     max_depth and splits at the first rougher one (:372-375); final_gather times, the split
 *     vertex takes another light sample and one BSDF-sampled ray whose hit the EMA cache predicts
 *     (styled at that depth) (:436-582, 877-965); the split vertex's radiance is Le +
 *     direct / (n + 1) + indirect / n, propagated to the camera with the style node at every
 *     depth (:969-1047). Paths that never split are path traced without the cache.
 * `programs` is a HOST array.
 * Calls on one scene are serialised by the caller (the scene keeps the render's buffers).
 * Reference flags are taken after the vertex's own set_style update (as in sty_pf_render). */
typedef struct sty_nrc_render_config {
    uint32_t max_depth;
    uint32_t training_iters;
    uint32_t batches_per_iter;
    uint32_t training_paths;
    uint32_t repeats;
    uint32_t per_level_training;
    int32_t no_first_hit_stylization;
    int32_t learn_stylized_radiance;
    uint32_t final_gather;
    uint32_t reserved;
    uint64_t seed;
} sty_nrc_render_config;
typedef struct sty_nrc_render_stats {
    uint64_t training_rows;      /* training rows over all iterations */
    uint64_t inference_queries;  /* cache queries over training and rendering */
    float last_loss;             /* mean loss of the last training call */
    uint32_t reserved;
} sty_nrc_render_stats;
STY_API sty_status sty_nrc_render(sty_scene *scene, sty_nrc *nrc, const sty_nrc_render_config *config,
                                  const sty_style_program *programs, uint32_t n_programs, double *film,
                                  sty_nrc_render_stats *stats, void *stream);

/* NL-PF and NL-NRC together: NL-PF's screen-space filter over the first `cache_depth` bounces, the
 * neural radiance cache for the rest of the path. First the cache is trained by the NL-NRC
 * training loop of `nrc` (sty_nrc_render's training iterations: nrc.training_iters,
 * batches_per_iter, training_paths, per_level_training, learn_stylized_radiance, seed, max_depth;
 * its rendering fields are not used). Then, `pf.repeats` times, the paths of a STY_PF_MODE_SCREEN
 * render of `pf` (branch paths per pixel, pf.seed) are traced to depth K = cache_depth; at every
 * depth-K vertex the cache's EMA prediction, styled at depth K (unless the cache learns styled
 * radiance), is the radiance leaving the vertex (out_K, as the cache's prediction stands in for the
 * traced continuation in nrc_pt.rs:723-776); sty_pf_screen_filter_depth filters depths K - 1 .. 0
 * (each depth's input rad + thr * out of the depth below) and the film receives (1 / pf.repeats) of
 * the pixel means of out_0. pf.max_depth is not used; the cache's rows are those of
 * sty_nrc_render (11 inputs, or 20 + nrc.max_depth), and 1 <= cache_depth <= nrc.max_depth. */
typedef struct sty_pf_nrc_config {
    sty_pf_render_config pf;     /* mode STY_PF_MODE_SCREEN: branch, repeats, seed, screen, screen_style */
    sty_nrc_render_config nrc;   /* the cache's training loop */
    uint32_t cache_depth;
    uint32_t reserved;
} sty_pf_nrc_config;
STY_API sty_status sty_pf_nrc_render(sty_scene *scene, sty_nrc *nrc, const sty_pf_nrc_config *config,
                                     const sty_style_program *programs, uint32_t n_programs, double *film,
                                     sty_nrc_render_stats *stats, void *stream);

/* Branching path tracer (crates/akari_integrator/src/branching_pt.rs, Config :77-100): the paper's
 * BrPT baseline, and with inner_samples = {1} the plain stylized path tracer of
 * configs/teaser/pt.json. Per pixel a tree of vertices: the k-th rough vertex (average roughness
 * > 0.01) of a path takes inner_samples[k] branches (1 beyond n_levels, 1 at smooth vertices, none
 * at max_depth), each one light sample + one BSDF-sampled child; bottom-up a vertex's radiance is
 * style(Le + mean over branches of (direct + throughput * child radiance * child emission MIS)),
 * the depth-0 radiance is the pixel sample (the non-debiased estimator; the jackknife / Russian-
 * roulette debiasing option is not built). Pixel samples (pixel x repeat) go through in passes
 * whose worst-case vertex trees fit vram_mb (100 bytes per vertex slot). Adds (1/repeats) of each pixel's sample into
 * `film` (device, width*height*3 doubles; the caller zeroes it). `programs` is a HOST array.
 * Sampling keys on (seed, repeat, pixel) and, per child, on (parent, branch index): the image does
 * not depend on vram_mb. Deterministic. */
#define STY_BRPT_MAX_LEVELS 8
typedef struct sty_brpt_config {
    uint32_t max_depth;                          /* Config::max_depth (reference default 7) */
    uint32_t n_levels;                           /* entries of inner_samples used, 1..8 */
    uint32_t inner_samples[STY_BRPT_MAX_LEVELS]; /* Config::inner_samples (default 256, 32, 8, 1) */
    uint32_t repeats;                            /* Config::repeats */
    uint32_t vram_mb;                            /* Config::vram: vertex-tree budget per pass, MB */
    uint64_t seed;
    uint32_t first_repeat; /* this call renders repeats first_repeat .. first_repeat + repeats - 1 of the
                              seed's sample sequence (0 for a whole render): replicas that split the
                              repeats of one render produce films whose repeat-weighted sum is that
                              render's film */
    uint32_t reserved;     /* 0 */
} sty_brpt_config;
typedef struct sty_brpt_stats {
    uint64_t vertices;        /* surface hits (tree vertices) over all passes and repeats */
    uint64_t slots;           /* vertex slots (hits + branches whose ray missed) */
    uint64_t passes;          /* pixel passes over all repeats */
    uint64_t pixels_per_pass; /* pixel samples (pixel x repeat) per pass */
    uint64_t max_pass_slots;
} sty_brpt_stats;
STY_API sty_status sty_brpt_render(sty_scene *scene, const sty_brpt_config *config,
                                   const sty_style_program *programs, uint32_t n_programs, double *film,
                                   sty_brpt_stats *stats, void *stream);

/* ----------------------------------------------------------------------------------------
 * Integer helpers (bit-exact with the reference)
 * -------------------------------------------------------------------------------------- */
/* Pcg32::new_seq_offset (sampler/mod.rs:94-100) for seq = first_seq + i, seed = seeds[i]
 * (device arrays of n), then `draws` calls of gen_u32 per stream written to out (device,
 * n * draws, stream-major) and the final states to states (device, n). */
STY_API sty_status sty_pcg32_streams(const uint64_t *seeds, uint64_t first_seq, uint64_t n,
                             uint32_t draws, uint32_t *out, sty_pcg32 *states, void *stream);

/* The gen::<u64>() outputs first .. first + n - 1 of rand's StdRng::seed_from_u64(seed) (rand 0.8.5:
 * ChaCha12Rng of rand_chacha 0.3.1 keyed by rand_core 0.6.4's PCG32 expansion of the seed), the
 * per-path seeds of init_pcg32_buffer_with_seed (sampler/mod.rs:157-173); device output. */
STY_API sty_status sty_std_rng_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t *out, void *stream);

/* Hash-grid cell index of each point (lm_path_filtering.rs:20-59): cell = clamp((p - pmin) /
 * (pmax - pmin), 0, 1) * res truncated and clamped to res-1; index = (x*73856093 ^ y*19349663
 * ^ z*83492791) mod table_size in 64-bit. `points` is device xyz-interleaved, n points. */
STY_API sty_status sty_hash_cells(const float *points, uint64_t n, const float pmin[3],
                          const float pmax[3], const uint32_t res[3], uint32_t table_size,
                          uint32_t *cell_xyz, uint32_t *cell_index, void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* STY_GB300_H */
