// scene.cuh -- device view of a scene: BVH2 nodes, triangles, materials; watertight intersection.
#pragma once

#include "common.cuh"

namespace sty {

struct BvhNode {        // 32 bytes
    float bmin[3];
    uint32_t a;         // internal: left child (right = a + 1); leaf: first triangle slot
    float bmax[3];
    uint32_t count;     // 0 = internal, else number of triangles in the leaf
};

struct TriGeom {        // 48 bytes, triangle slot order (BVH leaf order)
    float4 v0;          // w = original triangle id (as bits)
    float4 v1;
    float4 v2;
};

struct SceneView {
    const BvhNode *nodes;
    const TriGeom *tris;            // slot order
    const uint32_t *tri_material;   // by original id
    const float *tri_normal;        // by original id, 3 per triangle (unit geometric normal)
    const float *tri_area;          // by original id
    const sty_scene_material *materials;
    uint32_t n_tris, n_materials;
    // emitters: triangles with non-zero emission, sampled by area x luminance (CDF)
    const uint32_t *light_tris;     // original ids
    const float *light_cdf;         // n_lights + 1 entries, cdf[0] = 0, cdf[n] = 1
    uint32_t n_lights;
    const float *tri_pos;           // by original id, 9 per triangle
    const float *ggx_tab;           // the principled BSDF's albedo table (bsdf.cuh)
    uint32_t any_closure;           // some material is STY_MAT_PRINCIPLED / STY_MAT_GLASS
};

struct Hit {
    float t, b1, b2;
    uint32_t prim;  // original id, 0xffffffff = miss
};

// Watertight ray/triangle intersection (Woop, Benthin, Wald 2013) in explicitly rounded f32 with the
// double-precision fallback when an edge function is exactly zero. Returns true and updates *hit
// when the triangle is hit in (tmin, hit->t) or at hit->t with a lower id.
struct RayPre {
    float o[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float tmin;
};
__host__ __device__ inline RayPre ray_pre(const float o[3], const float d[3], float tmin) {
    RayPre r;
    for (int a = 0; a < 3; a++) r.o[a] = o[a];
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
#ifdef __CUDA_ARCH__
    r.Sx = __fdiv_rn(d[kx], d[kz]);
    r.Sy = __fdiv_rn(d[ky], d[kz]);
    r.Sz = __fdiv_rn(1.0f, d[kz]);
#else
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
#endif
    r.tmin = tmin;
    return r;
}

#ifdef __CUDA_ARCH__
#define STY_FM(a, b) __fmul_rn(a, b)
#define STY_FS(a, b) __fsub_rn(a, b)
#define STY_FA(a, b) __fadd_rn(a, b)
#define STY_FD(a, b) __fdiv_rn(a, b)
#define STY_DFMS(a, b, c, d) __dsub_rn(__dmul_rn(a, b), __dmul_rn(c, d))
#else
#define STY_DFMS(a, b, c, d) ((a) * (b) - (c) * (d))
#define STY_FM(a, b) ((a) * (b))
#define STY_FS(a, b) ((a) - (b))
#define STY_FA(a, b) ((a) + (b))
#define STY_FD(a, b) ((a) / (b))
#endif

__host__ __device__ inline bool intersect_tri(const RayPre &r, const float v0[3], const float v1[3], const float v2[3],
                                              uint32_t prim, Hit *hit) {
    const float A[3] = {STY_FS(v0[0], r.o[0]), STY_FS(v0[1], r.o[1]), STY_FS(v0[2], r.o[2])};
    const float B[3] = {STY_FS(v1[0], r.o[0]), STY_FS(v1[1], r.o[1]), STY_FS(v1[2], r.o[2])};
    const float C[3] = {STY_FS(v2[0], r.o[0]), STY_FS(v2[1], r.o[1]), STY_FS(v2[2], r.o[2])};
    const float Ax = STY_FS(A[r.kx], STY_FM(r.Sx, A[r.kz])), Ay = STY_FS(A[r.ky], STY_FM(r.Sy, A[r.kz]));
    const float Bx = STY_FS(B[r.kx], STY_FM(r.Sx, B[r.kz])), By = STY_FS(B[r.ky], STY_FM(r.Sy, B[r.kz]));
    const float Cx = STY_FS(C[r.kx], STY_FM(r.Sx, C[r.kz])), Cy = STY_FS(C[r.ky], STY_FM(r.Sy, C[r.kz]));
    float U = STY_FS(STY_FM(Cx, By), STY_FM(Cy, Bx));
    float V = STY_FS(STY_FM(Ax, Cy), STY_FM(Ay, Cx));
    float W = STY_FS(STY_FM(Bx, Ay), STY_FM(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {  // fall back to double on exact zeros
        U = (float)STY_DFMS((double)Cx, (double)By, (double)Cy, (double)Bx);
        V = (float)STY_DFMS((double)Ax, (double)Cy, (double)Ay, (double)Cx);
        W = (float)STY_DFMS((double)Bx, (double)Ay, (double)By, (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = STY_FA(STY_FA(U, V), W);
    if (det == 0.0f) return false;
    const float Az = STY_FM(r.Sz, A[r.kz]), Bz = STY_FM(r.Sz, B[r.kz]), Cz = STY_FM(r.Sz, C[r.kz]);
    const float T = STY_FA(STY_FA(STY_FM(U, Az), STY_FM(V, Bz)), STY_FM(W, Cz));
    const float t = STY_FD(T, det);
    if (!(t > r.tmin)) return false;
    if (t > hit->t || (t == hit->t && prim >= hit->prim)) return false;
    hit->t = t;
    hit->b1 = STY_FD(V, det);
    hit->b2 = STY_FD(W, det);
    hit->prim = prim;
    return true;
}

__device__ inline bool box_hit(const BvhNode &n, const float o[3], const float inv[3], float tmin, float tmax,
                               float *tnear) {
    float t0 = tmin, t1 = tmax;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float ta = (n.bmin[a] - o[a]) * inv[a], tb = (n.bmax[a] - o[a]) * inv[a];
        if (ta > tb) {
            const float x = ta;
            ta = tb;
            tb = x;
        }
        tb *= 1.0f + 2.0f * 1.1920929e-07f * 2.0f;  // conservative (robust BVH traversal, Ize 2013)
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
    }
    *tnear = t0;
    return t0 <= t1;
}

// Closest hit in (tmin, tmax]; `exclude` = original id skipped (the triangle the ray leaves).
__device__ inline Hit trace_closest(const SceneView &s, const float o[3], const float d[3], float tmin, float tmax,
                                    uint32_t exclude) {
    Hit h;
    h.t = tmax;
    h.prim = 0xffffffffu;
    h.b1 = h.b2 = 0.0f;
    const RayPre rp = ray_pre(o, d, tmin);
    const float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode n = s.nodes[stack[--sp]];
        float tn;
        // cull against a slightly inflated best distance: a flat leaf box's entry can round one ulp
        // past a triangle hit at exactly the best distance (a tie on a shared edge), and the lower id
        // must still be found
        const float tcull = h.t * (1.0f + 1e-6f);
        if (!box_hit(n, o, inv, tmin, tcull, &tn)) continue;
        if (n.count) {
            for (uint32_t k = 0; k < n.count; k++) {
                const TriGeom tg = s.tris[n.a + k];
                const uint32_t id = __float_as_uint(tg.v0.w);
                if (id == exclude) continue;
                const float a0[3] = {tg.v0.x, tg.v0.y, tg.v0.z}, a1[3] = {tg.v1.x, tg.v1.y, tg.v1.z},
                            a2[3] = {tg.v2.x, tg.v2.y, tg.v2.z};
                intersect_tri(rp, a0, a1, a2, id, &h);
            }
        } else if (sp < 62) {
            // push far child first so the near one is popped first
            const BvhNode &l = s.nodes[n.a], &r = s.nodes[n.a + 1];
            float tl, tr;
            const bool hl = box_hit(l, o, inv, tmin, tcull, &tl), hr = box_hit(r, o, inv, tmin, tcull, &tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp++] = n.a + 1;
                    stack[sp++] = n.a;
                } else {
                    stack[sp++] = n.a;
                    stack[sp++] = n.a + 1;
                }
            } else if (hl) {
                stack[sp++] = n.a;
            } else if (hr) {
                stack[sp++] = n.a + 1;
            }
        }
    }
    return h;
}

// Any hit in (tmin, tmax) skipping two triangles (shadow rays).
__device__ inline bool trace_any(const SceneView &s, const float o[3], const float d[3], float tmin, float tmax,
                                 uint32_t ex0, uint32_t ex1) {
    Hit h;
    h.t = tmax;
    h.prim = 0xffffffffu;
    const RayPre rp = ray_pre(o, d, tmin);
    const float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode n = s.nodes[stack[--sp]];
        float tn;
        if (!box_hit(n, o, inv, tmin, tmax, &tn)) continue;
        if (n.count) {
            for (uint32_t k = 0; k < n.count; k++) {
                const TriGeom tg = s.tris[n.a + k];
                const uint32_t id = __float_as_uint(tg.v0.w);
                if (id == ex0 || id == ex1) continue;
                const float a0[3] = {tg.v0.x, tg.v0.y, tg.v0.z}, a1[3] = {tg.v1.x, tg.v1.y, tg.v1.z},
                            a2[3] = {tg.v2.x, tg.v2.y, tg.v2.z};
                if (intersect_tri(rp, a0, a1, a2, id, &h)) return true;
            }
        } else if (sp < 62) {
            stack[sp++] = n.a;
            stack[sp++] = n.a + 1;
        }
    }
    return false;
}

SceneView scene_view(const sty_scene *s);
// device buffers kept by a scene between renders (defined in trace.cu)
void render_cache_free(void *cache);

}  // namespace sty
