/*
 * oracle.h — CPU oracle for the light-transport hot path. TEST
 * INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's CPU
 * baseline call it as the checker; the library never links or calls it.
 *
 * Parity is unpinned: the reference (`arukas`, src/lib.rs) ships no
 * implementation, no tests and no golden images, so nothing here is checked
 * against reference outputs. What is pinned are the reference's data facts
 * (tests/golden/reference_facts.json) and published algorithms:
 *   - watertight ray/triangle test, Woop, Benthin, Wald, JCGT 2(1) 2013
 *   - robust slab test, Ize, JCGT 2(2) 2013
 *   - GGX / Smith (Walter et al. EGSR 2007), VNDF (Heitz JCGT 7(4) 2018),
 *     Schlick Fresnel, power-heuristic MIS (Veach 1997)
 *   - PCG32 (O'Neill 2014), SplitMix64 (Steele et al. 2014)
 * Scene semantics follow scenes/cbox.json:1-628 (camera 516-543, Principled
 * 3-62, Point lights 544-561), CornellBox-Original.mtl:80-87 (quad light) and
 * scenes/integrator.json:5 (max_depth).
 *
 * Scene layout structures (aqua_material, aqua_light, aqua_camera) come from
 * include/aqua.h, the data contract both sides read.
 */
#ifndef AQUA_ORACLE_H
#define AQUA_ORACLE_H

#include <stdint.h>

#include "../include/aqua.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene {
    const float* nodes;        /* four-wide BVH, 32 floats per node     */
    int32_t n_nodes;
    const int32_t* tri_order;  /* leaf order -> scene triangle          */
    const float* verts;        /* 9 floats per triangle, scene order    */
    const float* uvs;          /* 6 floats per triangle                 */
    const int32_t* tri_mat;
    const int32_t* tri_light;
    int32_t n_tris;
    const aqua_material* mats;
    int32_t n_mats;
    const aqua_light* lights;
    int32_t n_lights;
    const uint8_t* const* tex_rgba; /* n_tex pointers, sRGB RGBA8    */
    const int32_t* tex_w;
    const int32_t* tex_h;
    int32_t n_tex;
    aqua_camera cam;
    float env[3];
    const float* nrm;          /* 9 floats per triangle (vertex normals),
                                  scene order, or NULL: flat shading      */
    const float* qnodes;       /* the quantized copy of the BVH, 16 floats
                                  per node, when the device walks it (the
                                  FP32 walk then decodes it as the device
                                  does), else NULL                        */
} orc_scene;

/* FP32 traversal of the flattened BVH with the same node order, slab test
 * and triangle arithmetic as the device kernels. rays: 8 floats per ray;
 * hits: 4 floats (t, u, v, prim bits) per ray; counts: per-ray node visits
 * and triangle tests (2 uint32 per ray), may be NULL. */
void orc_trace_bvh_f32(const orc_scene* s, const float* rays, int64_t n, int any_hit, float* hits,
                       uint32_t* counts, int threads);
/* FP32 watertight test against every triangle; min (t, prim). */
void orc_trace_brute_f32(const orc_scene* s, const float* rays, int64_t n, int any_hit, float* hits, int threads);
/* FP64 watertight test against every triangle; hits: 4 doubles per ray. */
void orc_trace_brute_f64(const orc_scene* s, const float* rays, int64_t n, double* hits, int threads);

/* Path tracer with the device's estimator and random-number use, in
 * double (precision 64) or float (precision 32). Renders pixels
 * [pixel_begin, pixel_end) into out (width*height*3 floats, mean of spp).
 * stats: [paths, extension rays, shadow rays]. Returns 0 on success. */
int orc_render(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
               int32_t rr_depth, uint64_t seed, int threads, int64_t pixel_begin, int64_t pixel_end,
               float* out, double* stats);

/* As orc_render, for an arbitrary set of pixels: pixels[k] (each below
 * width*height) is rendered into out[3k..3k+2]. Returns 1 on a bad index. */
int orc_render_pixels(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
                      int32_t rr_depth, uint64_t seed, int threads, const uint32_t* pixels, int64_t n, float* out,
                      double* stats);

/* As orc_render, with a constant radiance cache: every path stops at bounce
 * query_depth (0 = first hit) and adds throughput x cache_rgb there;
 * query_depth -2 queries by the path-spread rule instead (the device's
 * AQUA_NRC_QUERY_SPREAD: from bounce 1 on, where spread^2 > 0.01 a0). */
int orc_render_cached(const orc_scene* s, int precision, int32_t spp, int32_t spp_offset, int32_t max_depth,
                      int32_t rr_depth, uint64_t seed, int threads, int64_t pixel_begin, int64_t pixel_end,
                      int32_t query_depth, const float* cache_rgb, float* out, double* stats);

/* Radiance-cache network (64 -> 5 x 64 ReLU -> 3, no biases; weights FP32
 * row-major [out][in], W1..W5 then W6: 20,672 values), in double.
 * emulate_bf16 = 1 rounds weights, inputs, stored activations and stored
 * gradients to bfloat16 (round to nearest even) where the device kernels
 * store them, so the only remaining difference is accumulation order.
 * x: n x 64 floats. out: n x 3. */
void orc_mlp_forward(const float* w, const float* x, int64_t n, int emulate_bf16, float* out);
void orc_mlp_forward_f64(const float* w, const float* x, int64_t n, int emulate_bf16, double* out);
/* Gradient of the mean relative L2 loss, mean over n x 3 of
 * (y - t)^2 / (y^2 + 0.01) with the denominator held constant (Mueller et al.
 * 2021), w.r.t. every weight; loss = that mean. */
void orc_mlp_grad(const float* w, const float* x, const float* target, int64_t n, int emulate_bf16,
                  double* grad, double* loss);
/* Input encoding of raw vertex features (16 floats each) to 64 floats. */
void orc_nrc_encode(const float* raw, int64_t n, const float* bmin, const float* bmax, float* x);

/* The Principled BSDF of the path tracer in double precision, in the local
 * shading frame (z = normal, wo.z > 0): f (3 values, not times cos) and the
 * sampling pdf (solid angle) for n direction pairs, and n sampled
 * directions from n triples of uniform numbers (wi.z < 0: refraction,
 * wi.z == 0: no sample). front = wo on the side of the winding normal. */
void orc_bsdf_eval(const aqua_material* m, int front, const double* wo, const double* wi, int64_t n, double* f,
                   double* pdf);
void orc_bsdf_sample(const aqua_material* m, int front, const double* wo, const double* u, int64_t n, double* wi);

/* Reference values the tests print. */
double orc_srgb_to_linear(double c);
uint32_t orc_pcg32_first(uint64_t initstate, uint64_t initseq, uint32_t* out, int n);

#ifdef __cplusplus
}
#endif

#endif
