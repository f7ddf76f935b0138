/*
 * pt_oracle.h -- C-ABI of the CPU oracle for the path-tracing-with-MIS path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of
 * PupilOptixLab's integrator (example/path_tracer/main.cu:38-246) and of the
 * render-layer math it calls (framework/render/..., framework/optix/util.h,
 * framework/cuda/random.h).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  The product library
 * never links, loads or calls it.
 *
 * It consumes the same scene descriptor as the product (include/pt_api.h),
 * so both sides see identical inputs.  Every buffer here is a HOST buffer.
 */
#ifndef PT_ORACLE_H_
#define PT_ORACLE_H_

#include "../include/pt_api.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene oracle_scene;

/* build_bvh: 0 = brute force only, 1 = also build the host binned-SAH BVH2. */
int oracle_scene_create(const pt_scene_desc *desc, int build_bvh, oracle_scene **out);
void oracle_scene_destroy(oracle_scene *scene);
int oracle_scene_num_prims(const oracle_scene *scene, uint32_t *num_triangles, uint32_t *num_spheres);
/* Curve segments of all curve instances and the round-cone pieces (primitives) they became. */
int oracle_scene_num_curves(const oracle_scene *scene, uint32_t *segments, uint32_t *pieces);
/* Piece table, 12 floats per piece: c0 xyz, r0, c1 xyz, r1, u0, u1, kind bits, segment. */
int oracle_scene_curve_pieces(const oracle_scene *scene, float *out);
/* Curve evaluation KAT: ctrl n*16 (4 control points xyzw), u n, ps n*3;
 * out n*15 = position4, velocity4, acceleration3, normal3, 0. */
int oracle_curve(uint32_t type, const float *ctrl, const float *u, const float *ps, float *out, uint32_t n);
/* World-space triangle vertices in primitive order: n_tri * 9 floats. */
int oracle_scene_world_triangles(const oracle_scene *scene, float *out);

/* Same ray / hit layout as pt_trace_rays. */
int oracle_trace_rays(const oracle_scene *scene, const float *rays, float *hits, uint32_t n,
                      int anyhit, int brute_force, int threads);

/* Camera rays of frame `seed` for all pixels (row-major, pixel = y*w + x):
 * out n_pixels * 8 floats in the pt_trace_rays ray layout (tmin 0.001, tmax 1e16). */
int oracle_camera_rays(const oracle_scene *scene, uint32_t rng_mode, uint32_t seed, float *out);

/* Full render, semantics of pt_render.  Buffers are host arrays of w*h
 * pixels (accum/frame float4, albedo/normal float3, test float; any may be
 * NULL except accum).  pixels / num_pixels optionally restrict the render to
 * a subset of pixel indices (NULL = all).  threads <= 0 uses all cores. */
int oracle_render(const oracle_scene *scene, const pt_render_params *params,
                  float *accum, float *frame, float *albedo, float *normal, float *test,
                  const uint32_t *pixels, uint32_t num_pixels, int threads);

/* Per-sample radiance (no accumulation) for one frame: out num_pixels * 3. */
int oracle_render_samples(const oracle_scene *scene, const pt_render_params *params, uint32_t frame_seed,
                          const uint32_t *pixels, uint32_t num_pixels, float *out_radiance, int threads);

/* Local BSDF batches, same layout as pt_bsdf_eval_batch / pt_bsdf_sample_batch. */
int oracle_bsdf_eval(const float *bsdf, const float *wo, const float *wi,
                     float *out_f, float *out_pdf, uint32_t n);
int oracle_bsdf_sample(const float *bsdf, const float *wo, uint32_t *rng_state,
                       float *out_wi, float *out_f, float *out_pdf, uint32_t *out_type, uint32_t n);
/* Local BSDF record of material m at texture coordinate uv (16 floats). */
int oracle_material_local_bsdf(const pt_material_desc *mat, float u, float v, float *out16);

/* Random streams: n draws of the stream of (pixel, seed). */
int oracle_rng_stream(uint32_t mode, uint32_t pixel, uint32_t seed, uint32_t n, float *out);
/* Raw 32-bit PCG32 outputs for (initstate, initseq). */
int oracle_pcg32_raw(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t *out);

/* Emitter KAT: sample emitter `index` of the scene's area/env table from a
 * shading point.  in: n * 8 floats (pos xyz, normal xyz, xi0, xi1);
 * out: n * 12 floats (radiance xyz, wi xyz, pdf, distance, pos xyz, valid). */
int oracle_emitter_sample(const oracle_scene *scene, int index, const float *in, float *out, uint32_t n);
/* Emitter table summary: count, then per emitter (type, select_probability). */
int oracle_emitter_table(const oracle_scene *scene, uint32_t *count, float *out_type_prob, uint32_t cap);

/* Known-answer entry points with the layouts of oracle/ref_kat.cpp. */
int oracle_fresnel_dielectric(const float *in, float *out, uint32_t n);
int oracle_fresnel_conductor(const float *in, float *out, uint32_t n);
int oracle_fresnel_diffuse(const float *eta, float *out, uint32_t n);
int oracle_ggx(const float *in, float *out, uint32_t n);
int oracle_sampling(const float *in, float *out, uint32_t n);
int oracle_emitter_sample_raw(int kind, const float *params, const float *in, float *out, uint32_t n);
int oracle_envmap(int mode, const float *pixels, uint32_t w, uint32_t h, float scale, const float *tw, const float *tl,
                  const float *in, float *out, uint32_t n, float *tables);
int oracle_select_emitter(const float *probs, uint32_t num, int has_env, const float *p, int32_t *out, uint32_t n);

int oracle_camera_make(float fov_y_deg, float aspect, float near_clip, float far_clip,
                       const float to_world[16], pt_camera_desc *out);

/* the shared trigonometry: fn 0 sin(x), 1 cos(x), 2 atan2(y, x), 3 acos(x) */
int oracle_trig(uint32_t fn, const float *x, const float *y, float *out, uint32_t n);

#ifdef __cplusplus
}
#endif

#endif
