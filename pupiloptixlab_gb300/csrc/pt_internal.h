// pt_internal.h -- host-side state shared by the translation units of
// libpt_gb300.so.  Not part of the public C-ABI (include/pt_api.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pt_api.h"
#include "pt_curve.h"
#include "pt_device.cuh"

// Thread-local last error (pt_last_error).
void pt_set_error(const char *fmt, ...);
#define PT_CUDA_TRY(expr)                                                                           \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            pt_set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;                      \
        }                                                                                           \
    } while (0)

// Device allocation owned by the scene; freed with cudaFree.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);  // grow (no copy) to at least n bytes
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

struct BatchWorkspace;  // pt_render_batch state (pt_render.cu)
void pt_batch_release(BatchWorkspace *b);

struct pt_context {
    int device = 0;
    int num_sms = 0;
    int max_smem_per_block = 0;
    BatchWorkspace *batch = nullptr;
    ~pt_context() { pt_batch_release(batch); }
};

struct MeshInstanceRef {  // where the world vertices of one mesh instance live
    uint32_t instance;
    uint32_t mesh;
    uint32_t vertex_offset;
    uint32_t prim_offset;
    float to_world[16];
};

// One emissive instance, kept so that the emitter table can be rebuilt after
// vertex updates (instance order = emitter order).
struct EmitterSource {
    bool sphere = false;
    float radiance[3] = {0, 0, 0};  // constant radiance (tex < 0)
    int32_t tex = -1;               // textured radiance: index into the scene's emitter textures
    float weight = 0.f;             // GetWeight of the radiance (world/emitter.cpp:77-101)
    std::vector<float> uvs;         // mesh: object texture coordinates, 2 per vertex (empty: none)
    uint32_t vertex_offset = 0;     // mesh: first world vertex of the instance
    std::vector<uint32_t> indices;  // mesh: object-space triangle indices
    std::vector<float> normals;     // mesh: object-space vertex normals (empty: geometric)
    float nm[9] = {0};              // mesh: normal matrix
    float center[3] = {0, 0, 0};    // sphere: world centre
    float radius = 0.f;
};

struct RenderWorkspace {
    size_t capacity = 0;  // path slots
    DevBuf ray_o, ray_d, hit, thr, rad, rng, meta, q0, q1, sh_o, sh_d, sh_c, mat_key, counters, sort_tmp;
    DevBuf bin_blocks;  // material binning: each block's count, then start, per bin
    size_t sort_capacity = 0;
    // CUDA-graph replay: an internal stream (the caller's may be the legacy
    // default stream, which cannot be captured), events that order it after
    // and before the caller's stream, and the instantiated graph.
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct pt_scene {
    pt_context *ctx = nullptr;  // creating context (may be destroyed before the scene)
    int device = 0;             // copies of the context's device facts
    int num_sms = 0;
    int max_smem_per_block = 0;
    pt_scene_desc desc_shallow{};  // sizes only (pointers are not kept)
    uint32_t num_tris = 0, num_spheres = 0, num_prims = 0;
    uint32_t num_curve_segments = 0, num_curve_pieces = 0;  // pieces follow the spheres in primitive order
    uint32_t num_vertices = 0;
    std::vector<MeshInstanceRef> mesh_instances;
    std::vector<uint32_t> mesh_num_vertices;
    float scene_mag = 1.f;  // max |coordinate| of the scene bounds and the camera

    // host copies used by refit / updates
    std::vector<float4> h_prims_world;  // 3 per primitive, world order

    // device data
    DevBuf prims_world;  // 3 float4 per prim (world order)
    DevBuf prims_bvh;    // 3 float4 per prim (leaf order)
    DevBuf nodes;
    DevBuf cnodes;       // width 8: compressed copies of the nodes (the traversal reads these)
    DevBuf tri_vidx, vpos, vnrm, vuv, prim_inst, inst, mats, emitters, emitter_cdf;
    DevBuf emitter_tex;  // textures of textured area-emitter radiance (DevTexture each)
    DevBuf curve_seg, curve_cp;  // piece -> segment; 4 world control points per segment
    DevBuf mesh_obj_pos;  // scratch for pt_scene_update_vertices
    // BVH build scratch and results
    DevBuf bvh_scratch;
    DevBuf bvh_order;  // primitive id of each leaf slot (sorted Morton order)
    DevBuf sah_scratch;     // two doubles for the SAH reduction
    DevBuf xform_table;     // per mesh instance: world vertex range + matrix (all-vertex updates)
    DevBuf all_obj_pos;     // host positions staged for pt_scene_update_all_vertices
    uint64_t total_mesh_vertices = 0;
    std::vector<EmitterSource> emitter_sources;
    // bitmap textures: one CUDA texture object per distinct (pixels, size, modes)
    struct BitmapTexture {
        const float *pixels;
        uint32_t w, h, address, filter;
        cudaArray_t array;
        cudaTextureObject_t obj;
    };
    std::vector<BitmapTexture> bitmaps;
    DevBuf env_row_cdf, env_col_cdf, env_row_weight;
    uint32_t env_type = 0;  // PT_ENV_*
    bool has_env = false;
    float env_radiance[3] = {0, 0, 0};
    bool has_emissive_mesh = false;
    std::vector<uint32_t> level_start;  // first wide node of each level; back() = num_nodes
    pt_bvh_opts bvh_opts{};
    pt_bvh_stats bvh_stats{};
    bool bvh_built = false;

    ptd::DevScene dev{};
    RenderWorkspace ws;
    pt_render_stats render_stats{};
    uint32_t tuned_block = 0;       // autotuned defaults (0 = built-in defaults)
    uint32_t tuned_wave_paths = 0;

    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ~pt_scene();
};

// pt_bvh.cu
int pt_bvh_build_impl(pt_scene *s, const pt_bvh_opts *opts, cudaStream_t stream);
int pt_bvh_refit_impl(pt_scene *s, cudaStream_t stream);
// Compressed copies of n 8-wide float nodes (6 float4 each, same indices).
int pt_compress_wide8(const float *nodes, uint32_t n, float4 *out, cudaStream_t stream);
// pt_render.cu
int pt_render_impl(pt_scene *s, const pt_render_params *p, const pt_frame_buffers *fb, cudaStream_t stream);
int pt_render_batch_impl(pt_context *ctx, pt_scene *const *scenes, const pt_render_params *p,
                         const pt_frame_buffers *fbs, uint32_t n, cudaStream_t stream);
int pt_render_batch_stats(const pt_context *ctx, pt_render_stats *out);
int pt_trace_rays_impl(pt_scene *s, const float *rays, float *hits, uint32_t n, int anyhit, cudaStream_t stream);
int pt_autotune_impl(pt_scene *s, const pt_render_params *p, const pt_frame_buffers *fb, pt_tune_result *out,
                     cudaStream_t stream);
int pt_bsdf_eval_impl(const float *bsdf, const float *wo, const float *wi, float *f, float *pdf, uint32_t n,
                      cudaStream_t stream);
int pt_bsdf_sample_impl(const float *bsdf, const float *wo, uint32_t *rng, float *wi, float *f, float *pdf,
                        uint32_t *type, uint32_t n, cudaStream_t stream);
int pt_trig_eval_impl(uint32_t fn, const float *x, const float *y, float *out, float *out_platform, uint32_t n,
                      cudaStream_t st);
// Re-transforms the world vertices / primitive records of mesh instances on the device.
int pt_update_world_vertices(pt_scene *s, uint32_t mesh, const float *d_obj_pos, uint32_t num_vertices,
                             cudaStream_t stream);
int pt_update_all_world_vertices(pt_scene *s, const float *d_obj_pos, cudaStream_t stream);
// pt_scene.cpp: (re)build the emitter table from the world vertices on the
// device (host_vpos, if given, holds them already).
int pt_rebuild_emitters(pt_scene *s, const float4 *host_vpos);
