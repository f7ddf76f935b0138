/*
 * pt_api.h -- C-ABI of the GB300 wavefront path tracer.
 *
 * This is the thin layer that the C++ host side (the Pass/System mirror and
 * the scene loader) calls into.  Every entry point is `extern "C"`, takes
 * plain pointers and sizes, returns a pt_status and never throws, asserts or
 * traps.  The last error message of the calling thread is available through
 * pt_last_error().  Device waits inside kernels are bounded; a wait that runs
 * out reports PT_ERR_TIMEOUT.
 *
 * Reference interfaces replaced (paths relative to the PupilOptixLab tree):
 *   pt_context_*      cuda::Context::Init         framework/cuda/context.cpp:9-49
 *                     optix::Context::Init        framework/optix/context.cpp:38-50
 *   pt_scene_upload   world::World::LoadScene     framework/world/world.cpp:108-146
 *                     (RenderObject, emitter tables, camera upload:
 *                      framework/world/render_object.cpp:10-65,
 *                      framework/world/emitter.cpp:169-243,321-390,
 *                      framework/world/camera.cpp:72-92)
 *   pt_bvh_build      GAS::Create / IAS::Create   framework/world/gas_manager.cpp:69-245,
 *                                                 framework/world/ias_manager.cpp:29-113
 *   pt_bvh_refit      IAS::Update (OPERATION_UPDATE) framework/world/ias_manager.cpp:116-151
 *   pt_render         PTPass::OnRun + optixLaunch  example/path_tracer/pt_pass.cpp:39-57,
 *                     framework/optix/pass.h:71-89, example/path_tracer/main.cu:38-246
 *   pt_trace_rays     optixTrace (closest hit, main.cu:80-85) and
 *                     Emitter::TraceShadowRay (any hit, framework/render/emitter.h:91-100)
 *   pt_bsdf_*_batch   LocalBsdf::Sample / Eval     framework/render/material/optix_material.h:70-91
 *   pt_camera_make    util::Camera::GetSampleToCameraMatrix / GetToWorldMatrix
 *                     framework/util/camera.cpp:7-47
 */
#ifndef PT_API_H_
#define PT_API_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_API_VERSION 2

typedef enum pt_status {
    PT_OK = 0,
    PT_ERR_INVALID = 1,     /* bad argument, size or descriptor */
    PT_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    PT_ERR_OOM = 3,         /* device allocation failed */
    PT_ERR_TIMEOUT = 4,     /* a bounded device wait ran out */
    PT_ERR_NAN = 5,         /* NaN/Inf radiance (PT_RENDER_CHECK_FINITE) */
    PT_ERR_UNSUPPORTED = 6, /* feature not available (e.g. no GPU) */
    PT_ERR_OOB = 7,         /* index out of range in the scene data */
    PT_ERR_STATE = 8        /* call made in the wrong order (e.g. render before BVH build) */
} pt_status;

/* Material types: numerically equal to Pupil::EMatType
 * (framework/render/material/predefine.h:15-22, framework/decl/material_decl.inl:4-10). */
typedef enum pt_material_type {
    PT_MAT_UNKNOWN = 0,
    PT_MAT_DIFFUSE = 1,
    PT_MAT_DIELECTRIC = 2,
    PT_MAT_ROUGH_DIELECTRIC = 3,
    PT_MAT_CONDUCTOR = 4,
    PT_MAT_ROUGH_CONDUCTOR = 5,
    PT_MAT_PLASTIC = 6,
    PT_MAT_ROUGH_PLASTIC = 7
} pt_material_type;

/* BSDF lobe flags: equal to optix::EBsdfLobeType (framework/render/material/bsdf/bsdf.h:7-24). */
typedef enum pt_lobe {
    PT_LOBE_UNKNOWN = 0,
    PT_LOBE_NULL = 1,
    PT_LOBE_DIFFUSE_REFLECTION = 1 << 1,
    PT_LOBE_DIFFUSE_TRANSMISSION = 1 << 2,
    PT_LOBE_GLOSSY_REFLECTION = 1 << 3,
    PT_LOBE_GLOSSY_TRANSMISSION = 1 << 4,
    PT_LOBE_DELTA_REFLECTION = 1 << 5,
    PT_LOBE_DELTA_TRANSMISSION = 1 << 6,
    PT_LOBE_DELTA = (1 << 5) | (1 << 6)
} pt_lobe;

/* Texture kinds: equal to util::ETextureType for RGB and Checkerboard
 * (framework/util/texture.h). Bitmap textures are not supported yet. */
typedef enum pt_texture_type { PT_TEX_RGB = 0, PT_TEX_BITMAP = 1, PT_TEX_CHECKERBOARD = 2 } pt_texture_type;

/* Random streams.  PT_RNG_REF_LCG is the reference's cuda::Random (TEA-4
 * seeding + LCG, framework/cuda/random.h:14-40); PT_RNG_PCG32 is PCG32
 * (O'Neill, pcg_basic) seeded with initstate = pixel index, initseq = frame
 * seed, 24-bit float output.  Both are drawn in the reference's order. */
typedef enum pt_rng_mode { PT_RNG_REF_LCG = 0, PT_RNG_PCG32 = 1 } pt_rng_mode;

/* Bitmap sampling modes: the values of cudaTextureAddressMode /
 * cudaTextureFilterMode, as the reference casts its own enums to them
 * (framework/cuda/texture.cpp:82-84). */
enum { PT_TEX_ADDRESS_WRAP = 0, PT_TEX_ADDRESS_CLAMP = 1, PT_TEX_ADDRESS_MIRROR = 2 };
enum { PT_TEX_FILTER_POINT = 0, PT_TEX_FILTER_LINEAR = 1 };

/* One texture: cuda::Texture (framework/cuda/texture.h:10-57).  color0 is the
 * RGB value or checkerboard patch1, color1 is patch2.  uv_transform holds
 * the first two rows of the 4x4 texture-coordinate transform (row-major).
 * PT_TEX_BITMAP: pixels are RGBA floats, width*height*4, row-major, in HOST
 * memory during pt_scene_upload (util::BitmapTexture, framework/util/texture.h);
 * they are sampled like the reference's float4 CUDA texture object
 * (normalized coordinates, framework/cuda/texture.cpp:60-102). */
typedef struct pt_texture_desc {
    uint32_t type;
    float color0[3];
    float color1[3];
    float uv_transform[8];
    const float *pixels;
    uint32_t width, height;
    uint32_t address_mode;  /* PT_TEX_ADDRESS_* */
    uint32_t filter;        /* PT_TEX_FILTER_* */
} pt_texture_desc;

/* Texture slots per material type (tex[i]):
 *   DIFFUSE          0 reflectance
 *   DIELECTRIC       0 specular_reflectance, 1 specular_transmittance
 *   ROUGH_DIELECTRIC 0 specular_reflectance, 1 specular_transmittance, 2 alpha (.x)
 *   CONDUCTOR        0 specular_reflectance, 1 eta, 2 k
 *   ROUGH_CONDUCTOR  0 specular_reflectance, 1 eta, 2 k, 3 alpha (.x)
 *   PLASTIC          0 diffuse_reflectance, 1 specular_reflectance
 *   ROUGH_PLASTIC    0 diffuse_reflectance, 1 specular_reflectance, 2 alpha (.x)
 * Mirrors resource::Material (framework/resource/material.h:16-80). */
typedef struct pt_material_desc {
    uint32_t type;      /* pt_material_type */
    uint32_t twosided;  /* flip the shading normal toward the ray (geometry.h:176-180) */
    uint32_t nonlinear; /* plastic / rough plastic */
    float int_ior;
    float ext_ior;
    pt_texture_desc tex[4];
} pt_material_desc;

/* Triangle mesh in object space (resource::Shape mesh, framework/resource/shape.h). */
typedef struct pt_mesh_desc {
    const float *positions; /* num_vertices * 3 */
    const float *normals;   /* num_vertices * 3, or NULL: geometric normal cross(p1-p0,p2-p0) */
    const float *texcoords; /* num_vertices * 2, or NULL: uv = 0 */
    const uint32_t *indices; /* num_triangles * 3 */
    uint32_t num_vertices;
    uint32_t num_triangles;
} pt_mesh_desc;

typedef struct pt_sphere_desc {
    float center[3];
    float radius;
} pt_sphere_desc;

/* Curve strands (hair) in object space: resource::Shape _hair
 * (framework/resource/shape.cpp:369-420) as handed to the OptiX curve build
 * input (framework/world/gas_manager.cpp:112-150).  Segment i uses the
 * control points segments[i] .. segments[i] + degree (degree 1 linear,
 * 2 quadratic B-spline, 3 cubic B-spline and Catmull-Rom); radii are the
 * per-point radii the reference calls widths.  Segments of one strand are
 * consecutive control-point indices, so a strand ends where segments[i+1] !=
 * segments[i] + 1.  Round segments: linear segments have spherical caps at
 * both ends; the spline types are open at strand ends (OptiX's default end
 * caps).  Only hits entering the tube from outside are reported. */
enum {
    PT_CURVE_LINEAR = 0,
    PT_CURVE_QUADRATIC_BSPLINE = 1,
    PT_CURVE_CUBIC_BSPLINE = 2,
    PT_CURVE_CATMULL_ROM = 3
};
typedef struct pt_curves_desc {
    const float *positions;   /* num_points * 3 */
    const float *radii;       /* num_points */
    const uint32_t *segments; /* num_segments: first control point of each segment */
    uint32_t num_points;
    uint32_t num_segments;
    uint32_t type;            /* PT_CURVE_* */
} pt_curves_desc;

enum { PT_SHAPE_MESH = 0, PT_SHAPE_SPHERE = 1, PT_SHAPE_CURVES = 2 };
enum { PT_INST_FLIP_NORMALS = 1, PT_INST_FLIP_TEXCOORDS = 2 };

/* One shape instance (resource::ShapeInstance; world::RenderObject,
 * framework/world/render_object.h:11-38).  to_world is a row-major 4x4 with
 * the translation in the last column (util::Transform).  Spheres accept
 * similarity transforms only (rotation, uniform scale, translation); curve
 * radii scale by the length of the transformed x axis.  Curves cannot be
 * emitters.  An emissive instance is an area emitter (AreaEmitter,
 * framework/resource/emitter.h:17-19): its radiance is radiance[3], or, with
 * radiance_textured = 1, the texture radiance_tex (RGB, checkerboard or
 * bitmap, sampled at the surface's texture coordinates as
 * framework/render/emitter/area.h:17-45 and sphere.h:14-42 do; its selection
 * weight is the texture's mean maximum channel times the area,
 * framework/world/emitter.cpp:77-101). */
typedef struct pt_instance_desc {
    uint32_t shape_type;  /* PT_SHAPE_* */
    uint32_t shape_index; /* into meshes[], spheres[] or curves[] */
    uint32_t material;    /* into materials[] */
    uint32_t flags;       /* PT_INST_* */
    float to_world[16];
    uint32_t is_emitter;  /* area emitter */
    float radiance[3];    /* its constant RGB radiance (radiance_textured = 0) */
    uint32_t radiance_textured;
    pt_texture_desc radiance_tex;
} pt_instance_desc;

/* optix::Camera (framework/render/camera.h:7-10): two row-major 4x4 matrices. */
typedef struct pt_camera_desc {
    float sample_to_camera[16];
    float camera_to_world[16];
} pt_camera_desc;

enum { PT_ENV_NONE = 0, PT_ENV_CONST = 1, PT_ENV_MAP = 2 };
/* PT_ENV_CONST: ConstEnvEmitter (framework/render/emitter/env.h:67-86), radiance.
 * PT_ENV_MAP: EnvMapEmitter (env.h:6-65): an equirectangular RGBA float map
 * (pixels in HOST memory, width*height*4), times scale, oriented by the upper
 * 3x3 of to_world (row-major); sampled by luminance (the CDF tables of
 * framework/world/emitter.cpp:107-149), filtered bilinearly with wrap-around. */
typedef struct pt_env_desc {
    uint32_t type;
    float radiance[3];
    const float *pixels;
    uint32_t width, height;
    float scale;
    float to_world[16];
} pt_env_desc;

typedef struct pt_scene_desc {
    const pt_mesh_desc *meshes;
    uint32_t num_meshes;
    const pt_sphere_desc *spheres;
    uint32_t num_spheres;
    const pt_material_desc *materials;
    uint32_t num_materials;
    const pt_instance_desc *instances;
    uint32_t num_instances;
    pt_env_desc env;
    pt_camera_desc camera;
    uint32_t width;     /* film size (resource::Film); width x height < 2^31 */
    uint32_t height;
    uint32_t max_depth; /* integrator max_depth (resource::Integrator) */
    const pt_curves_desc *curves;
    uint32_t num_curves;
} pt_scene_desc;

typedef struct pt_context pt_context;
typedef struct pt_scene pt_scene;

typedef struct pt_device_opts {
    int device;      /* CUDA ordinal */
    uint32_t flags;  /* reserved, 0 */
} pt_device_opts;

/* BVH options.  width: 2, 4 or 8 children per node, collapsed with an SAH
 * cost model from a binary tree built over Morton-sorted primitives: by
 * default PLOC (parallel locally-ordered clustering, higher quality), with
 * PT_BVH_FAST_BUILD the Karras radix tree (faster build, for per-frame
 * rebuilds); scenes whose primitives are mostly curve pieces always get the
 * radix tree, which traces them faster.  Leaves are chosen by SAH with curve
 * pieces weighted as three triangle tests.  max_leaf_size: primitives per
 * leaf (1..15).  smem_nodes: number
 * of top nodes staged in shared memory by the traversal kernels (0 = none;
 * width 8 ignores it).  Width-8 trees are traversed as compressed 96-byte
 * nodes (per-node grid, 8-bit child boxes, children in octant order). */
enum { PT_BVH_FAST_BUILD = 1 };
enum { PT_BVH_BUILDER_RADIX = 0, PT_BVH_BUILDER_PLOC = 1 };
typedef struct pt_bvh_opts {
    uint32_t width;
    uint32_t max_leaf_size;
    uint32_t smem_nodes;
    uint32_t flags;
} pt_bvh_opts;

typedef struct pt_bvh_stats {
    uint32_t width;
    uint32_t num_nodes;
    uint32_t num_leaves;
    uint32_t num_prims;
    uint32_t max_depth;
    float sah_cost;        /* SAH cost of the wide tree (node cost 1.2, primitive cost 1) */
    float build_ms;        /* device time of the last build or refit */
    uint64_t node_bytes;   /* bytes of the nodes the traversal reads (32 * width; 96 per node for width 8) */
    uint64_t prim_bytes;
    uint32_t builder;      /* PT_BVH_BUILDER_*: how the binary tree was built */
} pt_bvh_stats;

/* Render parameters: PTPass launch params (example/path_tracer/type.h:9-33).
 * A call renders `spp` frames; frame f uses random seed `seed + f` and
 * sample count `sample_cnt + f`, exactly as spp consecutive PTPass::OnRun
 * calls (pt_pass.cpp:39-57) would. */
typedef struct pt_render_params {
    uint32_t spp;
    uint32_t max_depth;   /* 0 = scene value */
    uint32_t seed;        /* random_seed of the first frame */
    uint32_t sample_cnt;  /* sample_cnt of the first frame */
    uint32_t accumulate;  /* accumulated_flag */
    uint32_t rng;         /* pt_rng_mode */
    uint32_t wave_spp;    /* frames per wavefront wave (0 = auto; frames x pixels < 2^31) */
    uint32_t block_size;  /* threads per block of the wavefront kernels (0 = auto) */
    uint32_t flags;       /* PT_RENDER_* */
} pt_render_params;

enum {
    PT_RENDER_NO_MATERIAL_SORT = 1, /* shade hits in queue order instead of binned by material */
    PT_RENDER_COUNTERS = 2,      /* count node visits and primitive tests */
    PT_RENDER_NO_GRAPH = 4,      /* launch the bounce kernels one by one instead of a CUDA graph */
    PT_RENDER_KERNEL_TIMING = 8, /* time each traversal / shading launch with CUDA events
                                    (launches directly, without the CUDA graph) */
    PT_RENDER_CHECK_FINITE = 32,  /* return PT_ERR_NAN when a sample's radiance was NaN or infinite
                                     (after the render; counted in pt_render_stats either way) */
    PT_RENDER_DROP_NONFINITE = 16 /* accumulate a sample whose radiance is NaN or infinite as zero.
                                     Off by default: the reference's integrator (main.cu:97-101)
                                     accumulates such samples, which then stay in the pixel. */
};

/* Caller-owned DEVICE buffers (BufferManager buffers, framework/system/buffer.h:26-63):
 * accum and frame are float4 per pixel, albedo and normal float3, test float.
 * Any pointer except accum may be NULL. */
typedef struct pt_frame_buffers {
    float *accum;
    float *frame;
    float *albedo;
    float *normal;
    float *test;
} pt_frame_buffers;

/* Traversal / shading counters collected with PT_RENDER_COUNTERS. */
typedef struct pt_render_stats {
    uint64_t samples;
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint64_t nodes_visited;       /* wide nodes fetched, closest + any hit */
    uint64_t prims_tested;        /* primitive records fetched */
    uint64_t shadow_nodes_visited;
    uint64_t shadow_prims_tested;
    float render_ms;              /* device time of the last pt_render */
    float extend_ms;              /* closest-hit launches (PT_RENDER_KERNEL_TIMING) */
    float shadow_ms;              /* any-hit launches (PT_RENDER_KERNEL_TIMING) */
    float shade_ms;               /* shading launches (PT_RENDER_KERNEL_TIMING) */
    uint32_t extend_launches;
    uint32_t shadow_launches;
    uint32_t shade_launches;
    uint32_t kernel_launches;     /* all kernels launched by the last pt_render */
    uint32_t waves;
    uint32_t overflow;            /* traversal stack overflows (must be 0) */
    uint32_t nonfinite_samples;   /* samples whose radiance was NaN or infinite */
} pt_render_stats;

/* Flat local BSDF record used by the BSDF batch entry points (16 floats):
 *  [0] type  [1] alpha  [2] eta  [3] int_fdr  [4] specular_sampling_weight
 *  [5] nonlinear  [6..8] colour A  [9..11] colour B  [12..14] colour C  [15] unused
 * colour A = diffuse reflectance (diffuse, plastics) or specular_reflectance;
 * colour B = specular_transmittance (dielectrics), eta (conductors) or
 *            specular_reflectance (plastics);
 * colour C = k (conductors). */
#define PT_LOCAL_BSDF_FLOATS 16

/* ---- context ---------------------------------------------------------- */
int pt_context_create(const pt_device_opts *opts, pt_context **out);
int pt_context_destroy(pt_context *ctx);
/* Copies the calling thread's last error message into buf (always NUL-terminated). */
int pt_last_error(char *buf, size_t buf_size);
int pt_api_version(void);

/* ---- scene ------------------------------------------------------------ */
/* The library copies everything it needs; the descriptor can be freed after.
 * A scene holds at most PT_MAX_PRIMITIVES primitives after instancing
 * (triangles + spheres + the round-cone pieces of its curves); a larger one
 * is refused with PT_ERR_UNSUPPORTED before any device memory is allocated. */
#define PT_MAX_PRIMITIVES 134217727u /* 2^27 - 1 */
int pt_scene_upload(pt_context *ctx, const pt_scene_desc *desc, pt_scene **out);
int pt_scene_destroy(pt_scene *scene);
int pt_scene_set_camera(pt_scene *scene, const pt_camera_desc *camera);
/* Replace the object-space positions of one mesh (all instances of it are
 * re-transformed).  positions: num_vertices*3 host floats.  The BVH must be
 * refit or rebuilt afterwards. */
int pt_scene_update_vertices(pt_scene *scene, uint32_t mesh, const float *positions, uint32_t num_vertices);
/* Replace the object-space positions of every mesh at once: `positions` is
 * the concatenation, in mesh order, of each mesh's num_vertices*3 floats, on
 * the host (on_device = 0) or the device (on_device = 1).  All instances are
 * re-transformed on the device.  The BVH must be refit or rebuilt afterwards.
 * When an emissive instance is a mesh, its light triangles (positions, areas,
 * selection probabilities) are rebuilt too; the call then waits for `stream`.
 * Same role as the per-instance GAS/IAS updates of
 * framework/world/ias_manager.cpp:116-151, for animated vertices. */
int pt_scene_update_all_vertices(pt_scene *scene, const float *positions, int on_device, void *stream);
/* Number of primitives (triangles then spheres) in world order. */
int pt_scene_num_prims(const pt_scene *scene, uint32_t *num_triangles, uint32_t *num_spheres);
/* Curve segments of all curve instances and the round-cone pieces they were
 * split into (each piece is one acceleration-structure primitive). */
int pt_scene_num_curves(const pt_scene *scene, uint32_t *num_segments, uint32_t *num_pieces);

/* ---- acceleration structure ------------------------------------------ */
int pt_bvh_build(pt_scene *scene, const pt_bvh_opts *opts, void *stream);
int pt_bvh_refit(pt_scene *scene, void *stream);
int pt_bvh_get_stats(const pt_scene *scene, pt_bvh_stats *out);

/* ---- rendering -------------------------------------------------------- */
int pt_render(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, void *stream);
int pt_render_get_stats(const pt_scene *scene, pt_render_stats *out);
/* No counterpart in the reference.  Same result as pt_render, for callers
 * that cannot allocate device memory (hosts that hand out device memory only
 * from their own fixed pools or budgets, and interactive callers that must not
 * allocate per frame, since an allocation can synchronise the device).  The
 * render's path state lives in a fixed device array inside the library (about
 * 9.3 MiB, held by every GPU that loads the library until exit) instead of a
 * workspace allocated on first use; the call makes no allocation.  Limit: at
 * most 65,536 pixels (width * height) per call; larger images are rejected
 * with PT_ERR_INVALID.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU (on
 * different streams or threads) race.  No statistics are recorded; the
 * traversal block size is the caller's, else the one pt_autotune chose, as in
 * pt_render, and PT_RENDER_CHECK_FINITE returns PT_ERR_NAN as there. */
int pt_render_noalloc(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, void *stream);

/* Autotuner result: the configuration pt_autotune found fastest. */
typedef struct pt_tune_result {
    uint32_t bvh_width;       /* 2, 4 or 8 */
    uint32_t block_size;      /* threads per block of the traversal kernels */
    uint32_t wave_paths;      /* paths in flight per wave (the queue chunk, in path slots) */
    uint32_t trials;          /* configurations timed */
    float msamples_per_s;     /* throughput of the winner on the tuning render */
    float baseline_msamples_per_s; /* throughput of the configuration the scene had before */
} pt_tune_result;

/* Multi-scene launch (replaces n PTPass::OnRun frame loops,
 * example/path_tracer/pt_pass.cpp:39-57, one per scene): renders params->spp
 * frames of every scene -- each with its own camera, resolution and frame
 * buffers fbs[k] -- with one launch per kernel per bounce.  The scenes' BVHs
 * (all of one width) are merged into one node array for the launch, the
 * path slots of a wave cover every scene's pixels, and the shading queues
 * are shared and binned by (scene, material type).  Each scene gets the
 * image pt_render with the same params would give it (same random streams);
 * max_depth 0 means each scene's own depth.  Statistics:
 * pt_render_batch_get_stats. */
int pt_render_batch(pt_context *ctx, pt_scene *const *scenes, const pt_render_params *params,
                    const pt_frame_buffers *fbs, uint32_t n, void *stream);
int pt_render_batch_get_stats(const pt_context *ctx, pt_render_stats *out);

/* No reference counterpart (the reference has a single OptiX configuration).
 * Times `params` renders on this scene (coordinate search): every
 * combination of BVH width {2, 4, 8} (the BVH is rebuilt) and traversal block
 * size {64, 128, 256} at the default wave size (128 Mi paths), then wave
 * sizes {16Mi, 32Mi, 64Mi paths} with the best pair.  The BVH is rebuilt with the winning width
 * and its block size and wave size become the scene's defaults (used when
 * pt_render_params.block_size / wave_spp are 0).  fb receives the tuning
 * renders.  Use the spp of the renders to be tuned for: the best wave size
 * depends on it. */
int pt_autotune(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb,
                pt_tune_result *out, void *stream);

/* ---- query entry points used by the parity tests ---------------------- */
/* rays: n * 8 floats (ox,oy,oz,tmin, dx,dy,dz,tmax), hits: n * 4 floats
 * (t, prim id as float bits (-1 = miss), u, v) for closest hit; for any hit
 * hits[4i] is 1.0 (occluded) or 0.0.  Both are DEVICE pointers. */
int pt_trace_rays(pt_scene *scene, const float *rays, float *hits, uint32_t n, int anyhit, void *stream);
/* DEVICE pointers.  bsdf: n * 16 floats; wo, wi: n * 3; out_f: n * 3; out_pdf: n. */
int pt_bsdf_eval_batch(const float *bsdf, const float *wo, const float *wi,
                       float *out_f, float *out_pdf, uint32_t n, void *stream);
/* rng_state: n uint32 reference-LCG seeds, updated in place; out_wi, out_f: n*3;
 * out_pdf: n; out_type: n lobe flags. */
int pt_bsdf_sample_batch(const float *bsdf, const float *wo, uint32_t *rng_state,
                         float *out_wi, float *out_f, float *out_pdf, uint32_t *out_type,
                         uint32_t n, void *stream);
/* The library's own trigonometry on the device (no counterpart in the
 * reference, which calls the platform's sinf/cosf/atan2f/acosf): fn 0 sin(x),
 * 1 cos(x), 2 atan2(y, x), 3 acos(x).  out: the functions every kernel uses;
 * out_platform (may be NULL): CUDA's own function of the same name, for
 * accuracy checks.  DEVICE pointers, n floats each (y only for atan2). */
int pt_trig_eval(uint32_t fn, const float *x, const float *y, float *out, float *out_platform,
                 uint32_t n, void *stream);

/* ---- learned denoiser ------------------------------------------------- */
/* Replaces the OptiX HDR denoiser of the reference's DenoisePass
 * (framework/system/denoise_pass.cpp:50-75 -> optix::Denoiser::Execute,
 * framework/optix/denoiser.cpp:171-267; inputs colour + albedo + normal guide
 * layers of the path tracer) with a 5-level U-Net (14 convolutions, 3x3,
 * widths 32-48-64-128-256, 1,259,072 parameters) trained by this library on
 * pairs the tracer renders.  Weights and activations are BF16 with FP32
 * accumulation; every convolution (forward, data and weight gradient) runs
 * on the tensor cores (tcgen05) with TMA-staged operands.  The network works
 * in the log domain: channels 0-2 of its input are log(1 + colour), its
 * output is added to them to give log(1 + denoised colour), the loss is L1
 * on log(1 + x).
 *
 * Training inputs are 9-channel FP16 pixels (colour RGB, albedo RGB, normal
 * XYZ), targets FP32 RGB, both NHWC and on the device. */
typedef struct pt_denoiser pt_denoiser;

typedef struct pt_denoiser_opts {
    float lr;          /* Adam step size (1e-3) */
    float beta1;       /* 0.9 */
    float beta2;       /* 0.999 */
    float eps;         /* 1e-8 */
    uint64_t seed;     /* weight initialisation (He-uniform) */
} pt_denoiser_opts;

typedef struct pt_denoise_io {
    uint32_t width, height;
    const float *color;   /* device, width*height float4 (the renderer's accum/frame buffer) */
    const float *albedo;  /* device, width*height float3 */
    const float *normal;  /* device, width*height float3 */
    float *output;        /* device, width*height float4 (denoised, alpha 1) */
    uint32_t tile;        /* fallback tile side in pixels (0: 16) */
    float fallback_rel;   /* fall back to the raw colour where a tile's mean luminance moved by more */
    float fallback_sigma; /* than max(fallback_rel * mean, fallback_sigma * standard error); <= 0: no fallback */
    uint8_t *tile_fallback; /* device, optional: one byte per tile, 1 = raw colour kept */
    uint32_t flags;       /* PT_DENOISE_* */
} pt_denoise_io;
/* PT_DENOISE_FLIP_ENSEMBLE: run the network on the frame and on its
 * left-right mirror image and average the two outputs (mirrored back) before
 * the output step: one more network pass per frame for a lower error. */
enum { PT_DENOISE_FLIP_ENSEMBLE = 1 };

typedef struct pt_denoise_stats {
    uint32_t tiles;          /* tiles of the last pt_denoise */
    uint32_t fallback_tiles; /* of which kept the raw colour */
    float last_ms;           /* device time of the last pt_denoise */
} pt_denoise_stats;

/* No reference counterpart (OptiX denoiser models are fixed).  opts may be
 * NULL for the defaults. */
int pt_denoiser_create(pt_context *ctx, const pt_denoiser_opts *opts, pt_denoiser **out);
void pt_denoiser_destroy(pt_denoiser *dn);
/* Number of FP32 parameters (per layer: weights [cout][9][cin] then bias[cout],
 * layers in the order of pt_denoiser_layer); the first layer's cin is 16
 * (9 used) and the last layer's cout is 16 (3 used). */
int pt_denoiser_num_params(const pt_denoiser *dn, uint64_t *count);
int pt_denoiser_layer(const pt_denoiser *dn, uint32_t index, uint32_t *cin, uint32_t *cout, uint64_t *offset);
/* HOST pointers: copy the FP32 master parameters out / in (in: also resets Adam). */
int pt_denoiser_get_params(const pt_denoiser *dn, float *params);
int pt_denoiser_set_params(pt_denoiser *dn, const float *params);
/* Optimizer state, so that training can stop and resume (no counterpart in
 * the reference, whose OptiX denoiser is not trained): HOST pointers to
 * 2 * num_params + 4 floats -- Adam's first moments, second moments, then the
 * step count, the two bias corrections and the step size.  set_state after
 * set_params continues the saved run (set_params resets the state). */
int pt_denoiser_get_state(const pt_denoiser *dn, float *state);
int pt_denoiser_set_state(pt_denoiser *dn, const float *state);
/* Forward + backward of the L1 log loss on a batch; gradients stay on the
 * device (pt_denoiser_get_grads, HOST pointer), *loss (HOST) the batch mean. */
int pt_denoiser_compute_grads(pt_denoiser *dn, const void *input_f16, const float *target, uint32_t n,
                              uint32_t height, uint32_t width, float *loss, void *stream);
int pt_denoiser_get_grads(const pt_denoiser *dn, float *grads);
/* One Adam step on a batch (height = width = crop side, multiples of 16).
 * The step runs as one CUDA graph; the batch loss is summed on the device
 * and read (mean over the steps since the last read) by pt_denoiser_read_loss. */
int pt_denoiser_train_step(pt_denoiser *dn, const void *input_f16, const float *target, uint32_t n, uint32_t crop,
                           void *stream);
int pt_denoiser_read_loss(pt_denoiser *dn, float *mean_loss);
/* Adam step size of the following training steps (e.g. a decay schedule). */
int pt_denoiser_set_lr(pt_denoiser *dn, float lr);
/* Network output for a batch: out = width*height*n*3 FP32 linear RGB (device). */
int pt_denoiser_forward(pt_denoiser *dn, const void *input_f16, uint32_t n, uint32_t height, uint32_t width,
                        float *out, void *stream);
/* Denoise one rendered frame (any size; padded internally to multiples of 16),
 * with the per-tile fallback to the raw colour. */
int pt_denoise(pt_denoiser *dn, const pt_denoise_io *io, void *stream);
int pt_denoise_get_stats(const pt_denoiser *dn, pt_denoise_stats *out);
/* Pack a rendered frame (device float4 colour, float3 albedo, float3 normal)
 * into the 9-channel FP16 training layout (device, width*height*9 halves). */
int pt_denoise_pack(const float *color, const float *albedo, const float *normal, uint32_t width, uint32_t height,
                    void *out_f16, void *stream);

/* Convolution kernels of the denoiser, exposed for the gradient checks.
 * DEVICE pointers, NHWC BF16 tensors (raw 16-bit), weights [cout_pad][9][cin]
 * with cout_pad = cout rounded up to 16, cin a multiple of 16.
 * forward: y = x (*) w + bias, ReLU if relu, y BF16 [n][h][w][cout] or FP32 if out_f32.
 * backward_data: dx = dy (*) flip(w)^T, times (mask > 0) where mask (BF16, the
 *   shape of dx) is given; dy has cout_pad channels.
 * backward_weights: dw[cout][9][cin] += sum_p x (x) dy, db[cout] += sum_p dy
 *   (FP32, caller zeroes); dy has cout channels (a multiple of 16). */
int pt_conv3x3_forward(const void *x, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, const void *weight,
                       const float *bias, uint32_t cout, int relu, int out_f32, void *y, void *stream);
int pt_conv3x3_backward_data(const void *dy, uint32_t n, uint32_t h, uint32_t w, uint32_t cout, const void *weight,
                             uint32_t cin, const void *mask, void *dx, void *stream);
int pt_conv3x3_backward_weights(const void *x, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, const void *dy,
                                uint32_t cout, float *dweight, float *dbias, void *stream);
/* Bounded waits of the convolution kernels (no counterpart in the reference,
 * whose closed OptiX denoiser has none): every mbarrier wait gives up after
 * wait_ns of GPU time (0 restores the default, 2 s); the kernel then records
 * an error, lets the copies and MMAs it issued finish, frees its tensor memory
 * and returns, and the call reports PT_ERR_TIMEOUT.  stall_next = 1 makes the
 * next forward convolution that is prepared first wait on a barrier that
 * nothing arrives at, so that this path can be tested without a fault.
 * Process-wide; applies to convolutions prepared after the call (the
 * denoiser's training and inference graphs keep the limit they were built
 * with). */
int pt_conv_set_wait_limit(uint64_t wait_ns, uint32_t stall_next);

/* ---- host helpers (no GPU needed) ------------------------------------- */
/* Camera matrices from a mitsuba-style sensor: fov_y in degrees,
 * to_world row-major 4x4 in Pupil's convention (+Z points away from the view).
 * Restates util::Camera (framework/util/camera.cpp:7-47). */
int pt_camera_make(float fov_y_deg, float aspect, float near_clip, float far_clip,
                   const float to_world[16], pt_camera_desc *out);

#ifdef __cplusplus
}
#endif

#endif /* PT_API_H_ */
