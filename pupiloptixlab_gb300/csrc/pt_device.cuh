// pt_device.cuh -- device-side vector math, random streams and scene layout
// of the GB300 wavefront path tracer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/pt_api.h"

#define PT_DI __device__ __forceinline__
#define PT_HDI __host__ __device__ __forceinline__

namespace ptd {

constexpr float kPi = 3.14159265358979323846f;      // M_PIf
constexpr float kInvPi = 0.318309886183790671538f;  // M_1_PIf
constexpr float kEps = 0.000001f;                   // optix/util.h:8 (IsZero)
constexpr float kMaxDistance = 1e16f;               // optix/util.h:9

// ---------------------------------------------------------------- float3 ops
// Vector / scalar multiplies by the reciprocal, normalize uses 1/sqrt: the
// same operation sequence as the reference's vector helpers, so that with
// contraction disabled the results agree bit for bit where no
// transcendental function is involved.
PT_HDI float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
PT_HDI float3 f3s(float s) { return make_float3(s, s, s); }
PT_HDI float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
PT_HDI float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
PT_HDI float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
PT_HDI float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
PT_HDI float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
PT_HDI float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
PT_HDI float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
PT_HDI float3 operator/(float3 a, float s) {
    float inv = 1.0f / s;
    return a * inv;
}
PT_HDI float3 operator-(float s, float3 a) { return f3(s - a.x, s - a.y, s - a.z); }
PT_HDI float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
PT_HDI float2 operator*(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
PT_HDI float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PT_HDI float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
PT_HDI float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
PT_HDI float length(float3 v) { return sqrtf(dot(v, v)); }
PT_HDI float3 normalize(float3 v) {
    float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
PT_HDI float4 normalize4(float4 v) {
    float inv = 1.0f / sqrtf(dot4(v, v));
    return make_float4(v.x * inv, v.y * inv, v.z * inv, v.w * inv);
}
PT_HDI float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
PT_HDI float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
PT_HDI float comp(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// ---------------------------------------------------------------- random streams
// Reference stream: framework/cuda/random.h:14-40 (TEA-4 seeding of
// (pixel, frame seed), LCG A=1664525 C=1013904223, 24-bit float output).
PT_HDI uint32_t tea4(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
#pragma unroll
    for (int n = 0; n < 4; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

// PCG32 (O'Neill, pcg_basic): XSH-RR output of a 64-bit LCG; initstate =
// pixel index, initseq = frame seed; float = top 24 bits / 2^24.
constexpr uint64_t kPcgMult = 6364136223846793005ULL;
PT_HDI uint32_t pcg_output(uint64_t old) {
    uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = static_cast<uint32_t>(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
}
PT_HDI uint64_t pcg_seed(uint64_t initstate, uint64_t inc) {
    uint64_t state = 0;
    state = state * kPcgMult + inc;
    state += initstate;
    state = state * kPcgMult + inc;
    return state;
}

// Sampler over either stream.  state holds the LCG seed (low 32 bits) or the
// PCG state; inc is the PCG increment (2 * frame seed + 1).
struct Sampler {
    uint64_t state;
    uint64_t inc;
    uint32_t mode;
    PT_HDI void init(uint32_t m, uint32_t pixel, uint32_t seed) {
        mode = m;
        if (mode == PT_RNG_PCG32) {
            inc = (static_cast<uint64_t>(seed) << 1u) | 1u;
            state = pcg_seed(pixel, inc);
        } else {
            inc = 0;
            state = tea4(pixel, seed);
        }
    }
    PT_HDI float next() {
        if (mode == PT_RNG_PCG32) {
            uint64_t old = state;
            state = old * kPcgMult + inc;
            return static_cast<float>(pcg_output(old) >> 8) * (1.0f / 16777216.0f);
        }
        uint32_t s = static_cast<uint32_t>(state) * 1664525u + 1013904223u;
        state = s;
        return static_cast<float>(s & 0x00FFFFFFu) / 16777216.0f;
    }
    // x is drawn before y.
    PT_HDI float2 next2() {
        float a = next();
        float b = next();
        return make_float2(a, b);
    }
};

// ---------------------------------------------------------------- device scene layout
// Texture (cuda::Texture, framework/cuda/texture.h:10-57): 16 words.
struct DevTexture {
    uint32_t type;
    float c0[3];
    float c1[3];
    float pad;
    float4 r0, r1;          // rows 0 and 1 of the uv transform
    unsigned long long obj; // bitmap: cudaTextureObject_t (float4, normalized coordinates)
    unsigned long long pad2;
};

// Material (optix::material::Material + host precompute): 8 + 4*16 words.
struct DevMaterial {
    uint32_t type;
    uint32_t twosided;
    uint32_t nonlinear;
    float eta;
    float int_fdr;
    float spec_weight;
    float pad[2];
    DevTexture tex[4];
};

enum : uint32_t { kEmitNone = 0, kEmitTri = 1, kEmitSphere = 2, kEmitConstEnv = 3, kEmitEnvMap = 4 };

// EnvMapEmitter (framework/render/emitter/env.h:6-65) and its CDF tables
// (framework/world/emitter.cpp:107-149).
struct DevEnvMap {
    unsigned long long tex;  // cudaTextureObject_t: float4, bilinear, wrap, normalized coordinates
    const float *row_cdf;    // h + 1
    const float *col_cdf;    // (w + 1) * h
    const float *row_weight; // h
    uint32_t w, h;
    float normalization, scale;
    float4 to_world[3], to_local[3];  // rows (xyz)
};

// Emitter (optix::Emitter, framework/render/emitter.h:13-29): 8 float4.
struct DevEmitter {
    float4 a;   // type (bits), select_probability, area, radius
    float4 rad; // radiance xyz; w: bits of (1 + index into DevScene::emit_tex) for a textured radiance, else 0
    float4 p0, p1, p2;  // triangle vertices / sphere centre (p0); w: vertex texture coordinate u
    float4 n0, n1, n2;  // triangle vertex normals (normalised); w: vertex texture coordinate v
};

// Per-instance data used when shading a hit.
struct DevInstance {
    uint32_t material;
    uint32_t flags;         // PT_INST_* | kInstHasNormals | kInstHasUvs | kInstSphere | kInstCurve | curve type << kInstCurveTypeShift
    uint32_t prim_offset;   // first primitive id
    int32_t emitter_offset; // first area emitter, or -1
    float4 sphere;          // world centre, radius
    float4 inv0, inv1, inv2;    // world -> object (sphere texcoords)
    float4 obj_center;      // object-space sphere centre
};
enum : uint32_t { kInstHasNormals = 1u << 8, kInstHasUvs = 1u << 9, kInstSphere = 1u << 10, kInstCurve = 1u << 11 };
constexpr uint32_t kInstCurveTypeShift = 12;  // 2 bits: PT_CURVE_*

// Everything a kernel needs, passed by value.
struct DevScene {
    // acceleration structure
    const float4 *nodes;    // wide nodes, 8*width floats each
    const float4 *cnodes;   // width 8: the same nodes compressed (6 float4 each), which the traversal reads
    const float4 *prims;    // 3 float4 per primitive slot in leaf order
    uint32_t width;         // 2, 4 or 8
    uint32_t num_nodes;
    uint32_t root_is_leaf_count;  // >0: single leaf root with this many prims
    uint32_t smem_nodes;
    float pad_mag;          // scene magnitude the box padding was computed for
    // shading data (indexed by primitive id / vertex id)
    const uint32_t *tri_vidx;   // 3 per triangle
    const float4 *vpos;         // world positions
    const float4 *vnrm;         // world normals (not normalised)
    const float2 *vuv;
    const uint32_t *prim_inst;  // primitive -> instance
    const uint32_t *curve_seg;  // curve piece (primitive id - curve_prim0) -> segment
    const float4 *curve_cp;     // 4 world control points (xyz, radius) per segment
    uint32_t curve_prim0;       // first curve piece primitive id (after triangles and spheres)
    const DevInstance *inst;
    const DevMaterial *mats;
    const DevEmitter *emitters; // area emitters
    const DevTexture *emit_tex; // textures of textured emitter radiance
    const float *emitter_cdf;   // running sums of select probabilities
    uint32_t num_emitters;
    uint32_t num_tris;
    uint32_t has_env;
    DevEmitter env;        // type kEmitConstEnv or kEmitEnvMap (then envmap holds the map)
    DevEnvMap envmap;
    // camera (row-major 4x4 each)
    float4 s2c[4];
    float4 c2w[4];
    uint32_t width_px, height_px;
    uint32_t max_depth;  // the scene's integrator depth (used when a render asks for depth 0)
};

// Traversal stack entries per thread (shared-memory short stack plus local
// spill); a wide tree of depth D needs up to D * (width - 1).
constexpr int kTraversalStackEntries = 96;

// Primitives per BVH (one scene, or the merged scenes of a batch): a leaf on
// the traversal stack packs its first primitive slot into 27 bits.
constexpr uint32_t kMaxPrimitives = PT_MAX_PRIMITIVES;
static_assert(kMaxPrimitives == (1u << 27) - 1, "leaf items hold 27-bit primitive slots");

}  // namespace ptd
