// pt_oracle.cpp -- CPU oracle for PupilOptixLab's "path tracing with MIS" path.
//
// TEST INFRASTRUCTURE ONLY: a plain C++ restatement of the reference's
// integrator and render-layer math, used by tests/, __graft_entry__.smoke()
// and bench.py's CPU baseline as the checker.  The product never links it.
//
// Build: g++ -O3 -std=c++17 -ffp-contract=off (no FMA contraction, so x86-64
// and aarch64 hosts produce identical bits).  Each function cites the
// reference file:line it restates (paths relative to the PupilOptixLab tree).
//
// Definitions this oracle fixes where the reference leaves behaviour to the
// compiler or to uninitialised memory (the product follows the same rules):
//  * Next2() draws x first, then y (the reference's make_float2(Next(), Next())
//    has unspecified argument order in C++).
//  * sin, cos, atan2 and acos are the library's own deterministic functions
//    (pupiloptixlab_gb300/csrc/pt_trig.h, within 3 ulp of the exact values),
//    where the reference calls the platform's (CUDA's device math, or the C
//    library's on a host build), whose last bits differ between platforms.
//  * EmitterSampleRecord::is_delta is false for area/sphere emitters
//    (framework/render/emitter/types.h:25 leaves it uninitialised).
//  * EmitEvalRecord::pdf is 0 when the emitter faces away
//    (framework/render/emitter/area.h:37-45 leaves it uninitialised).
//  * A scene without any emitter skips NEE but still draws its three numbers.
//  * Geometry is flattened to world space: instance transforms are applied to
//    vertices at scene set-up (x' = m0*x + m1*y + m2*z + m3, left to right),
//    normals by the inverse transpose (double-precision inverse rounded to
//    float); hit positions interpolate world-space vertices.
//  * Ray/triangle: watertight test of Woop, Benthin and Wald (JCGT 2013) with
//    its double-precision fallback; closest hit = smallest t, ties broken by
//    the smaller primitive id.

#include "pt_oracle.h"
#include "pt_trig.h"
#include "tex_fetch.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace orc {

constexpr float kPi = 3.14159265358979323846f;      // M_PIf
constexpr float kInvPi = 0.318309886183790671538f;  // M_1_PIf
constexpr float kEps = 0.000001f;                   // optix/util.h:8
constexpr float kMaxDistance = 1e16f;               // optix/util.h:9

// ---------------------------------------------------------------- vectors
struct V2 { float x, y; };
struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

static inline V2 v2(float x, float y) { return {x, y}; }
static inline V3 v3(float x, float y, float z) { return {x, y, z}; }
static inline V3 v3s(float s) { return {s, s, s}; }
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
// Vector / scalar multiplies by the reciprocal (cuda/vec_math.h semantics).
static inline V3 operator/(V3 a, float s) { float inv = 1.0f / s; return a * inv; }
static inline V3 operator-(float s, V3 a) { return {s - a.x, s - a.y, s - a.z}; }
static inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
static inline V2 operator*(V2 a, float s) { return {a.x * s, a.y * s}; }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot4(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float length(V3 v) { return sqrtf(dot(v, v)); }
static inline V3 normalize(V3 v) { float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
static inline V4 normalize4(V4 v) {
    float inv = 1.0f / sqrtf(dot4(v, v));
    return {v.x * inv, v.y * inv, v.z * inv, v.w * inv};
}
static inline V3 lerp(V3 a, V3 b, float t) { return a + t * (b - a); }
static inline float comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// ---------------------------------------------------------------- random
// framework/cuda/random.h:14-40 (TEA-4 seeding, LCG A=1664525 C=1013904223,
// 24-bit float output).
struct RefLcg {
    uint32_t seed = 0;
    void init(uint32_t val0, uint32_t val1) {
        uint32_t v0 = val0, v1 = val1, s0 = 0;
        for (uint32_t n = 0; n < 4; n++) {
            s0 += 0x9e3779b9u;
            v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
            v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
        }
        seed = v0;
    }
    float next() {
        seed = 1664525u * seed + 1013904223u;
        return static_cast<float>(seed & 0x00FFFFFFu) / 16777216.0f;
    }
};

// PCG32 (M. O'Neill, pcg-random.org, pcg_basic): 64-bit LCG state with the
// XSH-RR output permutation.  Seeded with initstate = pixel index and
// initseq = frame seed; the float keeps the top 24 bits.
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    uint32_t raw() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
    }
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0;
        inc = (initseq << 1u) | 1u;
        raw();
        state += initstate;
        raw();
    }
    float next() { return static_cast<float>(raw() >> 8) * (1.0f / 16777216.0f); }
};

struct Sampler {
    uint32_t mode = PT_RNG_REF_LCG;
    RefLcg lcg;
    Pcg32 pcg;
    void init(uint32_t m, uint32_t pixel, uint32_t seed) {
        mode = m;
        if (mode == PT_RNG_PCG32) pcg.seed(pixel, seed);
        else lcg.init(pixel, seed);
    }
    float next() { return mode == PT_RNG_PCG32 ? pcg.next() : lcg.next(); }
    V2 next2() { float a = next(); float b = next(); return {a, b}; }
};

// ---------------------------------------------------------------- sampling utils
// framework/optix/util.h:33-183
static inline V3 uniform_sample_triangle(float u1, float u2) {  // util.h:33-36
    float s = sqrtf(u1);
    return {1.f - s, s * (1.f - u2), u2 * s};
}
static inline V3 uniform_sample_sphere(float u1, float u2) {  // util.h:38-43
    float z = 1.f - 2.f * u1;
    float sin_theta = sqrtf(std::max(0.f, 1.f - z * z));
    float phi = 2.f * kPi * u2;
    return {sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), z};
}
static inline V3 cosine_sample_hemisphere(float u1, float u2) {  // util.h:45-54
    float sin_theta = sqrtf(u1);
    float phi = 2.0f * kPi * u2;
    return {sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), sqrtf(fmaxf(0.f, 1.f - sin_theta * sin_theta))};
}
static inline float cosine_hemisphere_pdf(V3 v) { return v.z > 0.f ? kInvPi * v.z : 0.f; }  // util.h:55-57
static inline V3 uniform_sample_hemisphere(float u1, float u2) {  // util.h:59-69
    float z = 1.f - 2.f * u1;
    float sin_theta = sqrtf(fmaxf(0.f, 1.f - z * z));
    float phi = 2.0f * kPi * u2;
    return {sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), fabsf(z)};
}
static inline float uniform_hemisphere_pdf(V3 v) { return v.z > 0.f ? kInvPi * 0.5f : 0.f; }  // util.h:70-72
static inline V3 reflect_local(V3 v) { return {-v.x, -v.y, v.z}; }                         // util.h:74-78
static inline V3 reflect(V3 v, V3 n) { return -v + 2.f * dot(v, n) * n; }                 // util.h:80-82
static inline V3 refract_local(V3 v, float cos_t, float eta) {                             // util.h:84-87
    float scale = -(cos_t < 0.f ? 1.f / eta : eta);
    return normalize(v3(scale * v.x, scale * v.y, cos_t));
}
static inline V3 refract(V3 v, V3 n, float cos_t, float eta) {  // util.h:89-92
    if (cos_t < 0) eta = 1 / eta;
    return n * (dot(v, n) * eta + cos_t) - v * eta;
}
static inline void build_onb(V3 n, V3 &b1, V3 &b2) {  // util.h:95-101 (Duff et al. 2017)
    float sign = copysignf(1.f, n.z);
    float a = -1.f / (sign + n.z);
    float b = n.x * n.y * a;
    b1 = {1.f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    b2 = {b, sign + n.y * n.y * a, -n.y};
}
static inline V3 to_local(V3 v, V3 n) {  // util.h:103-108
    V3 b1, b2;
    build_onb(n, b1, b2);
    return {dot(v, b1), dot(v, b2), dot(v, n)};
}
static inline V3 to_world(V3 v, V3 n) {  // util.h:110-115
    V3 b1, b2;
    build_onb(n, b1, b2);
    return b1 * v.x + b2 * v.y + n * v.z;
}
static inline V2 sphere_texcoord(V3 p) {  // util.h:117-128
    float phi = pt_atan2f(p.y, p.x);
    phi = phi < 0.f ? phi + kPi * 2.f : phi;
    float theta = pt_acosf(p.z);
    return {phi * kInvPi * 0.5f, theta * kInvPi};
}
static inline float luminance(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }  // util.h:161-163
static inline float mis_weight(float x, float y) { return x / (x + y); }                      // util.h:165-167
static inline bool is_zero(float v) { return fabsf(v) < kEps; }                                // util.h:169-171
static inline bool is_zero(V3 v) { return fabsf(v.x) < kEps && fabsf(v.y) < kEps && fabsf(v.z) < kEps; }

// ---------------------------------------------------------------- fresnel / ggx
// framework/render/material/fresnel.h:7-85
static inline float dielectric_reflectance(float eta, float cos_i, float &cos_t) {
    float scale = cos_i > 0.f ? 1.f / eta : eta;
    float cos_t2 = 1.f - (1.f - cos_i * cos_i) * (scale * scale);
    if (cos_t2 <= 0.0f) {
        cos_t = 0.0f;
        return 1.0f;
    }
    float o_cos_i = cos_i;
    cos_i = fabsf(cos_i);
    cos_t = sqrtf(fmaxf(0.f, cos_t2));
    float rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    cos_t = o_cos_i > 0.f ? -cos_t : cos_t;
    return 0.5f * (rs * rs + rp * rp);
}
static inline float dielectric_reflectance(float eta, float cos_i) {
    float c;
    return dielectric_reflectance(eta, cos_i, c);
}
static inline float conductor_reflectance(float eta, float k, float cos_i) {
    float c2 = cos_i * cos_i;
    float s2 = 1.f - c2;
    float s4 = s2 * s2;
    float t1 = eta * eta - k * k - s2;
    float a2pb2 = sqrtf(fmaxf(0.f, t1 * t1 + 4.f * k * k * eta * eta));
    float a = sqrtf(fmaxf(0.f, 0.5f * (a2pb2 + t1)));
    float term1 = a2pb2 + c2;
    float term2 = 2.f * a * cos_i;
    float rs2 = (term1 - term2) / (term1 + term2);
    float term3 = a2pb2 * c2 + s4;
    float term4 = term2 * s2;
    float rp2 = rs2 * (term3 - term4) / (term3 + term4);
    return 0.5f * (rp2 + rs2);
}
static inline V3 conductor_reflectance(V3 eta, V3 k, float cos_i) {
    return {conductor_reflectance(eta.x, k.x, cos_i), conductor_reflectance(eta.y, k.y, cos_i),
            conductor_reflectance(eta.z, k.z, cos_i)};
}
static inline float diffuse_reflectance(float eta) {  // fresnel.h:58-85 (published fits)
    if (eta < 1) {
        return -1.4399f * (eta * eta) + 0.7099f * eta + 0.6681f + 0.0636f / eta;
    }
    float i1 = 1.0f / eta, i2 = i1 * i1, i3 = i2 * i1, i4 = i3 * i1, i5 = i4 * i1;
    return 0.919317f - 3.4793f * i1 + 6.75335f * i2 - 7.80989f * i3 + 4.98554f * i4 - 1.36881f * i5;
}

// framework/render/material/ggx.h:6-64 (isotropic, visible-normal sampling enabled)
static inline float ggx_lambda(V3 w, float alpha) {
    float a2 = alpha * alpha;
    V3 v2 = w * w;
    return (-1.f + sqrtf(1.f + (v2.x + v2.y) * a2 / v2.z)) / 2.f;
}
static inline float ggx_g1(V3 w, float alpha) { return 1.f / (1.f + ggx_lambda(w, alpha)); }
static inline float ggx_g(V3 wi, V3 wo, float alpha) { return ggx_g1(wi, alpha) * ggx_g1(wo, alpha); }
static inline float ggx_d(V3 wh, float alpha) {
    float a2 = alpha * alpha;
    V3 v2 = wh * wh;
    float t = (v2.x + v2.y) / a2 + v2.z;
    return 1.f / (kPi * a2 * t * t);
}
static inline float ggx_pdf(V3 wo, V3 wh, float alpha) {
    return ggx_d(wh, alpha) * ggx_g1(wo, alpha) * dot(wo, wh) / fabsf(wo.z);
}
static inline V3 ggx_sample(V3 wo, float alpha, V2 xi) {
    V3 vh = normalize(v3(alpha * wo.x, alpha * wo.y, wo.z));
    V3 t1v = wo.z < 0.9999f ? normalize(cross(v3(0.f, 0.f, 1.f), vh)) : v3(1.f, 0.f, 0.f);
    V3 t2v = cross(vh, t1v);
    float r = sqrtf(xi.x);
    float phi = 2.f * kPi * xi.y;
    float t1 = r * pt_cosf(phi);
    float t2 = r * pt_sinf(phi);
    float s = 0.5f * (1.f + vh.z);
    t2 = (1.f - s) * sqrtf(1.f - t1 * t1) + s * t2;
    V3 nh = t1 * t1v + t2 * t2v + sqrtf(fmaxf(0.f, 1.f - t1 * t1 - t2 * t2)) * vh;
    V3 ne = v3(alpha * nh.x, alpha * nh.y, fmaxf(0.f, nh.z));
    return normalize(ne);
}

// ---------------------------------------------------------------- BSDFs
enum : uint32_t {
    kLobeUnknown = 0,
    kDiffuseReflection = 1u << 1,
    kGlossyReflection = 1u << 3,
    kGlossyTransmission = 1u << 4,
    kDeltaReflection = 1u << 5,
    kDeltaTransmission = 1u << 6,
    kDelta = kDeltaReflection | kDeltaTransmission,
};

// BsdfSamplingRecord, framework/render/material/bsdf/bsdf.h:26-36
struct BsdfRecord {
    V3 wi{0.f, 0.f, 0.f};
    V3 wo{0.f, 0.f, 0.f};
    V3 f{0.f, 0.f, 0.f};
    float pdf = 0.f;
    uint32_t type = kLobeUnknown;
    Sampler *sampler = nullptr;
};

// Material::LocalBsdf, framework/render/material/optix_material.h:23-112, in a
// flat form: a = reflectance / specular_reflectance / diffuse_reflectance,
// b = specular_transmittance / eta (conductors) / specular_reflectance (plastics),
// c = k (conductors).
struct LocalBsdf {
    uint32_t type = PT_MAT_UNKNOWN;
    float alpha = 0.f, eta = 1.f, int_fdr = 0.f, spec_weight = 0.f;
    bool nonlinear = false;
    V3 a{0, 0, 0}, b{0, 0, 0}, c{0, 0, 0};

    // Plastic/RoughPlastic shared terms (plastic.h:38, rough_plastic.h:138)
    V3 plastic_diffuse() const {
        return a / (1.f - (nonlinear ? a * int_fdr : v3s(int_fdr)));
    }
    float specular_prob(float fresnel_o) const {  // plastic.h:48-50
        return (fresnel_o * spec_weight) / (fresnel_o * spec_weight + (1 - fresnel_o) * (1.f - spec_weight));
    }

    void get_bsdf(BsdfRecord &r) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:12-18
                V3 f = v3s(0.f);
                if (r.wi.z > 0.f && r.wo.z > 0.f) f = a * kInvPi;
                r.f = f;
            } break;
            case PT_MAT_DIELECTRIC:  // dielectric.h:23-25
            case PT_MAT_CONDUCTOR:   // conductor.h:19-21
                r.f = v3s(0.f);
                break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:21-30
                r.f = v3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                V3 wh = normalize(r.wi + r.wo);
                V3 fo = conductor_reflectance(b, c, dot(r.wo, wh));
                r.f = a * ggx_d(wh, alpha) * fo * ggx_g(r.wi, r.wo, alpha) / (4.f * r.wi.z * r.wo.z);
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:21-49
                r.f = v3s(0.f);
                if (is_zero(r.wo.z)) return;
                V3 wh;
                bool refl = r.wo.z * r.wi.z > 0.f;
                if (refl) wh = normalize(r.wo + r.wi);
                else wh = normalize(r.wo + r.wi * (r.wo.z > 0.f ? eta : 1.f / eta));
                wh = wh * (wh.z > 0.f ? 1.f : -1.f);
                float F = dielectric_reflectance(eta, dot(r.wo, wh));
                float G = ggx_g(r.wi, r.wo, alpha);
                float D = ggx_d(wh, alpha);
                if (refl) {
                    r.f = a * F * G * D / (4.f * fabsf(r.wi.z) * fabsf(r.wo.z));
                } else {
                    float e = r.wo.z > 0.f ? eta : 1.f / eta;
                    float sd = dot(r.wo, wh) + e * dot(r.wi, wh);
                    r.f = b * fabsf((1.f - F) * D * G * dot(r.wi, wh) * dot(r.wo, wh) /
                                    (sd * sd * r.wi.z * r.wo.z));
                }
            } break;
            case PT_MAT_PLASTIC: {  // plastic.h:32-41
                r.f = v3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float fi = dielectric_reflectance(eta, r.wi.z);
                V3 diff = plastic_diffuse();
                r.f = diff * (1.f - fi) * (1.f - fo) * cosine_hemisphere_pdf(r.wi) / (eta * eta * r.wi.z);
            } break;
            case PT_MAT_ROUGH_PLASTIC: {  // rough_plastic.h:22-35
                r.f = v3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                V3 wh = normalize(r.wi + r.wo);
                r.f = b * dielectric_reflectance(eta, dot(wh, r.wo)) * ggx_d(wh, alpha) *
                      ggx_g(r.wi, r.wo, alpha) / (4.f * r.wo.z * r.wi.z);
                float fi = dielectric_reflectance(eta, r.wi.z);
                V3 diff = plastic_diffuse();
                r.f = r.f + diff * (1.f - fi) * (1.f - fo) * kInvPi / (eta * eta);
            } break;
            default:
                break;
        }
    }

    void get_pdf(BsdfRecord &r) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:20-25
                float pdf = 0.f;
                if (r.wi.z > 0.f && r.wo.z > 0.f) pdf = cosine_hemisphere_pdf(r.wi);
                r.pdf = pdf;
            } break;
            case PT_MAT_DIELECTRIC:
            case PT_MAT_CONDUCTOR:
                r.pdf = 0.f;
                break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:32-38
                r.pdf = 0.f;
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                V3 wh = normalize(r.wi + r.wo);
                wh = normalize(wh);
                r.pdf = ggx_pdf(r.wo, wh, alpha) / (4.f * dot(r.wo, wh));
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:51-71
                r.pdf = 0.f;
                bool refl = r.wo.z * r.wi.z > 0.f;
                V3 wh;
                float dwh_dwo;
                if (refl) {
                    wh = normalize(r.wo + r.wi);
                    dwh_dwo = 1.f / (4.f * dot(r.wi, wh));
                } else {
                    float e = r.wo.z > 0.f ? eta : 1.f / eta;
                    wh = normalize(r.wo + r.wi * e);
                    float sd = dot(r.wo, wh) + e * dot(r.wi, wh);
                    dwh_dwo = (e * e * dot(r.wi, wh)) / (sd * sd);
                }
                wh = wh * (wh.z > 0.f ? 1.f : -1.f);
                V3 wo = r.wo * (r.wo.z > 0.f ? 1.f : -1.f);
                float F = dielectric_reflectance(eta, dot(r.wo, wh));
                r.pdf = fabsf(ggx_pdf(wo, wh, alpha) * (refl ? F : 1.f - F) * dwh_dwo);
            } break;
            case PT_MAT_PLASTIC: {  // plastic.h:43-53
                r.pdf = 0.f;
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float sp = specular_prob(fo);
                r.pdf = cosine_hemisphere_pdf(r.wi) * (1.f - sp);
            } break;
            case PT_MAT_ROUGH_PLASTIC: {  // rough_plastic.h:37-51
                r.pdf = 0.f;
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float sp = specular_prob(fo);
                float dp = 1.f - sp;
                V3 wh = normalize(r.wi + r.wo);
                r.pdf = sp * ggx_pdf(r.wo, wh, alpha) / (4.f * dot(r.wi, wh));
                r.pdf += dp * cosine_hemisphere_pdf(r.wi);
            } break;
            default:
                break;
        }
    }

    // LocalBsdf::Eval (optix_material.h:81-91): GetBsdf then GetPdf.
    void eval(BsdfRecord &r) const {
        get_bsdf(r);
        get_pdf(r);
    }

    // LocalBsdf::Sample (optix_material.h:70-79)
    void sample(BsdfRecord &r) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:27-33
                V2 xi = r.sampler->next2();
                r.wi = cosine_sample_hemisphere(xi.x, xi.y);
                get_pdf(r);
                get_bsdf(r);
                r.type = kDiffuseReflection;
            } break;
            case PT_MAT_DIELECTRIC: {  // dielectric.h:27-44
                float cos_t;
                float F = dielectric_reflectance(eta, r.wo.z, cos_t);
                if (r.sampler->next() < F) {
                    r.wi = reflect_local(r.wo);
                    r.pdf = F;
                    r.f = a * F / fabsf(r.wi.z);
                    r.type = kDeltaReflection;
                } else {
                    r.wi = refract_local(r.wo, cos_t, eta);
                    r.pdf = 1.f - F;
                    float factor = cos_t < 0.f ? 1.f / eta : eta;
                    r.f = b * (1.f - F) * factor * factor / fabsf(r.wi.z);
                    r.type = kDeltaTransmission;
                }
            } break;
            case PT_MAT_CONDUCTOR: {  // conductor.h:23-31
                r.wi = reflect_local(r.wo);
                r.pdf = 1.f;
                V3 fr = conductor_reflectance(b, c, r.wo.z);
                r.f = a * fr / fabsf(r.wi.z);
                r.type = kDeltaReflection;
            } break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:40-46 (lobe tag quirk kept)
                V2 xi = r.sampler->next2();
                r.wi = reflect(r.wo, ggx_sample(r.wo, alpha, xi));
                get_pdf(r);
                get_bsdf(r);
                r.type = kDiffuseReflection;
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:73-96
                V2 xi = r.sampler->next2();
                V3 wo = r.wo * (r.wo.z > 0.f ? 1.f : -1.f);
                V3 wh = ggx_sample(wo, alpha, xi);
                float cos_t = 0.f;
                float F = dielectric_reflectance(eta, dot(r.wo, wh), cos_t);
                if (r.sampler->next() < F) {
                    r.wi = reflect(r.wo, wh);
                    r.type = kGlossyReflection;
                } else {
                    if (is_zero(cos_t)) return;
                    r.wi = refract(r.wo, wh, cos_t, eta);
                    r.type = kGlossyTransmission;
                    if (r.wi.z * r.wo.z >= 0.f) return;
                }
                get_pdf(r);
                get_bsdf(r);
            } break;
            case PT_MAT_PLASTIC: {  // plastic.h:55-80
                if (r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                V2 xi = r.sampler->next2();
                float sp = specular_prob(fo);
                if (xi.x < sp) {
                    r.type = kDeltaReflection;
                    r.wi = reflect_local(r.wo);
                    r.f = b * fo / r.wi.z;
                    r.pdf = sp;
                } else {
                    r.type = kDiffuseReflection;
                    r.wi = cosine_sample_hemisphere((xi.x - sp) / (1.f - sp), xi.y);
                    float fi = dielectric_reflectance(eta, r.wi.z);
                    V3 diff = plastic_diffuse();
                    r.f = diff * (1.f - fi) * (1.f - fo) * cosine_hemisphere_pdf(r.wi) / (eta * eta * r.wi.z);
                    r.pdf = cosine_hemisphere_pdf(r.wi) * (1.f - sp);
                }
            } break;
            case PT_MAT_ROUGH_PLASTIC: {  // rough_plastic.h:53-80
                r.wi = v3s(0.f);
                if (r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float sp = specular_prob(fo);
                V2 xi = r.sampler->next2();
                if (xi.y < sp) {
                    xi.y /= sp;
                    V3 wh = ggx_sample(r.wo, alpha, xi);
                    r.wi = reflect(r.wo, wh);
                    r.type = kGlossyReflection;
                } else {
                    xi.y = (xi.y - sp) / (1.f - sp);
                    r.wi = cosine_sample_hemisphere(xi.x, xi.y);
                    r.type = kDiffuseReflection;
                }
                get_pdf(r);
                get_bsdf(r);
            } break;
            default:
                break;
        }
    }

    V3 albedo() const { return type == PT_MAT_UNKNOWN ? v3s(0.f) : a; }  // optix_material.h:93-111

    static LocalBsdf from_flat(const float *p) {
        LocalBsdf l;
        l.type = static_cast<uint32_t>(p[0]);
        l.alpha = p[1];
        l.eta = p[2];
        l.int_fdr = p[3];
        l.spec_weight = p[4];
        l.nonlinear = p[5] != 0.f;
        l.a = {p[6], p[7], p[8]};
        l.b = {p[9], p[10], p[11]};
        l.c = {p[12], p[13], p[14]};
        return l;
    }
    void to_flat(float *p) const {
        p[0] = static_cast<float>(type);
        p[1] = alpha; p[2] = eta; p[3] = int_fdr; p[4] = spec_weight; p[5] = nonlinear ? 1.f : 0.f;
        p[6] = a.x; p[7] = a.y; p[8] = a.z;
        p[9] = b.x; p[10] = b.y; p[11] = b.z;
        p[12] = c.x; p[13] = c.y; p[14] = c.z;
        p[15] = 0.f;
    }
};

// ---------------------------------------------------------------- textures / materials
struct Bitmap {  // RGBA float pixels + sampling modes (util::BitmapTexture)
    std::vector<float> px;
    uint32_t w = 0, h = 0, address = 0, filter = 1;
    V3 fetch(float u, float v) const {
        texfetch::Float4 c = texfetch::fetch(px.data(), w, h, address, filter, u, v);
        return {c.x, c.y, c.z};
    }
};

struct Texture {  // cuda::Texture::Sample, framework/cuda/texture.h:33-57
    uint32_t type = PT_TEX_RGB;
    V3 c0{0, 0, 0}, c1{0, 0, 0};
    V4 r0{1, 0, 0, 0}, r1{0, 1, 0, 0};
    std::shared_ptr<Bitmap> bitmap;
    V3 sample(V2 uv) const {
        V4 tex{uv.x, uv.y, 0.f, 1.f};
        float tx = dot4(r0, tex), ty = dot4(r1, tex);
        if (type == PT_TEX_BITMAP && bitmap) return bitmap->fetch(tx, ty);  // tex2D<float4>
        if (type == PT_TEX_CHECKERBOARD) {
            tx = tx - (tx > 0.f ? floorf(tx) : ceilf(tx));
            ty = ty - (ty > 0.f ? floorf(ty) : ceilf(ty));
            if (tx < 0.f) tx += 1.f;
            if (ty < 0.f) ty += 1.f;
            if (tx > 0.5f) return ty > 0.5f ? c0 : c1;
            return ty > 0.5f ? c1 : c0;
        }
        return c0;
    }
    V3 average() const {  // GetPixelAverage, optix_material.cpp:8-35
        if (type == PT_TEX_CHECKERBOARD) return v3(c0.x + c1.x, c0.y + c1.y, c0.z + c1.z) * 0.5f;
        if (type == PT_TEX_BITMAP && bitmap) {
            float r = 0.f, g = 0.f, b = 0.f;
            size_t idx = 0;
            for (uint32_t y = 0; y < bitmap->h; y++)
                for (uint32_t x = 0; x < bitmap->w; x++) {
                    r += bitmap->px[idx++];
                    g += bitmap->px[idx++];
                    b += bitmap->px[idx++];
                    idx++;
                }
            const float n = 1.f * bitmap->h * bitmap->w;
            return {r / n, g / n, b / n};
        }
        return c0;
    }
    float max_weight() const {  // GetWeight, world/emitter.cpp:77-101
        auto mx = [](float r, float g, float b) { return r > g ? (r > b ? r : b) : (g > b ? g : b); };
        if (type == PT_TEX_CHECKERBOARD) return (mx(c0.x, c0.y, c0.z) + mx(c1.x, c1.y, c1.z)) * 0.5f;
        if (type == PT_TEX_BITMAP && bitmap) {
            // the reference's loop: i over the width, j over the height, pixel
            // i * w + j (past the last pixel for w > h, where the reference reads
            // beyond its array: the last pixel here)
            const size_t w = bitmap->w, h = bitmap->h, last = w * h - 1;
            float sum = 0.f;
            for (size_t i = 0; i < w; i++)
                for (size_t j = 0; j < h; j++) {
                    const size_t q = std::min(i * w + j, last);
                    sum += mx(bitmap->px[q * 4], bitmap->px[q * 4 + 1], bitmap->px[q * 4 + 2]);
                }
            return sum / (1.f * w * h);
        }
        return mx(c0.x, c0.y, c0.z);
    }
    static Texture from_desc(const pt_texture_desc &d) {
        Texture t;
        t.type = d.type;
        t.c0 = {d.color0[0], d.color0[1], d.color0[2]};
        t.c1 = {d.color1[0], d.color1[1], d.color1[2]};
        t.r0 = {d.uv_transform[0], d.uv_transform[1], d.uv_transform[2], d.uv_transform[3]};
        t.r1 = {d.uv_transform[4], d.uv_transform[5], d.uv_transform[6], d.uv_transform[7]};
        if (d.type == PT_TEX_BITMAP && d.pixels) {
            t.bitmap = std::make_shared<Bitmap>();
            t.bitmap->px.assign(d.pixels, d.pixels + 4ull * d.width * d.height);
            t.bitmap->w = d.width;
            t.bitmap->h = d.height;
            t.bitmap->address = d.address_mode;
            t.bitmap->filter = d.filter;
        }
        return t;
    }
};

// optix::material::Material + its host precompute (optix_material.cpp:87-132)
struct Material {
    uint32_t type = PT_MAT_UNKNOWN;
    bool twosided = false, nonlinear = false;
    float eta = 1.f, int_fdr = 0.f, spec_weight = 0.f;
    Texture tex[4];

    static Material from_desc(const pt_material_desc &d) {
        Material m;
        m.type = d.type;
        m.twosided = d.twosided != 0;
        m.nonlinear = d.nonlinear != 0;
        for (int i = 0; i < 4; i++) m.tex[i] = Texture::from_desc(d.tex[i]);
        m.eta = d.int_ior / d.ext_ior;
        if (m.type == PT_MAT_PLASTIC || m.type == PT_MAT_ROUGH_PLASTIC) {
            float dl = luminance(m.tex[0].average());
            float sl = luminance(m.tex[1].average());
            m.spec_weight = sl / (sl + dl);
            m.int_fdr = diffuse_reflectance(1.f / m.eta);
        }
        return m;
    }

    // Material::GetLocalBsdf (optix_material.h:119-131) and the per-type GetLocal.
    LocalBsdf local(V2 uv) const {
        LocalBsdf l;
        l.type = type;
        switch (type) {
            case PT_MAT_DIFFUSE:
                l.a = tex[0].sample(uv);
                break;
            case PT_MAT_DIELECTRIC:
            case PT_MAT_ROUGH_DIELECTRIC:
                l.eta = eta;
                l.a = tex[0].sample(uv);
                l.b = tex[1].sample(uv);
                if (type == PT_MAT_ROUGH_DIELECTRIC) l.alpha = tex[2].sample(uv).x;
                break;
            case PT_MAT_CONDUCTOR:
            case PT_MAT_ROUGH_CONDUCTOR:
                l.a = tex[0].sample(uv);
                l.b = tex[1].sample(uv);
                l.c = tex[2].sample(uv);
                if (type == PT_MAT_ROUGH_CONDUCTOR) l.alpha = tex[3].sample(uv).x;
                break;
            case PT_MAT_PLASTIC:
            case PT_MAT_ROUGH_PLASTIC:
                l.eta = eta;
                l.nonlinear = nonlinear;
                l.int_fdr = int_fdr;
                l.spec_weight = spec_weight;
                l.a = tex[0].sample(uv);
                l.b = tex[1].sample(uv);
                if (type == PT_MAT_ROUGH_PLASTIC) l.alpha = tex[2].sample(uv).x;
                break;
            default:
                break;
        }
        return l;
    }
};

// ---------------------------------------------------------------- geometry
struct LocalGeometry {  // optix::LocalGeometry, framework/render/geometry.h:34-38
    V3 position{0, 0, 0};
    V3 normal{0, 0, 0};
    V2 texcoord{0, 0};
};

struct Hit {
    float t = 0.f;
    int32_t prim = -1;
    float u = 0.f, v = 0.f;
};

enum : uint32_t { kEmitNone = 0, kEmitTri = 1, kEmitSphere = 2, kEmitConstEnv = 3, kEmitEnvMap = 4 };

// EnvMapEmitter (framework/render/emitter/env.h:6-65) with the tables of
// BuildEnvMapCdfTable (framework/world/emitter.cpp:107-149).
struct EnvMapData {
    Bitmap map;  // bilinear, wrap
    std::vector<float> row_cdf, col_cdf, row_weight;
    float normalization = 0.f, scale = 1.f;
    V3 to_world[3], to_local[3];

    void build(const float *pixels, uint32_t width, uint32_t height, float sc, const float *tw, const float *tl) {
        map.px.assign(pixels, pixels + 4ull * width * height);
        map.w = width;
        map.h = height;
        map.address = texfetch::kWrap;
        map.filter = texfetch::kLinear;
        scale = sc;
        const size_t w = width, h = height;
        col_cdf.assign((w + 1) * h, 0.f);
        row_cdf.assign(h + 1, 0.f);
        row_weight.assign(h, 0.f);
        size_t ci = 0, ri = 0;
        float row_sum = 0.f;
        row_cdf[ri++] = 0.f;
        for (size_t y = 0; y < h; ++y) {
            float col_sum = 0.f;
            col_cdf[ci++] = 0.f;
            for (size_t x = 0; x < w; ++x) {
                const size_t p = y * w + x;
                col_sum += luminance(v3(pixels[p * 4], pixels[p * 4 + 1], pixels[p * 4 + 2]));
                col_cdf[ci++] = col_sum;
            }
            for (size_t x = 1; x < w; ++x) col_cdf[ci - x - 1] /= col_sum;
            col_cdf[ci - 1] = 1.f;
            const float weight = std::sin((y + 0.5f) * kPi / h);
            row_weight[y] = weight;
            row_sum += col_sum * weight;
            row_cdf[ri++] = row_sum;
        }
        for (size_t y = 1; y < h; ++y) row_cdf[ri - y - 1] /= row_sum;
        row_cdf[ri - 1] = 1.f;
        normalization = 1.f / (row_sum * (2.f * kPi / w) * (kPi / h));
        for (int r = 0; r < 3; r++) {
            to_world[r] = {tw[3 * r], tw[3 * r + 1], tw[3 * r + 2]};
            to_local[r] = {tl[3 * r], tl[3 * r + 1], tl[3 * r + 2]};
        }
    }
    // first i in [0, n) with x <= cdf[i], else n (the linear scans of env.h:24-31)
    static uint32_t scan(const float *cdf, uint32_t n, float x) {
        uint32_t i = 0;
        for (; i < n; ++i)
            if (x <= cdf[i]) break;
        return i;
    }
    V3 lookup(float u, float v) const { return map.fetch(u, v) * scale; }
    // SampleDirect (env.h:23-49); the reads the reference makes past its
    // tables when the last row is drawn use row h - 1
    void sample(V2 xi, V3 &wi, V3 &rad, float &pdf) const {
        const uint32_t row = scan(row_cdf.data(), map.h, xi.x);
        const uint32_t crow = std::min(row, map.h - 1);
        const uint32_t col = scan(col_cdf.data() + (size_t)crow * (map.w + 1), map.w - 1, xi.y);
        const float phi = static_cast<float>(col) * kPi * 2.f / static_cast<float>(map.w);
        const float theta = static_cast<float>(row) * kPi / static_cast<float>(map.h);
        const float st = pt_sinf(theta);
        const V3 local{st * pt_sinf(kPi - phi), pt_cosf(theta), st * pt_cosf(kPi - phi)};
        wi = {dot(to_world[0], local), dot(to_world[1], local), dot(to_world[2], local)};
        rad = lookup(phi * 0.5f * kInvPi, theta * kInvPi);
        pdf = luminance(rad) * row_weight[crow] * normalization / std::max(1e-4f, std::fabs(st));
        if (pdf < 0.f) pdf = 0.f;
    }
    // Eval (env.h:51-64) for the emitter point scatter_pos + d
    void eval(V3 scatter_pos, V3 emit_pos, V3 &rad, float &pdf) const {
        V3 dir = normalize(emit_pos - scatter_pos);
        dir = {dot(to_local[0], dir), dot(to_local[1], dir), dot(to_local[2], dir)};
        const float phi = kPi - pt_atan2f(dir.x, dir.z);
        const float theta = pt_acosf(dir.y);
        const float tu = phi * 0.5f * kInvPi, tv = theta * kInvPi;
        uint32_t row = static_cast<uint32_t>(tv * static_cast<float>(map.h));
        row = std::min(row, map.h - 2u);
        rad = lookup(tu, tv);
        const float t = tv * static_cast<float>(map.h) - 1.f * static_cast<float>(row);
        pdf = luminance(rad) * (row_weight[row] + t * (row_weight[row + 1] - row_weight[row])) * normalization /
              std::max(1e-4f, std::fabs(pt_sinf(theta)));
    }
};

struct Emitter {  // optix::Emitter, framework/render/emitter.h:13-29
    uint32_t type = kEmitNone;
    std::shared_ptr<EnvMapData> envmap;
    float weight = 0.f, select_probability = 0.f;
    V3 radiance{0, 0, 0};
    float area = 0.f;
    V3 p[3]{};   // triangle: world vertices; sphere: p[0] = centre
    V3 n[3]{};   // triangle: world normals (normalised)
    V2 uv[3]{};
    float radius = 0.f;
    bool textured = false;  // radiance from `tex` (AreaEmitter radiance texture) instead of `radiance`
    Texture tex;

    V3 radiance_at(V2 texcoord) const { return textured ? tex.sample(texcoord) : radiance; }  // radiance.Sample

    struct SampleRecord {  // EmitterSampleRecord, emitter/types.h:17-26
        V3 radiance{0, 0, 0}, wi{0, 0, 0}, pos{0, 0, 0}, normal{0, 0, 0};
        float distance = 0.f;
        float pdf = 0.f;
        bool distance_set = false;
        bool is_delta = false;
    };

    void sample_direct(SampleRecord &ret, const LocalGeometry &hit, V2 xi) const {
        switch (type) {
            case kEmitTri: {  // emitter/area.h:17-35
                V3 t = uniform_sample_triangle(xi.x, xi.y);
                V3 position = p[0] * t.x + p[1] * t.y + p[2] * t.z;
                V3 normal = normalize(n[0] * t.x + n[1] * t.y + n[2] * t.z);
                V2 texcoord = uv[0] * t.x + uv[1] * t.y + uv[2] * t.z;  // area.h:21
                ret.radiance = radiance_at(texcoord);
                ret.wi = normalize(position - hit.position);
                float NoL = dot(hit.normal, ret.wi);
                float LNoL = dot(normal, -ret.wi);
                if (NoL > 0.f && LNoL > 0.f) {
                    float d = length(position - hit.position);
                    ret.pdf = d * d / (LNoL * area);
                    ret.distance = d;
                    ret.distance_set = true;
                }
                ret.pos = position;
                ret.normal = normal;
            } break;
            case kEmitSphere: {  // emitter/sphere.h:14-32
                V3 t = uniform_sample_sphere(xi.x, xi.y);
                V3 position = t * radius + p[0];
                V3 normal = normalize(t);
                ret.radiance = radiance_at(sphere_texcoord(t));  // sphere.h:19-20
                ret.wi = normalize(position - hit.position);
                float NoL = dot(hit.normal, ret.wi);
                float LNoL = dot(normal, -ret.wi);
                if (NoL > 0.f && LNoL > 0.f) {
                    float d = length(position - hit.position);
                    ret.pdf = d * d / (LNoL * area);
                    ret.distance = d;
                    ret.distance_set = true;
                }
                ret.pos = position;
                ret.normal = normal;
            } break;
            case kEmitEnvMap: {  // emitter/env.h:23-49
                envmap->sample(xi, ret.wi, ret.radiance, ret.pdf);
                ret.distance = kMaxDistance;
                ret.distance_set = true;
                ret.is_delta = false;
                ret.pos = hit.position + ret.wi * ret.distance;
            } break;
            case kEmitConstEnv: {  // emitter/env.h:69-80
                V3 local_wi = uniform_sample_hemisphere(xi.x, xi.y);
                ret.wi = to_world(local_wi, hit.normal);
                ret.pdf = uniform_hemisphere_pdf(local_wi);
                ret.distance = kMaxDistance;
                ret.distance_set = true;
                ret.radiance = radiance;
                ret.is_delta = false;
                ret.pos = hit.position + ret.wi * ret.distance;
            } break;
            default:
                break;
        }
    }

    // Emitter::Eval for the emitter at a hit (area.h:37-45, sphere.h:34-42, env.h:82-85)
    void eval(V3 &out_radiance, float &out_pdf, const LocalGeometry &g, V3 scatter_pos) const {
        out_pdf = 0.f;
        out_radiance = v3s(0.f);
        if (type == kEmitTri || type == kEmitSphere) {
            V3 dir = normalize(scatter_pos - g.position);
            float LNoL = dot(g.normal, dir);
            if (LNoL > 0.f) {
                float d = length(scatter_pos - g.position);
                out_pdf = d * d / (LNoL * area);
                out_radiance = radiance_at(g.texcoord);
            }
        } else if (type == kEmitConstEnv) {
            out_pdf = 0.25f * kInvPi;
            out_radiance = radiance;
        } else if (type == kEmitEnvMap) {
            envmap->eval(scatter_pos, g.position, out_radiance, out_pdf);
        }
    }
};

struct Instance {
    uint32_t shape_type = PT_SHAPE_MESH, shape_index = 0, material = 0, flags = 0;
    bool has_normals = false, has_uvs = false;
    uint32_t vertex_offset = 0;  // into the world vertex arrays
    uint32_t prim_offset = 0;    // first primitive id
    int32_t emitter_offset = -1;
    float inv[12]{};             // world -> object (spheres: texcoords)
    V3 center{0, 0, 0};
    float radius = 0.f;
    uint32_t curve_type = 0;     // PT_CURVE_* of a curves instance
};

static void mat_inverse_dd(const double *a, double out[16]) {
    // General 4x4 inverse by cofactors, in double.
    double inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    double rdet = det != 0.0 ? 1.0 / det : 0.0;
    for (int i = 0; i < 16; i++) out[i] = inv[i] * rdet;
}
static void mat_inverse_double(const float m[16], double out[16]) {
    double a[16];
    for (int i = 0; i < 16; i++) a[i] = m[i];
    mat_inverse_dd(a, out);
}

static inline V3 xform_point(const float m[16], V3 p) {  // util::Transform::TransformPoint (w = 1)
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
static inline V3 xform_vec3(const float n[9], V3 v) {
    return {n[0] * v.x + n[1] * v.y + n[2] * v.z, n[3] * v.x + n[4] * v.y + n[5] * v.z,
            n[6] * v.x + n[7] * v.y + n[8] * v.z};
}

// ---------------------------------------------------------------- intersection
struct Ray {
    V3 o, d;
    float tmin, tmax;
};

// Per-ray constants of the watertight test (Woop, Benthin, Wald, JCGT 2(1) 2013).
struct RayWT {
    int kx, ky, kz;
    float sx, sy, sz;
};
static inline RayWT ray_wt(V3 d) {
    RayWT r;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx = r.kz + 1 == 3 ? 0 : r.kz + 1;
    r.ky = r.kx + 1 == 3 ? 0 : r.kx + 1;
    if (comp(d, r.kz) < 0.f) std::swap(r.kx, r.ky);
    float dz = comp(d, r.kz);
    r.sx = comp(d, r.kx) / dz;
    r.sy = comp(d, r.ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

// Returns true and fills t/u/v (u = weight of v1, v = weight of v2) if the ray
// hits the triangle at tmin < t < tmax.
static inline bool intersect_triangle(const Ray &ray, const RayWT &w, V3 p0, V3 p1, V3 p2,
                                      float tmax, float &t_out, float &u_out, float &v_out) {
    V3 A = p0 - ray.o, B = p1 - ray.o, C = p2 - ray.o;
    float Akz = comp(A, w.kz), Bkz = comp(B, w.kz), Ckz = comp(C, w.kz);
    float Ax = comp(A, w.kx) - w.sx * Akz;
    float Ay = comp(A, w.ky) - w.sy * Akz;
    float Bx = comp(B, w.kx) - w.sx * Bkz;
    float By = comp(B, w.ky) - w.sy * Bkz;
    float Cx = comp(C, w.kx) - w.sx * Ckz;
    float Cy = comp(C, w.ky) - w.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        U = (float)(cxby - cybx);
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        V = (float)(axcy - aycx);
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        W = (float)(bxay - byax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    float det = U + V + W;
    if (det == 0.f) return false;
    float Az = w.sz * Akz, Bz = w.sz * Bkz, Cz = w.sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t > ray.tmin && t < tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// OptiX's built-in sphere intersector is closed; this is the library's own:
// the precise formulation of Haines, Guenther and Akenine-Moeller (Ray Tracing
// Gems 2019, ch. 7): discriminant r^2 - |f + (b'/a) d|^2 from the closest
// approach, roots c/q and q/a with q = b' + sign(b') sqrt(a disc), so that
// hits are accurate to a few ulp of t and never fall outside the sphere's box.
static inline bool intersect_sphere(const Ray &ray, V3 c, float r, float tmax, float &t_out) {
    V3 f = ray.o - c;
    float a = dot(ray.d, ray.d);
    float bp = -dot(f, ray.d);
    float s = bp / a;
    V3 l = {f.x + s * ray.d.x, f.y + s * ray.d.y, f.z + s * ray.d.z};
    float rr = r * r;
    float disc = rr - dot(l, l);
    if (!(disc >= 0.f)) return false;
    float cc = dot(f, f) - rr;
    float q = bp + copysignf(sqrtf(a * disc), bp);
    float t0 = cc / q, t1 = q / a;
    if (t0 > t1) std::swap(t0, t1);
    if (t0 > ray.tmin && t0 < tmax) { t_out = t0; return true; }
    if (t1 > ray.tmin && t1 < tmax) { t_out = t1; return true; }
    return false;
}

// ---------------------------------------------------------------- curves
// Round curve segments (hair).  Evaluation and the hit-point normal restate
// the reference's interpolators and SurfaceNormal (framework/render/curve.h:
// 35-342) in their operation order, as Geometry::GetHitLocalGeometry uses
// them per curve type (framework/render/geometry.h:101-172).  OptiX's curve
// intersector is closed, so a segment is intersected the way the library
// does it: as round-cone pieces (lateral frustum surface plus joint spheres,
// entering hits only), its curve parameter the projection onto the axis.

static inline V4 v4add(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
static inline V4 v4sub(V4 a, V4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
static inline V4 v4scale(float s, V4 a) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
static inline V4 v4over(V4 a, float s) { float inv = 1.0f / s; return v4scale(inv, a); }  // vec_math: times 1/s
static inline V3 v4xyz(V4 a) { return {a.x, a.y, a.z}; }

enum : int { kPieceCurve = 1, kPieceSphere0 = 2, kPieceSphere1 = 4, kPieceClampU = 8 };
constexpr float kCurveUMin = 9.5367431640625e-07f;     // 2^-20
constexpr float kCurveUMax = 0.99999904632568359375f;  // 1 - 2^-20

struct CurvePoly {
    uint32_t degree = 1;
    V4 p[4]{};  // power basis, highest power first (LinearInterpolator p[0] + u p[1], ...)
};

static CurvePoly curve_poly(uint32_t type, const V4 *q) {
    CurvePoly c;
    switch (type) {
        case PT_CURVE_LINEAR:  // LinearInterpolator::Initialize (curve.h:39-42)
            c.degree = 1;
            c.p[0] = q[0];
            c.p[1] = v4sub(q[1], q[0]);
            break;
        case PT_CURVE_QUADRATIC_BSPLINE:  // QuadraticInterpolator::InitializeFromBSpline (curve.h:81-89)
            c.degree = 2;
            c.p[0] = v4over(v4add(v4sub(q[0], v4scale(2.0f, q[1])), q[2]), 2.0f);
            c.p[1] = v4over(v4add(v4scale(-2.0f, q[0]), v4scale(2.0f, q[1])), 2.0f);
            c.p[2] = v4over(v4add(q[0], q[1]), 2.0f);
            break;
        case PT_CURVE_CUBIC_BSPLINE:  // CubicInterpolator::InitializeFromBSpline (curve.h:150-159)
            c.degree = 3;
            c.p[0] = v4over(v4add(v4add(v4add(v4scale(-1.0f, q[0]), v4scale(3.0f, q[1])), v4scale(-3.0f, q[2])), q[3]), 6.0f);
            c.p[1] = v4over(v4add(v4add(v4scale(3.0f, q[0]), v4scale(-6.0f, q[1])), v4scale(3.0f, q[2])), 6.0f);
            c.p[2] = v4over(v4add(v4scale(-3.0f, q[0]), v4scale(3.0f, q[2])), 6.0f);
            c.p[3] = v4over(v4add(v4add(v4scale(1.0f, q[0]), v4scale(4.0f, q[1])), v4scale(1.0f, q[2])), 6.0f);
            break;
        default:  // CubicInterpolator::InitializeFromCatrom (curve.h:180-189)
            c.degree = 3;
            c.p[0] = v4over(v4add(v4add(v4add(v4scale(-1.0f, q[0]), v4scale(3.0f, q[1])), v4scale(-3.0f, q[2])), v4scale(1.0f, q[3])), 2.0f);
            c.p[1] = v4over(v4add(v4add(v4add(v4scale(2.0f, q[0]), v4scale(-5.0f, q[1])), v4scale(4.0f, q[2])), v4scale(-1.0f, q[3])), 2.0f);
            c.p[2] = v4over(v4add(v4scale(-1.0f, q[0]), v4scale(1.0f, q[2])), 2.0f);
            c.p[3] = v4over(v4scale(2.0f, q[1]), 2.0f);
            break;
    }
    return c;
}

static V4 curve_position4(const CurvePoly &c, float u) {  // Position4 (Horner)
    if (c.degree == 1) return v4add(c.p[0], v4scale(u, c.p[1]));
    if (c.degree == 2) return v4add(v4scale(u, v4add(v4scale(u, c.p[0]), c.p[1])), c.p[2]);
    return v4add(v4scale(u, v4add(v4scale(u, v4add(v4scale(u, c.p[0]), c.p[1])), c.p[2])), c.p[3]);
}
static V4 curve_velocity4(const CurvePoly &c, float u) {  // Velocity4
    if (c.degree == 1) return c.p[1];
    if (c.degree == 2) return v4add(v4scale(u, v4scale(2.0f, c.p[0])), c.p[1]);
    if (u == 0) u = 0.000001f;  // curve.h:207-211 (triple knots)
    if (u == 1) u = 0.999999f;
    return v4add(v4scale(u, v4add(v4scale(u, v4scale(3.0f, c.p[0])), v4scale(2.0f, c.p[1]))), c.p[2]);
}
static V3 curve_acceleration3(const CurvePoly &c, float u) {  // Acceleration3
    if (c.degree == 1) return v3s(0.f);
    if (c.degree == 2) return v4xyz(v4scale(2.0f, c.p[0]));
    return v4xyz(v4add(v4scale(u, v4scale(6.0f, c.p[0])), v4scale(2.0f, c.p[1])));
}

// SurfaceNormal (curve.h:261-292 for the splines, 295-326 for linear segments).
static V3 curve_surface_normal(const CurvePoly &c, float u, V3 ps) {
    V3 normal;
    const bool linear = c.degree == 1;
    if (u == 0.0f) {
        normal = linear ? ps - v4xyz(c.p[0]) : -v4xyz(curve_velocity4(c, 0));
    } else if (linear ? u >= 1.0f : u == 1.0f) {
        normal = linear ? ps - (v4xyz(c.p[1]) + v4xyz(c.p[0])) : v4xyz(curve_velocity4(c, 1));
    } else {
        V4 p4 = curve_position4(c, u);
        V3 p = v4xyz(p4);
        float r = p4.w;
        V4 d4 = curve_velocity4(c, u);
        V3 d = v4xyz(d4);
        float dr = d4.w;
        float dd = dot(d, d);
        V3 o1 = ps - p;
        o1 = o1 - (dot(o1, d) / dd) * d;
        o1 = o1 * (r / length(o1));
        if (!linear) dd -= dot(curve_acceleration3(c, u), o1);
        normal = dd * o1 - (dr * r) * d;
    }
    return normalize(normal);
}

// Pieces per segment: chord deviation h^2/8 max|P''| <= 0.05 max radius,
// 1 .. 16 pieces, linear segments in one piece.
static uint32_t curve_pieces(const CurvePoly &c, float rmax) {
    if (c.degree == 1) return 1;
    V3 a0, a1;
    if (c.degree == 2) {
        a0 = a1 = v4xyz(v4scale(2.0f, c.p[0]));
    } else {
        a0 = v4xyz(v4scale(2.0f, c.p[1]));
        a1 = v4xyz(v4add(v4scale(6.0f, c.p[0]), v4scale(2.0f, c.p[1])));
    }
    float acc = std::max(length(a0), length(a1));
    float tol = 0.05f * rmax;
    if (!(tol > 0.f) || !(acc > 0.f)) return 1;
    float q = sqrtf(acc / (8.0f * tol));
    if (!(q < 16.0f)) return 16;
    uint32_t n = (uint32_t)ceilf(q);
    return n < 1 ? 1 : n;
}

struct CurvePiece {
    V3 c0, c1;
    float r0 = 0.f, r1 = 0.f, u0 = 0.f, u1 = 0.f;
    int kind = 0;
    uint32_t segment = 0;
};

// Sphere entry with the origin moved to the closest approach first.
static bool curve_sphere_entry(const Ray &ray, float dd, V3 c, float r, float tmax, float &t_out) {
    V3 f = ray.o - c;
    float tc = -dot(f, ray.d) / dd;
    V3 l = f + tc * ray.d;
    float h = r * r - dot(l, l);
    if (!(h >= 0.f)) return false;
    float t = tc - sqrtf(h / dd);
    if (!(t > ray.tmin && t < tmax)) return false;
    t_out = t;
    return true;
}

// Round-cone piece: entering root of the frustum quadratic formed from the
// components normal to the axis, s = projection onto the axis in [0, len],
// plus the end spheres the kind bits ask for; the smallest entering t wins.
static bool intersect_curve_piece(const Ray &ray, const CurvePiece &pc, float tmax, float &t_out, float &u_out) {
    const float dd = dot(ray.d, ray.d);
    bool hit = false;
    float best = tmax, bu = 0.f, t;
    if ((pc.kind & kPieceSphere0) && curve_sphere_entry(ray, dd, pc.c0, pc.r0, best, t)) { hit = true; best = t; bu = pc.u0; }
    if ((pc.kind & kPieceSphere1) && curve_sphere_entry(ray, dd, pc.c1, pc.r1, best, t)) { hit = true; best = t; bu = pc.u1; }
    V3 e = pc.c1 - pc.c0;
    float len = sqrtf(dot(e, e));
    if (len > 0.f) {
        float inv_len = 1.0f / len;
        V3 ax = {e.x * inv_len, e.y * inv_len, e.z * inv_len};
        float k = (pc.r1 - pc.r0) * inv_len;
        V3 f = ray.o - pc.c0;
        float tc = -dot(f, ray.d) / dd;
        V3 w = f + tc * ray.d;
        float we = dot(w, ax), de = dot(ray.d, ax);
        V3 wp = w + (-we) * ax, dp = ray.d + (-de) * ax;
        float rz = pc.r0 + k * we;
        float kde = k * de;
        float A = dot(dp, dp) - kde * kde;
        float B = dot(wp, dp) - kde * rz;
        float C = dot(wp, wp) - rz * rz;
        float disc = B * B - A * C;
        if (disc >= 0.f && A != 0.f) {
            float tp = (-B - sqrtf(disc)) / A;
            float z = we + tp * de;
            float tt = tc + tp;
            if (z >= 0.f && z <= len && tt > ray.tmin && tt < best) {
                hit = true;
                best = tt;
                bu = pc.u0 + (z * inv_len) * (pc.u1 - pc.u0);
            }
        }
    }
    if (!hit) return false;
    if (pc.kind & kPieceClampU) bu = std::min(std::max(bu, kCurveUMin), kCurveUMax);
    t_out = best;
    u_out = bu;
    return true;
}

struct Box {
    V3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
    void grow(V3 p) {
        lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
        hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
    }
    void grow(const Box &b) { grow(b.lo); grow(b.hi); }
    float area() const {
        V3 e = hi - lo;
        if (e.x < 0.f) return 0.f;
        return 2.f * (e.x * e.y + e.y * e.z + e.z * e.x);
    }
    V3 center() const { return (lo + hi) * 0.5f; }
};

// Reciprocal direction for the slab test; a zero component becomes +-1e30 so
// that a ray lying in a slab plane never produces 0 * inf.
static inline V3 safe_inv(V3 d) {
    return {d.x != 0.f ? 1.0f / d.x : copysignf(1e30f, d.x), d.y != 0.f ? 1.0f / d.y : copysignf(1e30f, d.y),
            d.z != 0.f ? 1.0f / d.z : copysignf(1e30f, d.z)};
}

struct BvhNode {
    Box box;
    uint32_t left = 0, right = 0;   // children (internal)
    uint32_t first = 0, count = 0;  // leaf range in prim_order
};

// ---------------------------------------------------------------- scene
struct Scene {
    uint32_t width = 0, height = 0, max_depth = 1;
    float s2c[16]{}, c2w[16]{};
    std::vector<Material> materials;
    std::vector<Instance> instances;
    // World-space vertex data (per mesh instance).
    std::vector<V3> vpos, vnrm;
    std::vector<V2> vuv;
    // Primitives in world order: triangles, spheres, then curve pieces.
    uint32_t num_tris = 0, num_spheres = 0, num_pieces = 0;
    std::vector<CurvePiece> pieces;
    std::vector<V4> curve_cp;             // 4 world control points per segment
    uint32_t num_prims() const { return num_tris + num_spheres + num_pieces; }
    std::vector<uint32_t> tri_vidx;       // 3 per triangle, global vertex ids
    std::vector<uint32_t> prim_instance;  // per primitive
    std::vector<uint32_t> prim_local;     // index within its mesh
    std::vector<V3> tri_p;                // 3 per triangle (world vertices)
    std::vector<Emitter> areas;
    Emitter env;
    bool has_env = false;
    std::vector<float> area_cdf;          // running sums exactly as SelectOneEmiiter forms them
    // host BVH2
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> prim_order;

    Box prim_box(uint32_t p) const {
        Box b;
        if (p < num_tris) {
            b.grow(tri_p[3 * p]); b.grow(tri_p[3 * p + 1]); b.grow(tri_p[3 * p + 2]);
        } else if (p >= num_tris + num_spheres) {
            const CurvePiece &pc = pieces[p - num_tris - num_spheres];
            b.grow(pc.c0 - v3s(pc.r0));
            b.grow(pc.c0 + v3s(pc.r0));
            b.grow(pc.c1 - v3s(pc.r1));
            b.grow(pc.c1 + v3s(pc.r1));
        } else {
            const Instance &in = instances[prim_instance[p]];
            b.grow(in.center - v3s(in.radius));
            b.grow(in.center + v3s(in.radius));
        }
        return b;
    }

    bool intersect_prim(uint32_t p, const Ray &ray, const RayWT &w, float tmax, float &t, float &u, float &v) const {
        if (p < num_tris) return intersect_triangle(ray, w, tri_p[3 * p], tri_p[3 * p + 1], tri_p[3 * p + 2], tmax, t, u, v);
        u = v = 0.f;
        if (p >= num_tris + num_spheres) return intersect_curve_piece(ray, pieces[p - num_tris - num_spheres], tmax, t, u);
        const Instance &in = instances[prim_instance[p]];
        return intersect_sphere(ray, in.center, in.radius, tmax, t);
    }

    // Closest hit with (t, prim id) lexicographic order; any hit returns the first found.
    Hit trace_brute(const Ray &ray, bool anyhit) const {
        Hit best;
        best.t = ray.tmax;
        RayWT w = ray_wt(ray.d);
        uint32_t np = num_prims();
        for (uint32_t p = 0; p < np; p++) {
            float t, u, v;
            if (!intersect_prim(p, ray, w, ray.tmax, t, u, v)) continue;
            if (anyhit) { best.t = t; best.prim = (int32_t)p; return best; }
            if (t < best.t || (t == best.t && (int32_t)p < best.prim)) {
                best.t = t; best.prim = (int32_t)p; best.u = u; best.v = v;
            }
        }
        if (best.prim < 0) best.t = ray.tmax;
        return best;
    }

    // Slab test, conservative: the far distance is scaled by 1 + 2*gamma(3)
    // (robust traversal, Ize 2013) and the boxes are padded at build time.
    static inline bool slab(const Box &b, const Ray &ray, V3 inv, float tmax, float &tnear) {
        float tx0 = (b.lo.x - ray.o.x) * inv.x, tx1 = (b.hi.x - ray.o.x) * inv.x;
        float ty0 = (b.lo.y - ray.o.y) * inv.y, ty1 = (b.hi.y - ray.o.y) * inv.y;
        float tz0 = (b.lo.z - ray.o.z) * inv.z, tz1 = (b.hi.z - ray.o.z) * inv.z;
        float n = std::max(std::max(std::min(tx0, tx1), std::min(ty0, ty1)), std::max(std::min(tz0, tz1), ray.tmin));
        float f = std::min(std::min(std::max(tx0, tx1), std::max(ty0, ty1)), std::max(tz0, tz1));
        f = std::min(f * 1.0000004f, tmax * 1.0000004f);
        tnear = n;
        return n <= f;
    }

    Hit trace_bvh(const Ray &ray, bool anyhit) const {
        Hit best;
        best.t = ray.tmax;
        if (nodes.empty()) return best;
        RayWT w = ray_wt(ray.d);
        V3 inv = safe_inv(ray.d);
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const BvhNode &nd = nodes[stack[--sp]];
            float tn;
            if (!slab(nd.box, ray, inv, best.t, tn)) continue;
            if (nd.count > 0) {
                for (uint32_t i = 0; i < nd.count; i++) {
                    uint32_t p = prim_order[nd.first + i];
                    float t, u, v;
                    if (!intersect_prim(p, ray, w, best.t == ray.tmax ? ray.tmax : std::nextafter(best.t, INFINITY), t, u, v)) continue;
                    if (anyhit) { best.t = t; best.prim = (int32_t)p; return best; }
                    if (t < best.t || (t == best.t && (int32_t)p < best.prim)) {
                        best.t = t; best.prim = (int32_t)p; best.u = u; best.v = v;
                    }
                }
            } else {
                float tl, tr;
                bool hl = slab(nodes[nd.left].box, ray, inv, best.t, tl);
                bool hr = slab(nodes[nd.right].box, ray, inv, best.t, tr);
                if (hl && hr) {
                    if (tl <= tr) { stack[sp++] = nd.right; stack[sp++] = nd.left; }
                    else { stack[sp++] = nd.left; stack[sp++] = nd.right; }
                } else if (hl) stack[sp++] = nd.left;
                else if (hr) stack[sp++] = nd.right;
            }
        }
        return best;
    }

    Hit trace(const Ray &ray, bool anyhit) const { return nodes.empty() ? trace_brute(ray, anyhit) : trace_bvh(ray, anyhit); }

    // Binned-SAH BVH2 (16 bins on centroids, leaves of up to 4 primitives).
    void build_bvh() {
        uint32_t np = num_prims();
        nodes.clear();
        prim_order.resize(np);
        if (np == 0) return;
        std::vector<Box> boxes(np);
        std::vector<V3> cent(np);
        for (uint32_t p = 0; p < np; p++) {
            boxes[p] = prim_box(p);
            cent[p] = boxes[p].center();
            prim_order[p] = p;
        }
        nodes.reserve(2 * np);
        nodes.push_back(BvhNode{});
        struct Task { uint32_t node, first, count; };
        std::vector<Task> tasks{{0, 0, np}};
        while (!tasks.empty()) {
            Task tk = tasks.back();
            tasks.pop_back();
            Box b, cb;
            for (uint32_t i = 0; i < tk.count; i++) {
                uint32_t p = prim_order[tk.first + i];
                b.grow(boxes[p]);
                cb.grow(cent[p]);
            }
            // pad so the exact primitive test is never culled by rounding
            V3 ext = b.hi - b.lo;
            float mag = std::max({fabsf(b.lo.x), fabsf(b.lo.y), fabsf(b.lo.z), fabsf(b.hi.x), fabsf(b.hi.y), fabsf(b.hi.z)});
            float pad = mag * 4e-7f + std::max({ext.x, ext.y, ext.z}) * 1e-6f + 1e-30f;
            b.lo = b.lo - v3s(pad);
            b.hi = b.hi + v3s(pad);
            nodes[tk.node].box = b;
            auto make_leaf = [&]() { nodes[tk.node].first = tk.first; nodes[tk.node].count = tk.count; };
            if (tk.count <= 4) { make_leaf(); continue; }
            constexpr int kBins = 16;
            float best_cost = INFINITY;
            int best_axis = -1, best_split = 0;
            for (int axis = 0; axis < 3; axis++) {
                float lo = comp(cb.lo, axis), hi = comp(cb.hi, axis);
                if (!(hi > lo)) continue;
                float scale = kBins / (hi - lo);
                Box bb[kBins];
                uint32_t bc[kBins] = {0};
                for (uint32_t i = 0; i < tk.count; i++) {
                    uint32_t p = prim_order[tk.first + i];
                    int bi = std::min(kBins - 1, (int)((comp(cent[p], axis) - lo) * scale));
                    bb[bi].grow(boxes[p]);
                    bc[bi]++;
                }
                float la[kBins], ra[kBins];
                uint32_t lc[kBins], rc[kBins];
                Box acc; uint32_t cnt = 0;
                for (int i = 0; i < kBins; i++) { acc.grow(bb[i]); cnt += bc[i]; la[i] = acc.area(); lc[i] = cnt; }
                acc = Box(); cnt = 0;
                for (int i = kBins - 1; i >= 0; i--) { acc.grow(bb[i]); cnt += bc[i]; ra[i] = acc.area(); rc[i] = cnt; }
                for (int i = 0; i < kBins - 1; i++) {
                    if (lc[i] == 0 || rc[i + 1] == 0) continue;
                    float c = la[i] * lc[i] + ra[i + 1] * rc[i + 1];
                    if (c < best_cost) { best_cost = c; best_axis = axis; best_split = i; }
                }
            }
            uint32_t mid;
            if (best_axis < 0) {
                mid = tk.first + tk.count / 2;  // all centroids equal: split in the middle
            } else {
                float lo = comp(cb.lo, best_axis), hi = comp(cb.hi, best_axis);
                float scale = kBins / (hi - lo);
                auto it = std::partition(prim_order.begin() + tk.first, prim_order.begin() + tk.first + tk.count,
                                         [&](uint32_t p) {
                                             int bi = std::min(kBins - 1, (int)((comp(cent[p], best_axis) - lo) * scale));
                                             return bi <= best_split;
                                         });
                mid = (uint32_t)(it - prim_order.begin());
                if (mid == tk.first || mid == tk.first + tk.count) mid = tk.first + tk.count / 2;
            }
            uint32_t l = (uint32_t)nodes.size();
            nodes.push_back(BvhNode{});
            nodes.push_back(BvhNode{});
            nodes[tk.node].left = l;
            nodes[tk.node].right = l + 1;
            nodes[tk.node].count = 0;
            tasks.push_back({l, tk.first, mid - tk.first});
            tasks.push_back({l + 1, mid, tk.first + tk.count - mid});
        }
    }

    // Geometry::GetHitLocalGeometry (framework/render/geometry.h:60-100,176-180) in world space.
    LocalGeometry hit_geometry(const Hit &h, const Ray &ray) const {
        LocalGeometry g;
        uint32_t p = (uint32_t)h.prim;
        const Instance &in = instances[prim_instance[p]];
        const Material &m = materials[in.material];
        if (p >= num_tris + num_spheres) {  // geometry.h:101-172 (world space)
            g.position = ray.o + h.t * ray.d;
            const CurvePiece &pc = pieces[p - num_tris - num_spheres];
            CurvePoly c = curve_poly(in.curve_type, &curve_cp[4 * (size_t)pc.segment]);
            g.normal = curve_surface_normal(c, h.u, g.position);
        } else if (p < num_tris) {
            uint32_t i0 = tri_vidx[3 * p], i1 = tri_vidx[3 * p + 1], i2 = tri_vidx[3 * p + 2];
            float w0 = 1.f - h.u - h.v;
            g.position = w0 * vpos[i0] + h.u * vpos[i1] + h.v * vpos[i2];
            V3 n;
            if (in.has_normals) n = w0 * vnrm[i0] + h.u * vnrm[i1] + h.v * vnrm[i2];
            else n = cross(vpos[i1] - vpos[i0], vpos[i2] - vpos[i0]);
            g.normal = normalize(n);
            if (in.flags & PT_INST_FLIP_NORMALS) g.normal = g.normal * -1.f;
            if (in.has_uvs) {
                g.texcoord = vuv[i0] * w0 + vuv[i1] * h.u + vuv[i2] * h.v;
                if (in.flags & PT_INST_FLIP_TEXCOORDS) g.texcoord.y = 1.f - g.texcoord.y;
            }
        } else {
            g.position = ray.o + h.t * ray.d;
            V3 local = {in.inv[0] * g.position.x + in.inv[1] * g.position.y + in.inv[2] * g.position.z + in.inv[3],
                        in.inv[4] * g.position.x + in.inv[5] * g.position.y + in.inv[6] * g.position.z + in.inv[7],
                        in.inv[8] * g.position.x + in.inv[9] * g.position.y + in.inv[10] * g.position.z + in.inv[11]};
            g.normal = normalize(g.position - in.center);
            g.texcoord = sphere_texcoord(normalize(local - sphere_local_center(in)));
            if (in.flags & PT_INST_FLIP_NORMALS) g.normal = g.normal * -1.f;
        }
        if (dot(-ray.d, g.normal) < 0.f && m.twosided) g.normal = -g.normal;
        return g;
    }
    std::vector<V3> sphere_centers_obj;
    V3 sphere_local_center(const Instance &in) const { return sphere_centers_obj[in.shape_index]; }

    // EmitterGroup::SelectOneEmiiter (framework/render/emitter.h:110-136)
    const Emitter *select_emitter(float p) const {
        for (size_t i = 0; i < areas.size(); i++)
            if (p <= area_cdf[i]) return &areas[i];
        if (has_env) return &env;
        return areas.empty() ? nullptr : &areas.back();
    }
};

static int build_scene(const pt_scene_desc *d, Scene &s) {
    if (!d) return PT_ERR_INVALID;
    s.width = d->width;
    s.height = d->height;
    s.max_depth = d->max_depth;
    memcpy(s.s2c, d->camera.sample_to_camera, sizeof(s.s2c));
    memcpy(s.c2w, d->camera.camera_to_world, sizeof(s.c2w));
    for (uint32_t i = 0; i < d->num_materials; i++) s.materials.push_back(Material::from_desc(d->materials[i]));
    for (uint32_t i = 0; i < d->num_spheres; i++)
        s.sphere_centers_obj.push_back({d->spheres[i].center[0], d->spheres[i].center[1], d->spheres[i].center[2]});
    // pass 1: triangles
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        Instance in;
        in.shape_type = id.shape_type;
        in.shape_index = id.shape_index;
        in.material = id.material;
        in.flags = id.flags;
        if (id.material >= d->num_materials) return PT_ERR_OOB;
        double invd[16];
        mat_inverse_double(id.to_world, invd);
        for (int k = 0; k < 12; k++) in.inv[k] = (float)invd[k];
        if (id.shape_type == PT_SHAPE_MESH) {
            if (id.shape_index >= d->num_meshes) return PT_ERR_OOB;
            const pt_mesh_desc &m = d->meshes[id.shape_index];
            in.has_normals = m.normals != nullptr;
            in.has_uvs = m.texcoords != nullptr;
            in.vertex_offset = (uint32_t)s.vpos.size();
            in.prim_offset = s.num_tris;
            // normal matrix = inverse transpose of the upper 3x3
            float nm[9] = {(float)invd[0], (float)invd[4], (float)invd[8], (float)invd[1], (float)invd[5],
                           (float)invd[9], (float)invd[2], (float)invd[6], (float)invd[10]};
            for (uint32_t v = 0; v < m.num_vertices; v++) {
                V3 p{m.positions[3 * v], m.positions[3 * v + 1], m.positions[3 * v + 2]};
                s.vpos.push_back(xform_point(id.to_world, p));
                if (m.normals) {
                    V3 n{m.normals[3 * v], m.normals[3 * v + 1], m.normals[3 * v + 2]};
                    s.vnrm.push_back(xform_vec3(nm, n));
                } else {
                    s.vnrm.push_back(v3s(0.f));
                }
                if (m.texcoords) s.vuv.push_back({m.texcoords[2 * v], m.texcoords[2 * v + 1]});
                else s.vuv.push_back({0.f, 0.f});
            }
            for (uint32_t t = 0; t < m.num_triangles; t++) {
                uint32_t a = m.indices[3 * t], b = m.indices[3 * t + 1], c = m.indices[3 * t + 2];
                if (a >= m.num_vertices || b >= m.num_vertices || c >= m.num_vertices) return PT_ERR_OOB;
                s.tri_vidx.push_back(in.vertex_offset + a);
                s.tri_vidx.push_back(in.vertex_offset + b);
                s.tri_vidx.push_back(in.vertex_offset + c);
                s.tri_p.push_back(s.vpos[in.vertex_offset + a]);
                s.tri_p.push_back(s.vpos[in.vertex_offset + b]);
                s.tri_p.push_back(s.vpos[in.vertex_offset + c]);
                s.prim_instance.push_back(ii);
                s.prim_local.push_back(t);
            }
            s.num_tris += m.num_triangles;
        } else if (id.shape_type == PT_SHAPE_SPHERE) {
            if (id.shape_index >= d->num_spheres) return PT_ERR_OOB;
        } else if (id.shape_type == PT_SHAPE_CURVES) {
            if (id.shape_index >= d->num_curves || id.is_emitter) return PT_ERR_INVALID;
            in.curve_type = d->curves[id.shape_index].type;
        } else {
            return PT_ERR_INVALID;
        }
        s.instances.push_back(in);
    }
    // pass 2: spheres after all triangles
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (id.shape_type != PT_SHAPE_SPHERE) continue;
        Instance &in = s.instances[ii];
        const pt_sphere_desc &sp = d->spheres[id.shape_index];
        V3 c{sp.center[0], sp.center[1], sp.center[2]};
        V3 cw = xform_point(id.to_world, c);
        V3 pw = xform_point(id.to_world, v3(c.x + sp.radius, c.y, c.z));
        in.center = cw;
        in.radius = length(cw - pw);  // world/emitter.cpp:231-237
        in.prim_offset = s.num_tris + s.num_spheres;
        s.prim_instance.push_back(ii);
        s.prim_local.push_back(0);
        s.num_spheres++;
    }
    // pass 3: curve segments as round-cone pieces, after the spheres
    uint32_t nseg = 0;
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (id.shape_type != PT_SHAPE_CURVES) continue;
        Instance &in = s.instances[ii];
        const pt_curves_desc &cv = d->curves[id.shape_index];
        if (cv.type > PT_CURVE_CATMULL_ROM) return PT_ERR_INVALID;
        in.prim_offset = s.num_tris + s.num_spheres + s.num_pieces;
        const float *m = id.to_world;
        const float scale = length(v3(m[0], m[4], m[8]));
        const uint32_t deg = cv.type > 2 ? 3u : cv.type + 1u;  // shape.cpp:383
        for (uint32_t i = 0; i < cv.num_segments; i++, nseg++) {
            const uint32_t first = cv.segments[i];
            if ((uint64_t)first + deg >= cv.num_points) return PT_ERR_OOB;
            V4 q[4]{};
            float rmax = 0.f;
            for (uint32_t j = 0; j <= deg; j++) {
                const uint32_t v = first + j;
                V3 pw = xform_point(m, v3(cv.positions[3 * v], cv.positions[3 * v + 1], cv.positions[3 * v + 2]));
                q[j] = {pw.x, pw.y, pw.z, cv.radii[v] * scale};
                rmax = std::max(rmax, q[j].w);
            }
            for (int j = 0; j < 4; j++) s.curve_cp.push_back(q[j]);
            if (!(rmax > 0.f)) continue;
            const bool strand_first = i == 0 || cv.segments[i - 1] + 1 != first;
            const bool strand_last = i + 1 == cv.num_segments || cv.segments[i + 1] != first + 1;
            CurvePoly c = curve_poly(cv.type, q);
            uint32_t np = curve_pieces(c, rmax);
            for (uint32_t k = 0; k < np; k++) {
                CurvePiece pc;
                pc.u0 = (float)k / (float)np;
                pc.u1 = (float)(k + 1) / (float)np;
                V4 a = curve_position4(c, pc.u0), b = curve_position4(c, pc.u1);
                pc.c0 = v4xyz(a);
                pc.c1 = v4xyz(b);
                pc.r0 = std::max(a.w, 0.f);
                pc.r1 = std::max(b.w, 0.f);
                pc.kind = kPieceCurve;
                if (cv.type == PT_CURVE_LINEAR) {
                    pc.kind |= kPieceSphere0 | (strand_last ? kPieceSphere1 : 0);
                } else {
                    pc.kind |= kPieceClampU | ((k > 0 || !strand_first) ? kPieceSphere0 : 0);
                }
                pc.segment = nseg;
                s.pieces.push_back(pc);
                s.prim_instance.push_back(ii);
                s.prim_local.push_back(k);
                s.num_pieces++;
            }
        }
    }
    // emitters in instance order (world/emitter.cpp:169-263)
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (!id.is_emitter) continue;
        Instance &in = s.instances[ii];
        in.emitter_offset = (int32_t)s.areas.size();
        V3 rad{id.radiance[0], id.radiance[1], id.radiance[2]};
        Texture rtex = Texture::from_desc(id.radiance_tex);
        if (!id.radiance_textured) {
            rtex = Texture();
            rtex.c0 = rad;
        }
        const float w = rtex.max_weight();  // GetWeight (world/emitter.cpp:77-101)
        if (id.shape_type == PT_SHAPE_MESH) {
            const pt_mesh_desc &m = d->meshes[id.shape_index];
            double invd[16];
            mat_inverse_double(id.to_world, invd);
            float nm[9] = {(float)invd[0], (float)invd[4], (float)invd[8], (float)invd[1], (float)invd[5],
                           (float)invd[9], (float)invd[2], (float)invd[6], (float)invd[10]};
            for (uint32_t t = 0; t < m.num_triangles; t++) {
                Emitter e;
                e.type = kEmitTri;
                e.radiance = rad;
                e.textured = id.radiance_textured != 0;
                e.tex = rtex;
                for (int k = 0; k < 3; k++) {
                    uint32_t vi = m.indices[3 * t + k];
                    e.p[k] = s.vpos[in.vertex_offset + vi];
                    V3 n = m.normals ? V3{m.normals[3 * vi], m.normals[3 * vi + 1], m.normals[3 * vi + 2]}
                                     : cross(s.vpos[in.vertex_offset + m.indices[3 * t + 1]] - s.vpos[in.vertex_offset + m.indices[3 * t]],
                                             s.vpos[in.vertex_offset + m.indices[3 * t + 2]] - s.vpos[in.vertex_offset + m.indices[3 * t]]);
                    V3 nw = m.normals ? xform_vec3(nm, n) : n;
                    e.n[k] = nw / sqrtf(nw.x * nw.x + nw.y * nw.y + nw.z * nw.z);  // TransformNormal normalises
                    e.uv[k] = m.texcoords ? V2{m.texcoords[2 * vi], m.texcoords[2 * vi + 1]} : V2{0.f, 0.f};
                }
                e.area = length(cross(e.p[1] - e.p[0], e.p[2] - e.p[0])) * 0.5f;
                e.weight = w * e.area;
                s.areas.push_back(e);
            }
        } else {
            Emitter e;
            e.type = kEmitSphere;
            e.radiance = rad;
            e.textured = id.radiance_textured != 0;
            e.tex = rtex;
            e.p[0] = in.center;
            e.radius = in.radius;
            e.area = 4 * 3.14159265358979323846f * e.radius * e.radius;
            e.weight = w * e.area;
            s.areas.push_back(e);
        }
    }
    if (d->env.type == PT_ENV_CONST) {
        s.has_env = true;
        s.env.type = kEmitConstEnv;
        s.env.radiance = {d->env.radiance[0], d->env.radiance[1], d->env.radiance[2]};
        s.env.weight = 1.f;
    } else if (d->env.type == PT_ENV_MAP && d->env.pixels && d->env.width >= 2 && d->env.height >= 2) {
        s.has_env = true;
        s.env.type = kEmitEnvMap;
        s.env.weight = 1.f;
        float tw[9], tl[9];
        double inv[16];
        mat_inverse_double(d->env.to_world, inv);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                tw[3 * r + c] = d->env.to_world[4 * r + c];
                tl[3 * r + c] = static_cast<float>(inv[4 * r + c]);
            }
        s.env.envmap = std::make_shared<EnvMapData>();
        s.env.envmap->build(d->env.pixels, d->env.width, d->env.height, d->env.scale, tw, tl);
    }
    // EmitterHelper::ComputeProbability (world/emitter.cpp:321-337)
    float wsum = 0.f;
    for (auto &e : s.areas) wsum += e.weight;
    if (!s.areas.empty())
        for (auto &e : s.areas) e.select_probability = e.weight / wsum * (float)s.areas.size();
    size_t n_emit = (s.has_env ? 1 : 0) + s.areas.size();
    for (auto &e : s.areas) e.select_probability = e.select_probability / (float)n_emit;
    if (s.has_env) s.env.select_probability = s.env.weight / (float)n_emit;
    float acc = 0.f;
    for (auto &e : s.areas) {
        s.area_cdf.push_back(acc + e.select_probability);
        acc += e.select_probability;
    }
    return PT_OK;
}

// ---------------------------------------------------------------- integrator
struct SampleOut {
    V3 radiance{0, 0, 0};
    V3 albedo{0, 0, 0}, normal{0, 0, 0};
    float test = 0.f;
};

static inline V4 mat_mul4(const float m[16], V4 v) {  // cuda/matrix.h:7-9
    return {dot4({m[0], m[1], m[2], m[3]}, v), dot4({m[4], m[5], m[6], m[7]}, v),
            dot4({m[8], m[9], m[10], m[11]}, v), dot4({m[12], m[13], m[14], m[15]}, v)};
}

// Camera ray, example/path_tracer/main.cu:58-78.
static inline Ray camera_ray(const Scene &s, uint32_t x, uint32_t y, Sampler &rng) {
    float jx = rng.next();
    float jy = rng.next();
    float u = (static_cast<float>(x) + jx) / static_cast<float>(s.width);
    float v = (static_cast<float>(y) + jy) / static_cast<float>(s.height);
    V4 d = mat_mul4(s.s2c, {u, v, 0.f, 1.f});
    float inv = 1.0f / d.w;
    d = {d.x * inv, d.y * inv, d.z * inv, d.w * inv};
    d.w = 0.f;
    d = normalize4(d);
    V4 dw = mat_mul4(s.c2w, d);
    Ray r;
    r.d = normalize(v3(dw.x, dw.y, dw.z));
    r.o = {s.c2w[3], s.c2w[7], s.c2w[11]};
    r.tmin = 0.001f;
    r.tmax = 1e16f;
    return r;
}

// __raygen__main, example/path_tracer/main.cu:38-197 (one sample, no accumulation).
static SampleOut trace_path(const Scene &s, uint32_t pixel, uint32_t seed, uint32_t rng_mode, uint32_t max_depth) {
    SampleOut out;
    Sampler rng;
    rng.init(rng_mode, pixel, seed);
    uint32_t x = pixel % s.width, y = pixel / s.width;
    Ray ray = camera_ray(s, x, y, rng);
    V3 radiance = v3s(0.f), env_radiance = v3s(0.f), throughput = v3s(1.f);
    float env_pdf = 0.f;

    Hit h = s.trace(ray, false);
    bool done = h.prim < 0;
    LocalGeometry geo;
    LocalBsdf bsdf;
    int32_t emitter_index = -1;
    auto load_hit = [&](const Hit &hh, const Ray &rr) {
        geo = s.hit_geometry(hh, rr);
        const Instance &in = s.instances[s.prim_instance[hh.prim]];
        emitter_index = in.emitter_offset >= 0 ? in.emitter_offset + (int32_t)s.prim_local[hh.prim] : -1;
        bsdf = s.materials[in.material].local(geo.texcoord);
    };
    auto miss = [&](const Ray &rr) {  // __miss__default, main.cu:199-215
        if (s.has_env) {
            V3 rad; float pdf;
            LocalGeometry eg;
            eg.position = rr.o + normalize(rr.d);
            s.env.eval(rad, pdf, eg, rr.o);
            env_radiance = rad;
            env_pdf = pdf;
        }
    };
    if (!done) {
        load_hit(h, ray);
        if (emitter_index >= 0) radiance = radiance + s.areas[emitter_index].radiance_at(geo.texcoord);  // GetRadiance
        out.albedo = bsdf.albedo();
        out.normal = geo.normal;
    } else {
        miss(ray);
    }
    out.test = rng.next();

    uint32_t depth = 0;
    while (!done) {
        ++depth;
        if (depth >= max_depth) break;
        float rr = depth > 2 ? 0.95f : 1.0f;
        if (rng.next() > rr) break;
        throughput = throughput / rr;

        {  // next-event estimation, main.cu:117-144
            float sel = rng.next();
            V2 xi = rng.next2();
            const Emitter *e = s.select_emitter(sel);
            if (e) {
                Emitter::SampleRecord es;
                e->sample_direct(es, geo, xi);
                if (es.pdf != 0.f) {  // IsZero(f * pdf) below rejects every pdf == 0 sample
                    Ray sray{geo.position, es.wi, 0.0001f, es.distance - 0.0001f};
                    bool occluded = s.trace(sray, true).prim >= 0;
                    if (!occluded) {
                        BsdfRecord er;
                        er.wi = to_local(es.wi, geo.normal);
                        er.wo = to_local(-ray.d, geo.normal);
                        er.sampler = &rng;
                        bsdf.eval(er);
                        if (!is_zero(er.f * es.pdf)) {
                            float NoL = dot(geo.normal, es.wi);
                            if (NoL > 0.f) {
                                float mis = es.is_delta ? 1.f : mis_weight(es.pdf, er.pdf);
                                float pdf = es.pdf * e->select_probability;
                                radiance = radiance + throughput * es.radiance * er.f * NoL * mis / pdf;
                            }
                        }
                    }
                }
            }
        }
        {  // BSDF sampling, main.cu:146-186
            BsdfRecord br;
            br.wo = to_local(-ray.d, geo.normal);
            br.sampler = &rng;
            bsdf.sample(br);
            if (is_zero(br.f * fabsf(br.wi.z)) || is_zero(br.pdf)) break;
            throughput = throughput * (br.f * fabsf(br.wi.z) / br.pdf);
            Ray nray;
            nray.o = geo.position;
            nray.d = to_world(br.wi, geo.normal);
            nray.tmin = 0.001f;
            nray.tmax = 1e16f;
            Hit nh = s.trace(nray, false);
            ray = nray;
            if (nh.prim < 0) {
                miss(nray);
                float mis = mis_weight(br.pdf, env_pdf);
                env_radiance = env_radiance * (throughput * mis);
                break;
            }
            load_hit(nh, nray);
            if (emitter_index >= 0) {
                const Emitter &em = s.areas[emitter_index];
                V3 le; float epdf;
                em.eval(le, epdf, geo, nray.o);
                if (!is_zero(epdf)) {
                    float mis = (br.type & kDelta) ? 1.f : mis_weight(br.pdf, epdf * em.select_probability);
                    radiance = radiance + throughput * le * mis;
                }
            }
        }
    }
    radiance = radiance + env_radiance;
    out.radiance = radiance;
    return out;
}

static int resolve_threads(int threads) {
    if (threads > 0) return threads;
    unsigned hc = std::thread::hardware_concurrency();
    return hc ? (int)hc : 1;
}

template <class F>
static void parallel_for(uint32_t n, int threads, F fn) {
    threads = resolve_threads(threads);
    if (threads <= 1 || n < 64) {
        for (uint32_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    const uint32_t chunk = 64;
    for (int t = 0; t < threads; t++) {
        pool.emplace_back([&]() {
            for (;;) {
                uint32_t b = next.fetch_add(chunk);
                if (b >= n) break;
                uint32_t e = std::min(n, b + chunk);
                for (uint32_t i = b; i < e; i++) fn(i);
            }
        });
    }
    for (auto &th : pool) th.join();
}

}  // namespace orc

// ======================================================================== C ABI
using namespace orc;

struct oracle_scene {
    Scene s;
};

extern "C" {

int oracle_scene_create(const pt_scene_desc *desc, int build_bvh, oracle_scene **out) {
    if (!out) return PT_ERR_INVALID;
    auto sc = std::make_unique<oracle_scene>();
    int st = build_scene(desc, sc->s);
    if (st != PT_OK) return st;
    if (build_bvh) sc->s.build_bvh();
    *out = sc.release();
    return PT_OK;
}

void oracle_scene_destroy(oracle_scene *scene) { delete scene; }

int oracle_scene_num_prims(const oracle_scene *scene, uint32_t *nt, uint32_t *ns) {
    if (!scene) return PT_ERR_INVALID;
    if (nt) *nt = scene->s.num_tris;
    if (ns) *ns = scene->s.num_spheres;
    return PT_OK;
}

int oracle_scene_num_curves(const oracle_scene *scene, uint32_t *segments, uint32_t *pieces) {
    if (!scene) return PT_ERR_INVALID;
    if (segments) *segments = (uint32_t)(scene->s.curve_cp.size() / 4);
    if (pieces) *pieces = scene->s.num_pieces;
    return PT_OK;
}

// Piece table: 12 floats per piece (c0 xyz, r0, c1 xyz, r1, u0, u1, kind, segment).
int oracle_scene_curve_pieces(const oracle_scene *scene, float *out) {
    if (!scene || !out) return PT_ERR_INVALID;
    for (size_t i = 0; i < scene->s.pieces.size(); i++) {
        const CurvePiece &p = scene->s.pieces[i];
        float *o = out + 12 * i;
        o[0] = p.c0.x; o[1] = p.c0.y; o[2] = p.c0.z; o[3] = p.r0;
        o[4] = p.c1.x; o[5] = p.c1.y; o[6] = p.c1.z; o[7] = p.r1;
        o[8] = p.u0; o[9] = p.u1; o[10] = (float)p.kind; o[11] = (float)p.segment;
    }
    return PT_OK;
}

// Curve KAT (layout of ref_curve in oracle/ref_kat.cpp): per case 16 floats of
// control points (4 x xyzw), u, and a point ps; out 15 floats: position4,
// velocity4, acceleration3, surface normal3 (ps projected as the reference does).
int oracle_curve(uint32_t type, const float *ctrl, const float *u, const float *ps, float *out, uint32_t n) {
    if (type > PT_CURVE_CATMULL_ROM) return PT_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        V4 q[4];
        for (int j = 0; j < 4; j++) q[j] = {ctrl[16 * i + 4 * j], ctrl[16 * i + 4 * j + 1], ctrl[16 * i + 4 * j + 2], ctrl[16 * i + 4 * j + 3]};
        CurvePoly c = curve_poly(type, q);
        V4 p4 = curve_position4(c, u[i]), d4 = curve_velocity4(c, u[i]);
        V3 a3 = curve_acceleration3(c, u[i]);
        V3 nrm = curve_surface_normal(c, u[i], v3(ps[3 * i], ps[3 * i + 1], ps[3 * i + 2]));
        float *o = out + 15 * (size_t)i;
        o[0] = p4.x; o[1] = p4.y; o[2] = p4.z; o[3] = p4.w;
        o[4] = d4.x; o[5] = d4.y; o[6] = d4.z; o[7] = d4.w;
        o[8] = a3.x; o[9] = a3.y; o[10] = a3.z;
        o[11] = nrm.x; o[12] = nrm.y; o[13] = nrm.z; o[14] = 0.f;
    }
    return PT_OK;
}

int oracle_scene_world_triangles(const oracle_scene *scene, float *out) {
    if (!scene || !out) return PT_ERR_INVALID;
    for (size_t i = 0; i < scene->s.tri_p.size(); i++) {
        out[3 * i] = scene->s.tri_p[i].x;
        out[3 * i + 1] = scene->s.tri_p[i].y;
        out[3 * i + 2] = scene->s.tri_p[i].z;
    }
    return PT_OK;
}

int oracle_trace_rays(const oracle_scene *scene, const float *rays, float *hits, uint32_t n, int anyhit,
                      int brute_force, int threads) {
    if (!scene || (!rays && n) || (!hits && n)) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    parallel_for(n, threads, [&](uint32_t i) {
        const float *r = rays + 8 * (size_t)i;
        Ray ray{{r[0], r[1], r[2]}, {r[4], r[5], r[6]}, r[3], r[7]};
        Hit h = (brute_force || s.nodes.empty()) ? s.trace_brute(ray, anyhit != 0) : s.trace_bvh(ray, anyhit != 0);
        float *o = hits + 4 * (size_t)i;
        if (anyhit) {
            o[0] = h.prim >= 0 ? 1.f : 0.f;
            o[1] = o[2] = o[3] = 0.f;
        } else {
            int32_t pid = h.prim;
            o[0] = h.prim >= 0 ? h.t : ray.tmax;
            memcpy(&o[1], &pid, 4);
            o[2] = h.prim >= 0 ? h.u : 0.f;
            o[3] = h.prim >= 0 ? h.v : 0.f;
        }
    });
    return PT_OK;
}

int oracle_camera_rays(const oracle_scene *scene, uint32_t rng_mode, uint32_t seed, float *out) {
    if (!scene || !out) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    uint32_t np = s.width * s.height;
    for (uint32_t p = 0; p < np; p++) {
        Sampler rng;
        rng.init(rng_mode, p, seed);
        Ray r = camera_ray(s, p % s.width, p / s.width, rng);
        float *o = out + 8 * (size_t)p;
        o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z; o[3] = r.tmin;
        o[4] = r.d.x; o[5] = r.d.y; o[6] = r.d.z; o[7] = r.tmax;
    }
    return PT_OK;
}

int oracle_render(const oracle_scene *scene, const pt_render_params *p, float *accum, float *frame, float *albedo,
                  float *normal, float *test, const uint32_t *pixels, uint32_t num_pixels, int threads) {
    if (!scene || !p || !accum) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    uint32_t max_depth = p->max_depth ? p->max_depth : s.max_depth;
    uint32_t n = pixels ? num_pixels : s.width * s.height;
    parallel_for(n, threads, [&](uint32_t i) {
        uint32_t px = pixels ? pixels[i] : i;
        for (uint32_t f = 0; f < p->spp; f++) {
            SampleOut so = trace_path(s, px, p->seed + f, p->rng, max_depth);
            V3 L = so.radiance;
            uint32_t cnt = p->sample_cnt + f;
            if (p->accumulate && cnt > 0) {  // main.cu:190-194
                const float t = 1.f / (cnt + 1.f);
                V3 pre{accum[4 * (size_t)px], accum[4 * (size_t)px + 1], accum[4 * (size_t)px + 2]};
                L = lerp(pre, L, t);
            }
            float *a = accum + 4 * (size_t)px;
            a[0] = L.x; a[1] = L.y; a[2] = L.z; a[3] = 1.f;
            if (frame) {
                float *fr = frame + 4 * (size_t)px;
                fr[0] = L.x; fr[1] = L.y; fr[2] = L.z; fr[3] = 1.f;
            }
            if (albedo) { albedo[3 * (size_t)px] = so.albedo.x; albedo[3 * (size_t)px + 1] = so.albedo.y; albedo[3 * (size_t)px + 2] = so.albedo.z; }
            if (normal) { normal[3 * (size_t)px] = so.normal.x; normal[3 * (size_t)px + 1] = so.normal.y; normal[3 * (size_t)px + 2] = so.normal.z; }
            if (test) test[px] = so.test;
        }
    });
    return PT_OK;
}

int oracle_render_samples(const oracle_scene *scene, const pt_render_params *p, uint32_t frame_seed,
                          const uint32_t *pixels, uint32_t num_pixels, float *out, int threads) {
    if (!scene || !p || !out) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    uint32_t max_depth = p->max_depth ? p->max_depth : s.max_depth;
    uint32_t n = pixels ? num_pixels : s.width * s.height;
    parallel_for(n, threads, [&](uint32_t i) {
        uint32_t px = pixels ? pixels[i] : i;
        SampleOut so = trace_path(s, px, frame_seed, p->rng, max_depth);
        out[3 * (size_t)i] = so.radiance.x;
        out[3 * (size_t)i + 1] = so.radiance.y;
        out[3 * (size_t)i + 2] = so.radiance.z;
    });
    return PT_OK;
}

int oracle_bsdf_eval(const float *bsdf, const float *wo, const float *wi, float *out_f, float *out_pdf, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        LocalBsdf l = LocalBsdf::from_flat(bsdf + 16 * (size_t)i);
        BsdfRecord r;
        r.wo = {wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
        r.wi = {wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]};
        l.eval(r);
        out_f[3 * i] = r.f.x; out_f[3 * i + 1] = r.f.y; out_f[3 * i + 2] = r.f.z;
        out_pdf[i] = r.pdf;
    }
    return PT_OK;
}

int oracle_bsdf_sample(const float *bsdf, const float *wo, uint32_t *rng_state, float *out_wi, float *out_f,
                       float *out_pdf, uint32_t *out_type, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        LocalBsdf l = LocalBsdf::from_flat(bsdf + 16 * (size_t)i);
        Sampler smp;
        smp.mode = PT_RNG_REF_LCG;
        smp.lcg.seed = rng_state[i];
        BsdfRecord r;
        r.wo = {wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
        r.sampler = &smp;
        l.sample(r);
        rng_state[i] = smp.lcg.seed;
        out_wi[3 * i] = r.wi.x; out_wi[3 * i + 1] = r.wi.y; out_wi[3 * i + 2] = r.wi.z;
        out_f[3 * i] = r.f.x; out_f[3 * i + 1] = r.f.y; out_f[3 * i + 2] = r.f.z;
        out_pdf[i] = r.pdf;
        out_type[i] = r.type;
    }
    return PT_OK;
}

int oracle_material_local_bsdf(const pt_material_desc *mat, float u, float v, float *out16) {
    if (!mat || !out16) return PT_ERR_INVALID;
    Material m = Material::from_desc(*mat);
    m.local({u, v}).to_flat(out16);
    return PT_OK;
}

int oracle_rng_stream(uint32_t mode, uint32_t pixel, uint32_t seed, uint32_t n, float *out) {
    Sampler s;
    s.init(mode, pixel, seed);
    for (uint32_t i = 0; i < n; i++) out[i] = s.next();
    return PT_OK;
}

int oracle_pcg32_raw(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t *out) {
    Pcg32 p;
    p.seed(initstate, initseq);
    for (uint32_t i = 0; i < n; i++) out[i] = p.raw();
    return PT_OK;
}

int oracle_emitter_sample(const oracle_scene *scene, int index, const float *in, float *out, uint32_t n) {
    if (!scene) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    const Emitter *e = nullptr;
    if (index >= 0 && (size_t)index < s.areas.size()) e = &s.areas[index];
    else if (index == -1 && s.has_env) e = &s.env;
    if (!e) return PT_ERR_OOB;
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 8 * (size_t)i;
        LocalGeometry g;
        g.position = {q[0], q[1], q[2]};
        g.normal = {q[3], q[4], q[5]};
        Emitter::SampleRecord r;
        e->sample_direct(r, g, {q[6], q[7]});
        float *o = out + 12 * (size_t)i;
        o[0] = r.radiance.x; o[1] = r.radiance.y; o[2] = r.radiance.z;
        o[3] = r.wi.x; o[4] = r.wi.y; o[5] = r.wi.z;
        o[6] = r.pdf; o[7] = r.distance_set ? r.distance : 0.f;
        o[8] = r.pos.x; o[9] = r.pos.y; o[10] = r.pos.z;
        o[11] = r.distance_set ? 1.f : 0.f;
    }
    return PT_OK;
}

int oracle_emitter_table(const oracle_scene *scene, uint32_t *count, float *out, uint32_t cap) {
    if (!scene || !count) return PT_ERR_INVALID;
    const Scene &s = scene->s;
    uint32_t n = (uint32_t)s.areas.size() + (s.has_env ? 1 : 0);
    *count = n;
    for (uint32_t i = 0; i < n && i < cap; i++) {
        const Emitter &e = i < s.areas.size() ? s.areas[i] : s.env;
        out[2 * i] = (float)e.type;
        out[2 * i + 1] = e.select_probability;
    }
    return PT_OK;
}

// util::Camera (framework/util/camera.cpp:7-20): sample_to_camera =
// transpose(inverse(P * T(1,1,0) * S(0.5,0.5,1))) with DirectXMath's
// row-vector PerspectiveFovRH; camera_to_world = the sensor transform.
int oracle_camera_make(float fov_y_deg, float aspect, float near_clip, float far_clip, const float to_world[16],
                       pt_camera_desc *out) {
    if (!out || !to_world || !(aspect > 0.f) || near_clip == far_clip) return PT_ERR_INVALID;
    double fov = (double)(fov_y_deg / 180.f * 3.14159265358979323846f);
    double h = cos(0.5 * fov) / sin(0.5 * fov);
    double w = h / aspect;
    double range = (double)far_clip / ((double)near_clip - (double)far_clip);
    // Row-vector matrices (v' = v * M).
    double P[16] = {w, 0, 0, 0, 0, h, 0, 0, 0, 0, range, -1, 0, 0, range * near_clip, 0};
    double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 1, 1, 0, 1};
    double S[16] = {0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    auto mul = [](const double *a, const double *b, double *c) {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double acc = 0;
                for (int k = 0; k < 4; k++) acc += a[4 * i + k] * b[4 * k + j];
                c[4 * i + j] = acc;
            }
    };
    double PT_[16], A[16], Ainv[16];
    mul(P, T, PT_);
    mul(PT_, S, A);
    mat_inverse_dd(A, Ainv);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out->sample_to_camera[4 * r + c] = (float)Ainv[4 * c + r];  // transpose
    memcpy(out->camera_to_world, to_world, 16 * sizeof(float));
    return PT_OK;
}

// ---- known-answer entry points with the layouts of oracle/ref_kat.cpp ----
int oracle_fresnel_dielectric(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        float ct = 0.f;
        out[2 * i] = dielectric_reflectance(in[2 * i], in[2 * i + 1], ct);
        out[2 * i + 1] = ct;
    }
    return PT_OK;
}
int oracle_fresnel_conductor(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) out[i] = conductor_reflectance(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
    return PT_OK;
}
int oracle_fresnel_diffuse(const float *eta, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) out[i] = diffuse_reflectance(eta[i]);
    return PT_OK;
}
int oracle_ggx(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 9 * (size_t)i;
        V3 wo{q[0], q[1], q[2]}, wh{q[3], q[4], q[5]};
        float a = q[6];
        float *o = out + 7 * (size_t)i;
        o[0] = ggx_d(wh, a);
        o[1] = ggx_g1(wo, a);
        o[2] = ggx_g(wo, wh, a);
        o[3] = ggx_pdf(wo, wh, a);
        V3 smp = ggx_sample(wo, a, {q[7], q[8]});
        o[4] = smp.x; o[5] = smp.y; o[6] = smp.z;
    }
    return PT_OK;
}
int oracle_sampling(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 8 * (size_t)i;
        float *o = out + 20 * (size_t)i;
        V3 nn{q[2], q[3], q[4]}, v{q[5], q[6], q[7]};
        V3 r[6] = {uniform_sample_triangle(q[0], q[1]), uniform_sample_sphere(q[0], q[1]),
                   cosine_sample_hemisphere(q[0], q[1]), uniform_sample_hemisphere(q[0], q[1]), to_local(v, nn),
                   to_world(v, nn)};
        for (int k = 0; k < 6; k++) { o[3 * k] = r[k].x; o[3 * k + 1] = r[k].y; o[3 * k + 2] = r[k].z; }
        V2 tc = sphere_texcoord(v);
        o[18] = tc.x;
        o[19] = tc.y;
    }
    return PT_OK;
}
int oracle_emitter_sample_raw(int kind, const float *params, const float *in, float *out, uint32_t n) {
    Emitter e;
    if (kind == 1) {
        e.type = kEmitTri;
        e.radiance = {params[0], params[1], params[2]};
        e.area = params[3];
        for (int k = 0; k < 3; k++) {
            const float *v = params + 4 + 8 * k;
            e.p[k] = {v[0], v[1], v[2]};
            e.n[k] = {v[3], v[4], v[5]};
            e.uv[k] = {v[6], v[7]};
        }
    } else if (kind == 2) {
        e.type = kEmitSphere;
        e.radiance = {params[0], params[1], params[2]};
        e.area = params[3];
        e.p[0] = {params[4], params[5], params[6]};
        e.radius = params[7];
    } else if (kind == 3) {
        e.type = kEmitConstEnv;
        e.radiance = {params[0], params[1], params[2]};
    } else {
        return PT_ERR_INVALID;
    }
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 8 * (size_t)i;
        LocalGeometry g;
        g.position = {q[0], q[1], q[2]};
        g.normal = {q[3], q[4], q[5]};
        Emitter::SampleRecord r;
        e.sample_direct(r, g, {q[6], q[7]});
        float *o = out + 12 * (size_t)i;
        o[0] = r.radiance.x; o[1] = r.radiance.y; o[2] = r.radiance.z;
        o[3] = r.wi.x; o[4] = r.wi.y; o[5] = r.wi.z;
        o[6] = r.pdf; o[7] = r.distance_set ? r.distance : 0.f;
        o[8] = r.pos.x; o[9] = r.pos.y; o[10] = r.pos.z;
        o[11] = r.distance_set ? 1.f : 0.f;
    }
    return PT_OK;
}
// EnvMapEmitter KAT counterpart of ref_envmap: builds the CDF tables from the
// map (written to tables: row_cdf h+1, col_cdf (w+1)*h, row_weight h,
// normalization 1), then samples (mode 0) or evaluates (mode 1) as
// ref_envmap does.
int oracle_envmap(int mode, const float *pixels, uint32_t w, uint32_t h, float scale, const float *tw, const float *tl,
                  const float *in, float *out, uint32_t n, float *tables) {
    if (!pixels || w < 2 || h < 2) return PT_ERR_INVALID;
    EnvMapData m;
    m.build(pixels, w, h, scale, tw, tl);
    if (tables) {
        float *t = tables;
        std::copy(m.row_cdf.begin(), m.row_cdf.end(), t);
        t += m.row_cdf.size();
        std::copy(m.col_cdf.begin(), m.col_cdf.end(), t);
        t += m.col_cdf.size();
        std::copy(m.row_weight.begin(), m.row_weight.end(), t);
        t += m.row_weight.size();
        *t = m.normalization;
    }
    for (uint32_t i = 0; i < n; i++) {
        if (mode == 0) {
            V3 wi, rad;
            float pdf;
            m.sample({in[2 * i], in[2 * i + 1]}, wi, rad, pdf);
            float *o = out + 7 * (size_t)i;
            o[0] = rad.x; o[1] = rad.y; o[2] = rad.z;
            o[3] = wi.x; o[4] = wi.y; o[5] = wi.z;
            o[6] = pdf;
        } else {
            const float *q = in + 6 * (size_t)i;
            const V3 o3{q[0], q[1], q[2]};
            const V3 d = normalize(V3{q[3], q[4], q[5]});
            V3 rad;
            float pdf;
            m.eval(o3, o3 + d, rad, pdf);
            float *o = out + 4 * (size_t)i;
            o[0] = rad.x; o[1] = rad.y; o[2] = rad.z;
            o[3] = pdf;
        }
    }
    return PT_OK;
}

// SelectOneEmiiter over a probability list (same running sums as the scene table).
int oracle_select_emitter(const float *probs, uint32_t num, int has_env, const float *p, int32_t *out, uint32_t n) {
    std::vector<float> cdf;
    float acc = 0.f;
    for (uint32_t i = 0; i < num; i++) {
        cdf.push_back(acc + probs[i]);
        acc += probs[i];
    }
    for (uint32_t i = 0; i < n; i++) {
        int32_t r = -2;
        for (uint32_t k = 0; k < num; k++)
            if (p[i] <= cdf[k]) { r = (int32_t)k; break; }
        if (r == -2) r = has_env ? -1 : (num ? (int32_t)num - 1 : -2);
        out[i] = r;
    }
    return PT_OK;
}

// The shared trigonometry (pt_trig.h) on the host: fn 0 sin(x), 1 cos(x),
// 2 atan2(y, x), 3 acos(x).
int oracle_trig(uint32_t fn, const float *x, const float *y, float *out, uint32_t n) {
    if (fn > 3) return PT_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        switch (fn) {
            case 0: out[i] = pt_sinf(x[i]); break;
            case 1: out[i] = pt_cosf(x[i]); break;
            case 2: out[i] = pt_atan2f(y[i], x[i]); break;
            default: out[i] = pt_acosf(x[i]); break;
        }
    }
    return PT_OK;
}

}  // extern "C"
