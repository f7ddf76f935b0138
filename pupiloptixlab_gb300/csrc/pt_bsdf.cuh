// pt_bsdf.cuh -- device material, texture, emitter and sampling math of the
// GB300 wavefront path tracer (FP32 throughout).
//
// Semantics follow PupilOptixLab's render layer; each function names the
// reference file:line it implements (paths relative to the PupilOptixLab
// tree).  Expressions keep the reference's operation order, and the
// trigonometric functions are the library's own (pt_trig.h), so that, compiled
// with -fmad=false, results equal a host build of the same arithmetic bit for
// bit.
#pragma once

#include "pt_device.cuh"
#include "pt_trig.h"

namespace ptd {

// ---------------------------------------------------------------- sampling utils
// framework/optix/util.h:33-183
PT_DI float3 uniform_sample_triangle(float u1, float u2) {  // util.h:33-36
    float s = sqrtf(u1);
    return f3(1.f - s, s * (1.f - u2), u2 * s);
}
PT_DI float3 uniform_sample_sphere(float u1, float u2) {  // util.h:38-43
    float z = 1.f - 2.f * u1;
    float sin_theta = sqrtf(fmaxf(0.f, 1.f - z * z));
    float phi = 2.f * kPi * u2;
    return f3(sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), z);
}
PT_DI float3 cosine_sample_hemisphere(float u1, float u2) {  // util.h:45-54
    float sin_theta = sqrtf(u1);
    float phi = 2.0f * kPi * u2;
    return f3(sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), sqrtf(fmaxf(0.f, 1.f - sin_theta * sin_theta)));
}
PT_DI float cosine_hemisphere_pdf(float3 v) { return v.z > 0.f ? kInvPi * v.z : 0.f; }  // util.h:55-57
PT_DI float3 uniform_sample_hemisphere(float u1, float u2) {                         // util.h:59-69
    float z = 1.f - 2.f * u1;
    float sin_theta = sqrtf(fmaxf(0.f, 1.f - z * z));
    float phi = 2.0f * kPi * u2;
    return f3(sin_theta * pt_cosf(phi), sin_theta * pt_sinf(phi), fabsf(z));
}
PT_DI float uniform_hemisphere_pdf(float3 v) { return v.z > 0.f ? kInvPi * 0.5f : 0.f; }  // util.h:70-72
PT_DI float3 reflect_local(float3 v) { return f3(-v.x, -v.y, v.z); }                     // util.h:74-78
PT_DI float3 reflect(float3 v, float3 n) { return -v + 2.f * dot(v, n) * n; }            // util.h:80-82
PT_DI float3 refract_local(float3 v, float cos_t, float eta) {                           // util.h:84-87
    float scale = -(cos_t < 0.f ? 1.f / eta : eta);
    return normalize(f3(scale * v.x, scale * v.y, cos_t));
}
PT_DI float3 refract(float3 v, float3 n, float cos_t, float eta) {  // util.h:89-92
    if (cos_t < 0.f) eta = 1.f / eta;
    return n * (dot(v, n) * eta + cos_t) - v * eta;
}
PT_DI void build_onb(float3 n, float3 &b1, float3 &b2) {  // util.h:95-101 (Duff et al. 2017)
    float sign = copysignf(1.f, n.z);
    float a = -1.f / (sign + n.z);
    float b = n.x * n.y * a;
    b1 = f3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    b2 = f3(b, sign + n.y * n.y * a, -n.y);
}
PT_DI float3 to_local(float3 v, float3 n) {  // util.h:103-108
    float3 b1, b2;
    build_onb(n, b1, b2);
    return f3(dot(v, b1), dot(v, b2), dot(v, n));
}
PT_DI float3 to_world(float3 v, float3 n) {  // util.h:110-115
    float3 b1, b2;
    build_onb(n, b1, b2);
    return b1 * v.x + b2 * v.y + n * v.z;
}
PT_DI float2 sphere_texcoord(float3 p) {  // util.h:117-128
    float phi = pt_atan2f(p.y, p.x);
    phi = phi < 0.f ? phi + kPi * 2.f : phi;
    float theta = pt_acosf(p.z);
    return make_float2(phi * kInvPi * 0.5f, theta * kInvPi);
}
PT_DI float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
PT_DI float mis_weight(float x, float y) { return x / (x + y); }  // util.h:165-167 (balance heuristic)
PT_DI bool is_zero(float v) { return fabsf(v) < kEps; }            // util.h:169-179
PT_DI bool is_zero(float3 v) { return fabsf(v.x) < kEps && fabsf(v.y) < kEps && fabsf(v.z) < kEps; }

// ---------------------------------------------------------------- Fresnel
// framework/render/material/fresnel.h:7-56
PT_DI float dielectric_reflectance(float eta, float cos_i, float &cos_t) {
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
PT_DI float dielectric_reflectance(float eta, float cos_i) {
    float c;
    return dielectric_reflectance(eta, cos_i, c);
}
PT_DI float conductor_reflectance1(float eta, float k, float cos_i) {
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
PT_DI float3 conductor_reflectance(float3 eta, float3 k, float cos_i) {
    return f3(conductor_reflectance1(eta.x, k.x, cos_i), conductor_reflectance1(eta.y, k.y, cos_i),
              conductor_reflectance1(eta.z, k.z, cos_i));
}

// ---------------------------------------------------------------- GGX
// framework/render/material/ggx.h:6-64, isotropic, visible-normal sampling.
PT_DI float ggx_lambda(float3 w, float alpha) {
    float a2 = alpha * alpha;
    float3 v2 = w * w;
    return (-1.f + sqrtf(1.f + (v2.x + v2.y) * a2 / v2.z)) / 2.f;
}
PT_DI float ggx_g1(float3 w, float alpha) { return 1.f / (1.f + ggx_lambda(w, alpha)); }
PT_DI float ggx_g(float3 wi, float3 wo, float alpha) { return ggx_g1(wi, alpha) * ggx_g1(wo, alpha); }
PT_DI float ggx_d(float3 wh, float alpha) {
    float a2 = alpha * alpha;
    float3 v2 = wh * wh;
    float t = (v2.x + v2.y) / a2 + v2.z;
    return 1.f / (kPi * a2 * t * t);
}
PT_DI float ggx_pdf(float3 wo, float3 wh, float alpha) {
    return ggx_d(wh, alpha) * ggx_g1(wo, alpha) * dot(wo, wh) / fabsf(wo.z);
}
PT_DI float3 ggx_sample(float3 wo, float alpha, float2 xi) {
    float3 vh = normalize(f3(alpha * wo.x, alpha * wo.y, wo.z));
    float3 t1v = wo.z < 0.9999f ? normalize(cross(f3(0.f, 0.f, 1.f), vh)) : f3(1.f, 0.f, 0.f);
    float3 t2v = cross(vh, t1v);
    float r = sqrtf(xi.x);
    float phi = 2.f * kPi * xi.y;
    float t1 = r * pt_cosf(phi);
    float t2 = r * pt_sinf(phi);
    float s = 0.5f * (1.f + vh.z);
    t2 = (1.f - s) * sqrtf(1.f - t1 * t1) + s * t2;
    float3 nh = t1 * t1v + t2 * t2v + sqrtf(fmaxf(0.f, 1.f - t1 * t1 - t2 * t2)) * vh;
    float3 ne = f3(alpha * nh.x, alpha * nh.y, fmaxf(0.f, nh.z));
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

// BsdfSamplingRecord (framework/render/material/bsdf/bsdf.h:26-36).
struct BsdfRecord {
    float3 wi, wo, f;
    float pdf;
    uint32_t type;
};

// Material::LocalBsdf (optix_material.h:23-112) in flat form:
// a = reflectance / specular_reflectance / diffuse_reflectance,
// b = specular_transmittance / conductor eta / plastic specular_reflectance,
// c = conductor k.
struct LocalBsdf {
    uint32_t type;
    float alpha, eta, int_fdr, spec_weight;
    bool nonlinear;
    float3 a, b, c;

    PT_DI float3 plastic_diffuse() const {  // plastic.h:38, rough_plastic.h:138
        return a / (1.f - (nonlinear ? a * int_fdr : f3s(int_fdr)));
    }
    PT_DI float specular_prob(float fo) const {  // plastic.h:48-50
        return (fo * spec_weight) / (fo * spec_weight + (1.f - fo) * (1.f - spec_weight));
    }

    PT_DI void get_bsdf(BsdfRecord &r) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:12-18
                float3 f = f3s(0.f);
                if (r.wi.z > 0.f && r.wo.z > 0.f) f = a * kInvPi;
                r.f = f;
            } break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:21-30
                r.f = f3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float3 wh = normalize(r.wi + r.wo);
                float3 fo = conductor_reflectance(b, c, dot(r.wo, wh));
                r.f = a * ggx_d(wh, alpha) * fo * ggx_g(r.wi, r.wo, alpha) / (4.f * r.wi.z * r.wo.z);
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:21-49
                r.f = f3s(0.f);
                if (is_zero(r.wo.z)) return;
                bool refl = r.wo.z * r.wi.z > 0.f;
                float3 wh = refl ? normalize(r.wo + r.wi) : normalize(r.wo + r.wi * (r.wo.z > 0.f ? eta : 1.f / eta));
                wh = wh * (wh.z > 0.f ? 1.f : -1.f);
                float F = dielectric_reflectance(eta, dot(r.wo, wh));
                float G = ggx_g(r.wi, r.wo, alpha);
                float D = ggx_d(wh, alpha);
                if (refl) {
                    r.f = a * F * G * D / (4.f * fabsf(r.wi.z) * fabsf(r.wo.z));
                } else {
                    float e = r.wo.z > 0.f ? eta : 1.f / eta;
                    float sd = dot(r.wo, wh) + e * dot(r.wi, wh);
                    r.f = b * fabsf((1.f - F) * D * G * dot(r.wi, wh) * dot(r.wo, wh) / (sd * sd * r.wi.z * r.wo.z));
                }
            } break;
            case PT_MAT_PLASTIC: {  // plastic.h:32-41
                r.f = f3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float fi = dielectric_reflectance(eta, r.wi.z);
                float3 diff = plastic_diffuse();
                r.f = diff * (1.f - fi) * (1.f - fo) * cosine_hemisphere_pdf(r.wi) / (eta * eta * r.wi.z);
            } break;
            case PT_MAT_ROUGH_PLASTIC: {  // rough_plastic.h:22-35
                r.f = f3s(0.f);
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float3 wh = normalize(r.wi + r.wo);
                r.f = b * dielectric_reflectance(eta, dot(wh, r.wo)) * ggx_d(wh, alpha) * ggx_g(r.wi, r.wo, alpha) /
                      (4.f * r.wo.z * r.wi.z);
                float fi = dielectric_reflectance(eta, r.wi.z);
                float3 diff = plastic_diffuse();
                r.f = r.f + diff * (1.f - fi) * (1.f - fo) * kInvPi / (eta * eta);
            } break;
            default:  // dielectric.h:23-25, conductor.h:19-21: delta lobes evaluate to 0
                r.f = f3s(0.f);
                break;
        }
    }

    PT_DI void get_pdf(BsdfRecord &r) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:20-25
                float pdf = 0.f;
                if (r.wi.z > 0.f && r.wo.z > 0.f) pdf = cosine_hemisphere_pdf(r.wi);
                r.pdf = pdf;
            } break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:32-38
                r.pdf = 0.f;
                if (r.wi.z <= 0.f || r.wo.z <= 0.f) return;
                float3 wh = normalize(r.wi + r.wo);
                wh = normalize(wh);
                r.pdf = ggx_pdf(r.wo, wh, alpha) / (4.f * dot(r.wo, wh));
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:51-71
                bool refl = r.wo.z * r.wi.z > 0.f;
                float3 wh;
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
                float3 wo = r.wo * (r.wo.z > 0.f ? 1.f : -1.f);
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
                float3 wh = normalize(r.wi + r.wo);
                r.pdf = sp * ggx_pdf(r.wo, wh, alpha) / (4.f * dot(r.wi, wh));
                r.pdf += dp * cosine_hemisphere_pdf(r.wi);
            } break;
            default:
                r.pdf = 0.f;
                break;
        }
    }

    // LocalBsdf::Eval (optix_material.h:81-91)
    PT_DI void eval(BsdfRecord &r) const {
        get_bsdf(r);
        get_pdf(r);
    }

    // LocalBsdf::Sample (optix_material.h:70-79). The record must come in with
    // f = 0, pdf = 0, type = Unknown and wi = 0.
    PT_DI void sample(BsdfRecord &r, Sampler &rng) const {
        switch (type) {
            case PT_MAT_DIFFUSE: {  // diffuse.h:27-33
                float2 xi = rng.next2();
                r.wi = cosine_sample_hemisphere(xi.x, xi.y);
                get_pdf(r);
                get_bsdf(r);
                r.type = kDiffuseReflection;
            } break;
            case PT_MAT_DIELECTRIC: {  // dielectric.h:27-44
                float cos_t;
                float F = dielectric_reflectance(eta, r.wo.z, cos_t);
                if (rng.next() < F) {
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
                float3 fr = conductor_reflectance(b, c, r.wo.z);
                r.f = a * fr / fabsf(r.wi.z);
                r.type = kDeltaReflection;
            } break;
            case PT_MAT_ROUGH_CONDUCTOR: {  // rough_conductor.h:40-46 (tagged DiffuseReflection, as the reference)
                float2 xi = rng.next2();
                r.wi = reflect(r.wo, ggx_sample(r.wo, alpha, xi));
                get_pdf(r);
                get_bsdf(r);
                r.type = kDiffuseReflection;
            } break;
            case PT_MAT_ROUGH_DIELECTRIC: {  // rough_dielectric.h:73-96
                float2 xi = rng.next2();
                float3 wo = r.wo * (r.wo.z > 0.f ? 1.f : -1.f);
                float3 wh = ggx_sample(wo, alpha, xi);
                float cos_t = 0.f;
                float F = dielectric_reflectance(eta, dot(r.wo, wh), cos_t);
                if (rng.next() < F) {
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
                float2 xi = rng.next2();
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
                    float3 diff = plastic_diffuse();
                    r.f = diff * (1.f - fi) * (1.f - fo) * cosine_hemisphere_pdf(r.wi) / (eta * eta * r.wi.z);
                    r.pdf = cosine_hemisphere_pdf(r.wi) * (1.f - sp);
                }
            } break;
            case PT_MAT_ROUGH_PLASTIC: {  // rough_plastic.h:53-80
                r.wi = f3s(0.f);
                if (r.wo.z <= 0.f) return;
                float fo = dielectric_reflectance(eta, r.wo.z);
                float sp = specular_prob(fo);
                float2 xi = rng.next2();
                if (xi.y < sp) {
                    xi.y /= sp;
                    float3 wh = ggx_sample(r.wo, alpha, xi);
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

    PT_DI float3 albedo() const { return type == PT_MAT_UNKNOWN ? f3s(0.f) : a; }  // optix_material.h:93-111

    PT_DI static LocalBsdf from_flat(const float *p) {
        LocalBsdf l;
        l.type = static_cast<uint32_t>(p[0]);
        l.alpha = p[1];
        l.eta = p[2];
        l.int_fdr = p[3];
        l.spec_weight = p[4];
        l.nonlinear = p[5] != 0.f;
        l.a = f3(p[6], p[7], p[8]);
        l.b = f3(p[9], p[10], p[11]);
        l.c = f3(p[12], p[13], p[14]);
        return l;
    }
};

// ---------------------------------------------------------------- textures and materials
// cuda::Texture::Sample (framework/cuda/texture.h:33-57); RGB and checkerboard.
PT_DI float3 texture_sample(const DevTexture &t, float2 uv) {
    float4 tex = make_float4(uv.x, uv.y, 0.f, 1.f);
    float tx = dot4(t.r0, tex), ty = dot4(t.r1, tex);
    if (t.type == PT_TEX_CHECKERBOARD) {
        tx = tx - (tx > 0.f ? floorf(tx) : ceilf(tx));
        ty = ty - (ty > 0.f ? floorf(ty) : ceilf(ty));
        if (tx < 0.f) tx += 1.f;
        if (ty < 0.f) ty += 1.f;
        bool first = tx > 0.5f ? ty > 0.5f : !(ty > 0.5f);
        return first ? f3(t.c0[0], t.c0[1], t.c0[2]) : f3(t.c1[0], t.c1[1], t.c1[2]);
    }
    if (t.type == PT_TEX_BITMAP) {
        const float4 c = tex2D<float4>(static_cast<cudaTextureObject_t>(t.obj), tx, ty);
        return f3(c.x, c.y, c.z);
    }
    return f3(t.c0[0], t.c0[1], t.c0[2]);
}

// Material::GetLocalBsdf (optix_material.h:119-131) and each type's GetLocal.
PT_DI LocalBsdf material_local(const DevMaterial &m, float2 uv) {
    LocalBsdf l;
    l.type = m.type;
    l.alpha = 0.f;
    l.eta = 1.f;
    l.int_fdr = 0.f;
    l.spec_weight = 0.f;
    l.nonlinear = false;
    l.a = l.b = l.c = f3s(0.f);
    switch (m.type) {
        case PT_MAT_DIFFUSE:
            l.a = texture_sample(m.tex[0], uv);
            break;
        case PT_MAT_DIELECTRIC:
        case PT_MAT_ROUGH_DIELECTRIC:
            l.eta = m.eta;
            l.a = texture_sample(m.tex[0], uv);
            l.b = texture_sample(m.tex[1], uv);
            if (m.type == PT_MAT_ROUGH_DIELECTRIC) l.alpha = texture_sample(m.tex[2], uv).x;
            break;
        case PT_MAT_CONDUCTOR:
        case PT_MAT_ROUGH_CONDUCTOR:
            l.a = texture_sample(m.tex[0], uv);
            l.b = texture_sample(m.tex[1], uv);
            l.c = texture_sample(m.tex[2], uv);
            if (m.type == PT_MAT_ROUGH_CONDUCTOR) l.alpha = texture_sample(m.tex[3], uv).x;
            break;
        case PT_MAT_PLASTIC:
        case PT_MAT_ROUGH_PLASTIC:
            l.eta = m.eta;
            l.nonlinear = m.nonlinear != 0;
            l.int_fdr = m.int_fdr;
            l.spec_weight = m.spec_weight;
            l.a = texture_sample(m.tex[0], uv);
            l.b = texture_sample(m.tex[1], uv);
            if (m.type == PT_MAT_ROUGH_PLASTIC) l.alpha = texture_sample(m.tex[2], uv).x;
            break;
        default:
            break;
    }
    return l;
}

// ---------------------------------------------------------------- emitters
struct EmitterSample {  // EmitterSampleRecord (framework/render/emitter/types.h:17-26)
    float3 radiance, wi;
    float distance, pdf;
};

PT_DI uint32_t emitter_type(const DevEmitter &e) { return __float_as_uint(e.a.x); }

// An area emitter's radiance at texture coordinate uv: its constant RGB
// value, or its radiance texture (AreaEmitter radiance.Sample, area.h:22,43;
// sphere.h:20,40; Emitter::GetRadiance at a primary hit, main.cu:90-95).
PT_DI float3 emitter_radiance(const DevEmitter &e, const DevTexture *emit_tex, float2 uv) {
    const uint32_t t = __float_as_uint(e.rad.w);
    return t ? texture_sample(emit_tex[t - 1u], uv) : xyz(e.rad);
}

// Emitter::SampleDirect (emitter.h:124-139; area.h:17-35, sphere.h:14-32, env.h:69-80).
// pdf stays 0 when the sample is unusable; is_delta is always false here.
PT_DI void emitter_sample_direct(const DevEmitter &e, const DevTexture *emit_tex, float3 pos, float3 nrm, float2 xi,
                                 EmitterSample &r) {
    r.pdf = 0.f;
    r.distance = 0.f;
    uint32_t type = emitter_type(e);
    if (type == kEmitTri || type == kEmitSphere) {
        float3 position, normal;
        // the texture coordinates matter only for a textured radiance (and
        // cost two inverse trigonometric functions on a sphere)
        const bool textured = __float_as_uint(e.rad.w) != 0u;
        float2 tex = make_float2(0.f, 0.f);
        if (type == kEmitTri) {
            float3 t = uniform_sample_triangle(xi.x, xi.y);
            position = xyz(e.p0) * t.x + xyz(e.p1) * t.y + xyz(e.p2) * t.z;
            normal = normalize(xyz(e.n0) * t.x + xyz(e.n1) * t.y + xyz(e.n2) * t.z);
            // vertex texture coordinates (u in p*.w, v in n*.w), area.h:21
            if (textured)
                tex = make_float2(e.p0.w * t.x + e.p1.w * t.y + e.p2.w * t.z, e.n0.w * t.x + e.n1.w * t.y + e.n2.w * t.z);
        } else {
            float3 t = uniform_sample_sphere(xi.x, xi.y);
            position = t * e.a.w + xyz(e.p0);
            normal = normalize(t);
            if (textured) tex = sphere_texcoord(t);  // of the world-space sample direction, sphere.h:19
        }
        r.radiance = emitter_radiance(e, emit_tex, tex);
        r.wi = normalize(position - pos);
        float NoL = dot(nrm, r.wi);
        float LNoL = dot(normal, -r.wi);
        if (NoL > 0.f && LNoL > 0.f) {
            float d = length(position - pos);
            r.pdf = d * d / (LNoL * e.a.z);
            r.distance = d;
        }
    } else if (type == kEmitConstEnv) {
        float3 local_wi = uniform_sample_hemisphere(xi.x, xi.y);
        r.wi = to_world(local_wi, nrm);
        r.pdf = uniform_hemisphere_pdf(local_wi);
        r.distance = kMaxDistance;
        r.radiance = xyz(e.rad);
    }
}

// First i in [0, n) with x <= cdf[i], else n (the linear scans of
// EnvMapEmitter::SampleDirect, env.h:24-31, over non-decreasing running sums).
PT_DI uint32_t cdf_first_geq(const float *cdf, uint32_t n, float x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (x <= __ldg(cdf + mid)) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

PT_DI float3 envmap_lookup(const DevEnvMap &m, float2 tex) {
    const float4 c = tex2D<float4>(static_cast<cudaTextureObject_t>(m.tex), tex.x, tex.y);
    return f3(c.x, c.y, c.z) * m.scale;
}

// EnvMapEmitter::SampleDirect (env.h:23-49).  As in the reference the search
// returns the index after the interval xi falls in (row_cdf[0] = 0), so the
// last row selects index h; the reference then reads one row past the column
// table and row_weight[h], past their ends.  Here those two reads use row
// h - 1 instead.
PT_DI void envmap_sample_direct(const DevEnvMap &m, float2 xi, EmitterSample &r) {
    const uint32_t row = cdf_first_geq(m.row_cdf, m.h, xi.x);
    const uint32_t crow = min(row, m.h - 1);
    const uint32_t col = cdf_first_geq(m.col_cdf + (size_t)crow * (m.w + 1), m.w - 1, xi.y);
    const float phi = static_cast<float>(col) * kPi * 2.f / static_cast<float>(m.w);
    const float theta = static_cast<float>(row) * kPi / static_cast<float>(m.h);
    const float st = pt_sinf(theta);
    const float3 local = f3(st * pt_sinf(kPi - phi), pt_cosf(theta), st * pt_cosf(kPi - phi));
    r.wi = f3(dot(xyz(m.to_world[0]), local), dot(xyz(m.to_world[1]), local), dot(xyz(m.to_world[2]), local));
    r.distance = kMaxDistance;
    r.radiance = envmap_lookup(m, make_float2(phi * 0.5f * kInvPi, theta * kInvPi));
    r.pdf = luminance(r.radiance) * __ldg(m.row_weight + crow) * m.normalization / fmaxf(1e-4f, fabsf(st));
    if (r.pdf < 0.f) r.pdf = 0.f;
}

// EnvMapEmitter::Eval (env.h:51-64) for a ray leaving scatter_pos along d:
// the emitter point is scatter_pos + d, as the miss program builds it
// (main.cu:204-208).
PT_DI void envmap_eval(const DevEnvMap &m, float3 scatter_pos, float3 d, float3 &radiance, float &pdf) {
    const float3 pos = scatter_pos + d;
    float3 dir = normalize(pos - scatter_pos);
    dir = f3(dot(xyz(m.to_local[0]), dir), dot(xyz(m.to_local[1]), dir), dot(xyz(m.to_local[2]), dir));
    const float phi = kPi - pt_atan2f(dir.x, dir.z);
    const float theta = pt_acosf(dir.y);
    const float2 tex = make_float2(phi * 0.5f * kInvPi, theta * kInvPi);
    uint32_t row = static_cast<uint32_t>(tex.y * static_cast<float>(m.h));
    row = min(row, m.h - 2u);
    radiance = envmap_lookup(m, tex);
    const float w0 = __ldg(m.row_weight + row), w1 = __ldg(m.row_weight + row + 1);
    const float t = tex.y * static_cast<float>(m.h) - 1.f * static_cast<float>(row);
    pdf = luminance(radiance) * (w0 + t * (w1 - w0)) * m.normalization / fmaxf(1e-4f, fabsf(pt_sinf(theta)));
}

// Emitter::Eval at an emitter hit (area.h:37-45, sphere.h:34-42): pdf 0 if it faces away.
PT_DI float emitter_eval_pdf(const DevEmitter &e, float3 emit_pos, float3 emit_nrm, float3 scatter_pos) {
    float3 dir = normalize(scatter_pos - emit_pos);
    float LNoL = dot(emit_nrm, dir);
    if (LNoL > 0.f) {
        float d = length(scatter_pos - emit_pos);
        return d * d / (LNoL * e.a.z);
    }
    return 0.f;
}

// EmitterGroup::SelectOneEmiiter (emitter.h:110-136): the first area emitter
// whose running probability sum reaches p (binary search over the same running
// sums), else the environment, else the last area emitter.  Returns the area
// index, -1 for the environment, -2 for none.
PT_DI int select_emitter(const DevScene &s, float p) {
    uint32_t n = s.num_emitters;
    if (n > 0 && p <= s.emitter_cdf[n - 1]) {
        uint32_t lo = 0, hi = n - 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (p <= s.emitter_cdf[mid]) hi = mid;
            else lo = mid + 1;
        }
        return static_cast<int>(lo);
    }
    if (s.has_env) return -1;
    return n > 0 ? static_cast<int>(n - 1) : -2;
}

}  // namespace ptd
