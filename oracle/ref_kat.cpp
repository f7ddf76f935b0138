// ref_kat.cpp -- known-answer entry points built from the REFERENCE's own
// render-layer headers (included from the PupilOptixLab tree at build time,
// never copied), compiled for the host.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile builds this into
// oracle/_ref/libpupil_ref.so when the reference tree is present; the script
// tests/golden/make_golden.py calls it to write the golden vectors under
// tests/golden/, against which the oracle restatement (oracle/pt_oracle.cpp)
// and the CUDA kernels are pinned.
//
// Headers exercised (paths relative to the PupilOptixLab tree):
//   framework/render/material/bsdf/{diffuse,dielectric,rough_dielectric,
//     conductor,rough_conductor,plastic,rough_plastic}.h
//   framework/render/material/{fresnel,ggx}.h
//   framework/optix/util.h
//   framework/render/emitter.h, framework/render/emitter/{area,sphere,env}.h
//   framework/render/curve.h (curve interpolators, SurfaceNormal)
// Shims (oracle/ref_shims): optix.h, cuda/texture.h, cuda/random.h.
// The material dispatch (optix_material.h:70-91) uses MSVC-only token pasting,
// so the switch over the seven Local types below restates it.

#include "render/material/bsdf/bsdf.h"
#include "render/material/fresnel.h"
#include "render/material/ggx.h"
#include "optix/util.h"
#include "render/emitter.h"
#include "render/curve.h"

#include <cstdint>
#include <cstring>

using namespace Pupil;
using namespace Pupil::optix;
using namespace Pupil::optix::material;

namespace {

float3 col(const float *p) { return make_float3(p[0], p[1], p[2]); }

// Flat record layout: include/pt_api.h (PT_LOCAL_BSDF_FLOATS).
template <class F>
void with_local(const float *b, F &&fn) {
    unsigned type = static_cast<unsigned>(b[0]);
    switch (type) {
        case 1: {
            Diffuse::Local l;
            l.reflectance = col(b + 6);
            fn(l);
        } break;
        case 2: {
            Dielectric::Local l;
            l.eta = b[2];
            l.specular_reflectance = col(b + 6);
            l.specular_transmittance = col(b + 9);
            fn(l);
        } break;
        case 3: {
            RoughDielectric::Local l;
            l.alpha = b[1];
            l.eta = b[2];
            l.specular_reflectance = col(b + 6);
            l.specular_transmittance = col(b + 9);
            fn(l);
        } break;
        case 4: {
            Conductor::Local l;
            l.specular_reflectance = col(b + 6);
            l.eta = col(b + 9);
            l.k = col(b + 12);
            fn(l);
        } break;
        case 5: {
            RoughConductor::Local l;
            l.alpha = b[1];
            l.specular_reflectance = col(b + 6);
            l.eta = col(b + 9);
            l.k = col(b + 12);
            fn(l);
        } break;
        case 6: {
            Plastic::Local l;
            l.eta = b[2];
            l.int_fdr = b[3];
            l.specular_sampling_weight = b[4];
            l.nonlinear = b[5] != 0.f;
            l.diffuse_reflectance = col(b + 6);
            l.specular_reflectance = col(b + 9);
            fn(l);
        } break;
        case 7: {
            RoughPlastic::Local l;
            l.alpha = b[1];
            l.eta = b[2];
            l.int_fdr = b[3];
            l.specular_sampling_weight = b[4];
            l.nonlinear = b[5] != 0.f;
            l.diffuse_reflectance = col(b + 6);
            l.specular_reflectance = col(b + 9);
            fn(l);
        } break;
        default:
            break;
    }
}

void put3(float *o, float3 v) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
}

}  // namespace

extern "C" {

int ref_bsdf_eval(const float *bsdf, const float *wo, const float *wi, float *out_f, float *out_pdf, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        BsdfSamplingRecord r;
        r.wo = col(wo + 3 * i);
        r.wi = col(wi + 3 * i);
        with_local(bsdf + 16 * i, [&](auto &l) {
            l.GetBsdf(r);
            l.GetPdf(r);
        });
        put3(out_f + 3 * i, r.f);
        out_pdf[i] = r.pdf;
    }
    return 0;
}

int ref_bsdf_sample(const float *bsdf, const float *wo, uint32_t *rng, float *out_wi, float *out_f, float *out_pdf,
                    uint32_t *out_type, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        cuda::Random random;
        random.SetSeed(rng[i]);
        BsdfSamplingRecord r;
        r.wi = make_float3(0.f);  // the record leaves wi unset on early returns
        r.wo = col(wo + 3 * i);
        r.sampler = &random;
        with_local(bsdf + 16 * i, [&](auto &l) { l.Sample(r); });
        rng[i] = random.GetSeed();
        put3(out_wi + 3 * i, r.wi);
        put3(out_f + 3 * i, r.f);
        out_pdf[i] = r.pdf;
        out_type[i] = static_cast<uint32_t>(r.sampled_type);
    }
    return 0;
}

int ref_rng_stream(uint32_t pixel, uint32_t seed, uint32_t n, float *out) {
    cuda::Random r;
    r.Init(4, pixel, seed);
    for (uint32_t i = 0; i < n; i++) out[i] = r.Next();
    return 0;
}

// in: (eta, cos_i) pairs; out: (F, cos_t) pairs.
int ref_fresnel_dielectric(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        float ct = 0.f;
        out[2 * i] = fresnel::DielectricReflectance(in[2 * i], in[2 * i + 1], ct);
        out[2 * i + 1] = ct;
    }
    return 0;
}

// in: (eta, k, cos_i); out: F.
int ref_fresnel_conductor(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) out[i] = fresnel::ConductorReflectance(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
    return 0;
}

int ref_fresnel_diffuse(const float *eta, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) out[i] = fresnel::DiffuseReflectance(eta[i]);
    return 0;
}

// in: wo(3) wh(3) alpha xi(2) = 9 floats; out: D, G1(wo), G(wo, wh), Pdf, Sample(3) = 7 floats.
int ref_ggx(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 9 * i;
        float3 wo = col(q), wh = col(q + 3);
        float a = q[6];
        float2 xi = make_float2(q[7], q[8]);
        float *o = out + 7 * i;
        o[0] = ggx::D(wh, a);
        o[1] = ggx::G1(wo, a);
        o[2] = ggx::G(wo, wh, a);
        o[3] = ggx::Pdf(wo, wh, a);
        put3(o + 4, ggx::Sample(wo, a, xi));
    }
    return 0;
}

// in: u1 u2 n(3) v(3) = 8 floats; out: triangle(3) sphere(3) cosine(3)
// uniform-hemisphere(3) to_local(3) to_world(3) sphere_texcoord(2) = 20 floats.
int ref_sampling(const float *in, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 8 * i;
        float *o = out + 20 * i;
        float3 nn = col(q + 2), v = col(q + 5);
        put3(o, UniformSampleTriangle(q[0], q[1]));
        put3(o + 3, UniformSampleSphere(q[0], q[1]));
        put3(o + 6, CosineSampleHemisphere(q[0], q[1]));
        put3(o + 9, UniformSampleHemisphere(q[0], q[1]));
        put3(o + 12, ToLocal(v, nn));
        put3(o + 15, ToWorld(v, nn));
        float2 tc = GetSphereTexcoord(v);
        o[18] = tc.x;
        o[19] = tc.y;
    }
    return 0;
}

// Emitter SampleDirect KAT.  kind 1 = triangle area (params: radiance 3,
// area 1, v0 pos/normal/uv 8, v1 8, v2 8 = 28), 2 = sphere (radiance 3, area,
// centre 3, radius = 8), 3 = constant environment (radiance 3).
// in: shading point pos(3) normal(3) xi(2); out as oracle_emitter_sample.
int ref_emitter_sample(int kind, const float *params, const float *in, float *out, uint32_t n) {
    Emitter e;
    std::memset(static_cast<void *>(&e), 0, sizeof(e));  // the union leaves the shim texture's fields unset
    switch (kind) {
        case 1:
            e.type = EEmitterType::TriArea;
            e.area.radiance.rgb = col(params);
            e.area.area = params[3];
            e.area.geo.v0.pos = col(params + 4);
            e.area.geo.v0.normal = col(params + 7);
            e.area.geo.v0.tex = make_float2(params[10], params[11]);
            e.area.geo.v1.pos = col(params + 12);
            e.area.geo.v1.normal = col(params + 15);
            e.area.geo.v1.tex = make_float2(params[18], params[19]);
            e.area.geo.v2.pos = col(params + 20);
            e.area.geo.v2.normal = col(params + 23);
            e.area.geo.v2.tex = make_float2(params[26], params[27]);
            break;
        case 2:
            e.type = EEmitterType::Sphere;
            e.sphere.radiance.rgb = col(params);
            e.sphere.area = params[3];
            e.sphere.geo.center = col(params + 4);
            e.sphere.geo.radius = params[7];
            break;
        case 3:
            e.type = EEmitterType::ConstEnv;
            e.const_env.color = col(params);
            e.const_env.center = make_float3(0.f);
            break;
        default:
            return 1;
    }
    for (uint32_t i = 0; i < n; i++) {
        const float *q = in + 8 * i;
        LocalGeometry g;
        g.position = col(q);
        g.normal = col(q + 3);
        g.texcoord = make_float2(0.f);
        EmitterSampleRecord r;
        r.distance = -1.f;  // marks "not set by SampleDirect"
        e.SampleDirect(r, g, make_float2(q[6], q[7]));
        float *o = out + 12 * i;
        put3(o, r.radiance);
        put3(o + 3, r.wi);
        o[6] = r.pdf;
        o[7] = r.distance >= 0.f ? r.distance : 0.f;
        put3(o + 8, r.pos);
        o[11] = r.distance >= 0.f ? 1.f : 0.f;
    }
    return 0;
}

// EnvMapEmitter KAT (render/emitter/env.h): the reference's SampleDirect
// (mode 0; in: xi 2 per query; out: radiance 3, wi 3, pdf 1) and Eval
// (mode 1; in: scatter point 3, direction 3; out: radiance 3, pdf 1) over a
// bilinear, wrapping RGBA float map and CDF tables given by the caller.
int ref_envmap(int mode, const float *pixels, uint32_t w, uint32_t h, float scale, const float *tw, const float *tl,
               const float *row_cdf, const float *col_cdf, const float *row_weight, float normalization,
               const float *in, float *out, uint32_t n) {
    EnvMapEmitter e{};
    e.radiance.pixels = pixels;
    e.radiance.w = w;
    e.radiance.h = h;
    e.radiance.address = 0;
    e.radiance.filter = 1;
    e.center = make_float3(0.f);
    e.map_size = make_uint2(w, h);
    e.row_cdf.SetData(reinterpret_cast<CUdeviceptr>(row_cdf), h + 1);
    e.col_cdf.SetData(reinterpret_cast<CUdeviceptr>(col_cdf), (size_t)(w + 1) * h);
    e.row_weight.SetData(reinterpret_cast<CUdeviceptr>(row_weight), h);
    e.to_world.r0 = col(tw);
    e.to_world.r1 = col(tw + 3);
    e.to_world.r2 = col(tw + 6);
    e.to_local.r0 = col(tl);
    e.to_local.r1 = col(tl + 3);
    e.to_local.r2 = col(tl + 6);
    e.normalization = normalization;
    e.scale = scale;
    for (uint32_t i = 0; i < n; i++) {
        if (mode == 0) {
            const float *q = in + 2 * i;
            LocalGeometry g;
            g.position = make_float3(0.f);
            g.normal = make_float3(0.f, 1.f, 0.f);
            EmitterSampleRecord r;
            e.SampleDirect(r, g, make_float2(q[0], q[1]));
            float *o = out + 7 * i;
            put3(o, r.radiance);
            put3(o + 3, r.wi);
            o[6] = r.pdf;
        } else {
            const float *q = in + 6 * i;
            LocalGeometry g;
            const float3 o3 = col(q), d = normalize(col(q + 3));
            g.position = o3 + d;  // as __miss__default builds it (main.cu:204-208)
            EmitEvalRecord r;
            e.Eval(r, g, o3);
            float *o = out + 4 * i;
            put3(o, r.radiance);
            o[3] = r.pdf;
        }
    }
    return 0;
}

// EmitterGroup::SelectOneEmiiter over an area list with the given select
// probabilities (and an optional env); returns the selected index per p
// (-1 = env).
// Curve interpolators and SurfaceNormal as Geometry::GetHitLocalGeometry
// (framework/render/geometry.h:101-172) picks them per curve type.  Per case:
// ctrl 16 floats (4 control points xyzw), u, ps xyz; out 15 floats: Position4,
// Velocity4, Acceleration3, SurfaceNormal (of a copy of ps), 0.
int ref_curve(uint32_t type, const float *ctrl, const float *u, const float *ps, float *out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        float4 q[4];
        for (int j = 0; j < 4; j++)
            q[j] = make_float4(ctrl[16 * i + 4 * j], ctrl[16 * i + 4 * j + 1], ctrl[16 * i + 4 * j + 2], ctrl[16 * i + 4 * j + 3]);
        float3 p = make_float3(ps[3 * i], ps[3 * i + 1], ps[3 * i + 2]);
        float4 p4, d4;
        float3 a3, nrm;
        const float t = u[i];
        if (type == 0) {
            LinearInterpolator c;
            c.Initialize(q);
            p4 = c.Position4(t); d4 = c.Velocity4(t); a3 = c.Acceleration3(t);
            nrm = SurfaceNormal(c, t, p);
        } else if (type == 1) {
            QuadraticInterpolator c;
            c.InitializeFromBSpline(q);
            p4 = c.Position4(t); d4 = c.Velocity4(t); a3 = c.Acceleration3(t);
            nrm = SurfaceNormal(c, t, p);
        } else {
            CubicInterpolator c;
            if (type == 2) c.InitializeFromBSpline(q);
            else c.InitializeFromCatrom(q);
            p4 = c.Position4(t); d4 = c.Velocity4(t); a3 = c.Acceleration3(t);
            nrm = SurfaceNormal(c, t, p);
        }
        float *o = out + 15 * (size_t)i;
        o[0] = p4.x; o[1] = p4.y; o[2] = p4.z; o[3] = p4.w;
        o[4] = d4.x; o[5] = d4.y; o[6] = d4.z; o[7] = d4.w;
        o[8] = a3.x; o[9] = a3.y; o[10] = a3.z;
        o[11] = nrm.x; o[12] = nrm.y; o[13] = nrm.z; o[14] = 0.f;
    }
    return 0;
}

int ref_select_emitter(const float *probs, uint32_t num, int has_env, const float *p, int32_t *out, uint32_t n) {
    static thread_local Emitter *areas = nullptr;
    delete[] areas;
    areas = new Emitter[num ? num : 1];
    for (uint32_t i = 0; i < num; i++) {
        areas[i].type = EEmitterType::TriArea;
        areas[i].select_probability = probs[i];
    }
    Emitter env;
    env.type = EEmitterType::ConstEnv;
    EmitterGroup g;
    g.areas.SetData(reinterpret_cast<CUdeviceptr>(areas), num);
    if (has_env) g.env.SetData(reinterpret_cast<CUdeviceptr>(&env));
    for (uint32_t i = 0; i < n; i++) {
        const Emitter &s = g.SelectOneEmiiter(p[i]);
        out[i] = (&s == &env) ? -1 : static_cast<int32_t>(&s - areas);
    }
    return 0;
}

}  // extern "C"
