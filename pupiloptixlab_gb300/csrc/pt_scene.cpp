// pt_scene.cpp -- C-ABI glue, context, scene flattening and upload.
//
// Scene set-up replaces world::World::LoadScene (framework/world/world.cpp:
// 108-146), RenderObject (framework/world/render_object.cpp:10-65), the
// emitter table builder (framework/world/emitter.cpp:169-243,321-390) and the
// camera upload (framework/world/camera.cpp:72-92).  Instances are flattened
// to world space here, on the host, with contraction disabled, so that the
// world-space triangles are bit-identical to the CPU oracle's.

#include "pt_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>

namespace {
thread_local std::string g_last_error;

using ptd::DevEmitter;
using ptd::DevInstance;
using ptd::DevMaterial;
using ptd::DevTexture;

struct H3 {
    float x, y, z;
};
inline H3 h3(float x, float y, float z) { return {x, y, z}; }
inline H3 sub(H3 a, H3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float hdot(H3 a, H3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline H3 hcross(H3 a, H3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float hlen(H3 v) { return sqrtf(hdot(v, v)); }

// util::Transform::TransformPoint (framework/util/transform.cpp:100-107) for affine matrices.
inline H3 xform_point(const float m[16], H3 p) {
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
inline H3 xform_vec(const float n[9], H3 v) {
    return {n[0] * v.x + n[1] * v.y + n[2] * v.z, n[3] * v.x + n[4] * v.y + n[5] * v.z, n[6] * v.x + n[7] * v.y + n[8] * v.z};
}

void inverse4(const double *a, double out[16]) {  // cofactor inverse in double
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
void inverse4f(const float *m, double out[16]) {
    double a[16];
    for (int i = 0; i < 16; i++) a[i] = m[i];
    inverse4(a, out);
}
// Inverse transpose of the upper 3x3, rounded to float (normal matrix).
void normal_matrix(const double inv[16], float nm[9]) {
    const int idx[9] = {0, 4, 8, 1, 5, 9, 2, 6, 10};
    for (int k = 0; k < 9; k++) nm[k] = (float)inv[idx[k]];
}

float luminance(H3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }  // optix/util.h:161-163
// fresnel::DiffuseReflectance (framework/render/material/fresnel.h:58-85): published
// fits of Egan & Hilgeman (eta < 1) and d'Eon & Irving (eta >= 1).
float diffuse_reflectance(float eta) {
    if (eta < 1) return -1.4399f * (eta * eta) + 0.7099f * eta + 0.6681f + 0.0636f / eta;
    float i1 = 1.0f / eta, i2 = i1 * i1, i3 = i2 * i1, i4 = i3 * i1, i5 = i4 * i1;
    return 0.919317f - 3.4793f * i1 + 6.75335f * i2 - 7.80989f * i3 + 4.98554f * i4 - 1.36881f * i5;
}
H3 tex_average(const pt_texture_desc &t) {  // GetPixelAverage (optix_material.cpp:8-35)
    if (t.type == PT_TEX_CHECKERBOARD)
        return {(t.color0[0] + t.color1[0]) * 0.5f, (t.color0[1] + t.color1[1]) * 0.5f, (t.color0[2] + t.color1[2]) * 0.5f};
    if (t.type == PT_TEX_BITMAP) {  // RGB sums in row-major order, divided by (1.f * h) * w
        float r = 0.f, g = 0.f, b = 0.f;
        size_t idx = 0;
        for (uint32_t y = 0; y < t.height; y++)
            for (uint32_t x = 0; x < t.width; x++) {
                r += t.pixels[idx++];
                g += t.pixels[idx++];
                b += t.pixels[idx++];
                idx++;
            }
        const float n = 1.f * t.height * t.width;
        return {r / n, g / n, b / n};
    }
    return {t.color0[0], t.color0[1], t.color0[2]};
}

// GetWeight (world/emitter.cpp:77-101): the selection weight of an area
// emitter's radiance texture per unit area -- the largest channel of an RGB
// value, the mean of the two patches' largest channels of a checkerboard, and
// for a bitmap the mean largest channel over its pixels, summed in the
// reference's loop order (i over the width, j over the height, pixel
// i * width + j).  For a bitmap wider than high that index runs past the last
// pixel, where the reference reads beyond its array; here it reads the last
// pixel instead.
float emitter_weight(const pt_texture_desc &t) {
    auto max3 = [](float r, float g, float b) { return r > g ? (r > b ? r : b) : (g > b ? g : b); };
    if (t.type == PT_TEX_CHECKERBOARD) {
        float w1 = max3(t.color0[0], t.color0[1], t.color0[2]);
        float w2 = max3(t.color1[0], t.color1[1], t.color1[2]);
        return (w1 + w2) * 0.5f;
    }
    if (t.type == PT_TEX_BITMAP) {
        const size_t w = t.width, h = t.height, last = w * h - 1;
        float sum = 0.f;
        for (size_t i = 0; i < w; i++)
            for (size_t j = 0; j < h; j++) {
                const size_t px = std::min(i * w + j, last);
                sum += max3(t.pixels[px * 4 + 0], t.pixels[px * 4 + 1], t.pixels[px * 4 + 2]);
            }
        return sum / (1.f * w * h);
    }
    return max3(t.color0[0], t.color0[1], t.color0[2]);
}

// A float4 CUDA texture object over an RGBA float bitmap, made as the
// reference makes it (framework/cuda/texture.cpp:60-102): normalized
// coordinates, element reads, the given address and filter modes.
int bitmap_texture(pt_scene *s, const float *pixels, uint32_t w, uint32_t h, uint32_t address, uint32_t filter,
                   cudaTextureObject_t *out) {
    for (const auto &b : s->bitmaps)
        if (b.pixels == pixels && b.w == w && b.h == h && b.address == address && b.filter == filter) {
            *out = b.obj;
            return PT_OK;
        }
    pt_scene::BitmapTexture b{pixels, w, h, address, filter, nullptr, 0};
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float4>();
    PT_CUDA_TRY(cudaMallocArray(&b.array, &ch, w, h));
    s->bitmaps.push_back(b);  // owned from here on (freed with the scene)
    const size_t pitch = (size_t)w * 4 * sizeof(float);
    PT_CUDA_TRY(cudaMemcpy2DToArray(b.array, 0, 0, pixels, pitch, pitch, h, cudaMemcpyHostToDevice));
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = b.array;
    cudaTextureDesc td{};
    td.addressMode[0] = static_cast<cudaTextureAddressMode>(address);
    td.addressMode[1] = static_cast<cudaTextureAddressMode>(address);
    td.filterMode = static_cast<cudaTextureFilterMode>(filter);
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    td.maxAnisotropy = 1;
    td.maxMipmapLevelClamp = 99;
    td.minMipmapLevelClamp = 0;
    td.mipmapFilterMode = cudaFilterModePoint;
    td.borderColor[0] = 1.0f;
    td.sRGB = 0;
    PT_CUDA_TRY(cudaCreateTextureObject(&s->bitmaps.back().obj, &rd, &td, nullptr));
    *out = s->bitmaps.back().obj;
    return PT_OK;
}

DevTexture to_dev(const pt_texture_desc &t) {
    DevTexture d{};
    d.type = t.type;
    for (int i = 0; i < 3; i++) {
        d.c0[i] = t.color0[i];
        d.c1[i] = t.color1[i];
    }
    d.r0 = make_float4(t.uv_transform[0], t.uv_transform[1], t.uv_transform[2], t.uv_transform[3]);
    d.r1 = make_float4(t.uv_transform[4], t.uv_transform[5], t.uv_transform[6], t.uv_transform[7]);
    return d;
}

bool affine(const float *m) { return m[12] == 0.f && m[13] == 0.f && m[14] == 0.f && m[15] == 1.f; }

template <class T>
int upload(DevBuf &b, const std::vector<T> &v) {
    size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    int st = b.ensure(bytes);
    if (st != PT_OK) return st;
    if (!v.empty()) PT_CUDA_TRY(cudaMemcpy(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PT_OK;
}

int validate(const pt_scene_desc *d) {
    if (!d) { pt_set_error("scene descriptor is NULL"); return PT_ERR_INVALID; }
    if ((d->num_meshes && !d->meshes) || (d->num_spheres && !d->spheres) || (d->num_materials && !d->materials) ||
        (d->num_instances && !d->instances) || (d->num_curves && !d->curves)) {
        pt_set_error("scene descriptor has a non-zero count with a NULL array");
        return PT_ERR_INVALID;
    }
    if (d->width == 0 || d->height == 0) { pt_set_error("film size must be non-zero"); return PT_ERR_INVALID; }
    if ((uint64_t)d->width * d->height > 0x7fffffffu) {  // path slots and pixel indices are 32-bit
        pt_set_error("film of %u x %u pixels: at most 2^31 - 1 pixels are supported", d->width, d->height);
        return PT_ERR_UNSUPPORTED;
    }
    for (uint32_t i = 0; i < d->num_materials; i++) {
        const pt_material_desc &m = d->materials[i];
        if (m.type < PT_MAT_DIFFUSE || m.type > PT_MAT_ROUGH_PLASTIC) {
            pt_set_error("material %u has unknown type %u", i, m.type);
            return PT_ERR_INVALID;
        }
        for (int k = 0; k < 4; k++) {
            const pt_texture_desc &t = m.tex[k];
            if (t.type != PT_TEX_RGB && t.type != PT_TEX_CHECKERBOARD && t.type != PT_TEX_BITMAP) {
                pt_set_error("material %u texture %d: unknown texture type %u", i, k, t.type);
                return PT_ERR_INVALID;
            }
            if (t.type == PT_TEX_BITMAP &&
                (!t.pixels || !t.width || !t.height || t.address_mode > PT_TEX_ADDRESS_MIRROR || t.filter > PT_TEX_FILTER_LINEAR)) {
                pt_set_error("material %u texture %d: bitmap without pixels, of zero size or with unknown modes", i, k);
                return PT_ERR_INVALID;
            }
        }
    }
    for (uint32_t i = 0; i < d->num_meshes; i++) {
        const pt_mesh_desc &m = d->meshes[i];
        if ((m.num_vertices && !m.positions) || (m.num_triangles && !m.indices)) {
            pt_set_error("mesh %u has NULL positions or indices", i);
            return PT_ERR_INVALID;
        }
        for (uint64_t t = 0; t < 3ull * m.num_triangles; t++)
            if (m.indices[t] >= m.num_vertices) {
                pt_set_error("mesh %u index %llu out of range (%u >= %u)", i, (unsigned long long)t, m.indices[t], m.num_vertices);
                return PT_ERR_OOB;
            }
        for (uint64_t v = 0; v < 3ull * m.num_vertices; v++)
            if (!std::isfinite(m.positions[v])) {
                pt_set_error("mesh %u has a non-finite vertex coordinate", i);
                return PT_ERR_INVALID;
            }
    }
    for (uint32_t i = 0; i < d->num_curves; i++) {
        const pt_curves_desc &c = d->curves[i];
        if (c.type > PT_CURVE_CATMULL_ROM) { pt_set_error("curves %u: unknown curve type %u", i, c.type); return PT_ERR_INVALID; }
        if ((c.num_points && (!c.positions || !c.radii)) || (c.num_segments && !c.segments)) {
            pt_set_error("curves %u has NULL positions, radii or segments", i);
            return PT_ERR_INVALID;
        }
        const uint32_t deg = ptd::curve_degree(c.type);
        for (uint32_t k = 0; k < c.num_segments; k++)
            if ((uint64_t)c.segments[k] + deg >= c.num_points) {
                pt_set_error("curves %u segment %u: control points %u..%u out of range (%u points)", i, k, c.segments[k],
                             c.segments[k] + deg, c.num_points);
                return PT_ERR_OOB;
            }
        for (uint64_t v = 0; v < 3ull * c.num_points; v++)
            if (!std::isfinite(c.positions[v])) { pt_set_error("curves %u has a non-finite position", i); return PT_ERR_INVALID; }
        for (uint32_t v = 0; v < c.num_points; v++)
            if (!(c.radii[v] >= 0.f) || !std::isfinite(c.radii[v])) {
                pt_set_error("curves %u point %u: radius must be finite and >= 0", i, v);
                return PT_ERR_INVALID;
            }
    }
    for (uint32_t i = 0; i < d->num_instances; i++) {
        const pt_instance_desc &in = d->instances[i];
        if (in.material >= d->num_materials) { pt_set_error("instance %u: material out of range", i); return PT_ERR_OOB; }
        if (in.shape_type == PT_SHAPE_MESH) {
            if (in.shape_index >= d->num_meshes) { pt_set_error("instance %u: mesh out of range", i); return PT_ERR_OOB; }
        } else if (in.shape_type == PT_SHAPE_SPHERE) {
            if (in.shape_index >= d->num_spheres) { pt_set_error("instance %u: sphere out of range", i); return PT_ERR_OOB; }
            if (!(d->spheres[in.shape_index].radius > 0.f)) { pt_set_error("instance %u: sphere radius must be > 0", i); return PT_ERR_INVALID; }
        } else if (in.shape_type == PT_SHAPE_CURVES) {
            if (in.shape_index >= d->num_curves) { pt_set_error("instance %u: curves out of range", i); return PT_ERR_OOB; }
            if (in.is_emitter) { pt_set_error("instance %u: curves cannot be emitters", i); return PT_ERR_UNSUPPORTED; }
        } else {
            pt_set_error("instance %u: unknown shape type %u", i, in.shape_type);
            return PT_ERR_INVALID;
        }
        if (in.is_emitter && in.radiance_textured) {
            const pt_texture_desc &t = in.radiance_tex;
            if (t.type != PT_TEX_RGB && t.type != PT_TEX_CHECKERBOARD && t.type != PT_TEX_BITMAP) {
                pt_set_error("instance %u: unknown emitter radiance texture type %u", i, t.type);
                return PT_ERR_INVALID;
            }
            if (t.type == PT_TEX_BITMAP &&
                (!t.pixels || !t.width || !t.height || t.address_mode > PT_TEX_ADDRESS_MIRROR || t.filter > PT_TEX_FILTER_LINEAR)) {
                pt_set_error("instance %u: emitter radiance bitmap without pixels, of zero size or with unknown modes", i);
                return PT_ERR_INVALID;
            }
        }
        if (!affine(in.to_world)) { pt_set_error("instance %u: to_world must be affine", i); return PT_ERR_INVALID; }
        for (int k = 0; k < 16; k++)
            if (!std::isfinite(in.to_world[k])) { pt_set_error("instance %u: non-finite transform", i); return PT_ERR_INVALID; }
    }
    // primitives after instancing; curve segments count once here (each gets
    // at least one piece when visible), their pieces are counted as they are made
    uint64_t nprim = 0;
    for (uint32_t i = 0; i < d->num_instances; i++) {
        const pt_instance_desc &in = d->instances[i];
        nprim += in.shape_type == PT_SHAPE_MESH     ? d->meshes[in.shape_index].num_triangles
                 : in.shape_type == PT_SHAPE_SPHERE ? 1u
                                                    : 0u;
    }
    if (nprim > ptd::kMaxPrimitives) {
        pt_set_error("scene has %llu primitives after instancing; at most %u are supported", (unsigned long long)nprim,
                     ptd::kMaxPrimitives);
        return PT_ERR_UNSUPPORTED;
    }
    if (d->env.type != PT_ENV_NONE && d->env.type != PT_ENV_CONST && d->env.type != PT_ENV_MAP) {
        pt_set_error("environment type %u not supported", d->env.type);
        return PT_ERR_UNSUPPORTED;
    }
    if (d->env.type == PT_ENV_MAP && (!d->env.pixels || d->env.width < 2 || d->env.height < 2)) {
        pt_set_error("environment map without pixels or smaller than 2x2");
        return PT_ERR_INVALID;
    }
    return PT_OK;
}

void set_camera(pt_scene *s, const pt_camera_desc &c) {
    for (int r = 0; r < 4; r++) {
        s->dev.s2c[r] = make_float4(c.sample_to_camera[4 * r], c.sample_to_camera[4 * r + 1], c.sample_to_camera[4 * r + 2],
                                    c.sample_to_camera[4 * r + 3]);
        s->dev.c2w[r] = make_float4(c.camera_to_world[4 * r], c.camera_to_world[4 * r + 1], c.camera_to_world[4 * r + 2],
                                    c.camera_to_world[4 * r + 3]);
    }
    float cm = std::max({fabsf(c.camera_to_world[3]), fabsf(c.camera_to_world[7]), fabsf(c.camera_to_world[11])});
    s->scene_mag = std::max(s->scene_mag, cm);
}

// Environment map: texture object (bilinear, wrap) and the luminance CDF
// tables of BuildEnvMapCdfTable (framework/world/emitter.cpp:107-149), with
// the same float arithmetic in the same order.
int build_env_map(pt_scene *s, const pt_env_desc &e) {
    const size_t w = e.width, h = e.height;
    std::vector<float> col_cdf((w + 1) * h), row_cdf(h + 1), row_weight(h);
    size_t ci = 0, ri = 0;
    float row_sum = 0.f;
    row_cdf[ri++] = 0.f;
    for (size_t y = 0; y < h; ++y) {
        float col_sum = 0.f;
        col_cdf[ci++] = 0.f;
        for (size_t x = 0; x < w; ++x) {
            const size_t px = y * w + x;
            const float r = e.pixels[px * 4 + 0], g = e.pixels[px * 4 + 1], b = e.pixels[px * 4 + 2];
            col_sum += 0.2126f * r + 0.7152f * g + 0.0722f * b;  // GetLuminance
            col_cdf[ci++] = col_sum;
        }
        for (size_t x = 1; x < w; ++x) col_cdf[ci - x - 1] /= col_sum;
        col_cdf[ci - 1] = 1.f;
        const float weight = std::sin((y + 0.5f) * 3.14159265358979323846f / h);
        row_weight[y] = weight;
        row_sum += col_sum * weight;
        row_cdf[ri++] = row_sum;
    }
    for (size_t y = 1; y < h; ++y) row_cdf[ri - y - 1] /= row_sum;
    row_cdf[ri - 1] = 1.f;
    int st;
    if ((st = upload(s->env_row_cdf, row_cdf)) != PT_OK || (st = upload(s->env_col_cdf, col_cdf)) != PT_OK ||
        (st = upload(s->env_row_weight, row_weight)) != PT_OK)
        return st;
    cudaTextureObject_t obj = 0;
    if ((st = bitmap_texture(s, e.pixels, e.width, e.height, PT_TEX_ADDRESS_WRAP, PT_TEX_FILTER_LINEAR, &obj)) != PT_OK)
        return st;
    ptd::DevEnvMap &m = s->dev.envmap;
    m.tex = static_cast<unsigned long long>(obj);
    m.row_cdf = s->env_row_cdf.as<float>();
    m.col_cdf = s->env_col_cdf.as<float>();
    m.row_weight = s->env_row_weight.as<float>();
    m.w = e.width;
    m.h = e.height;
    m.normalization = 1.f / (row_sum * (2.f * 3.14159265358979323846f / w) * (3.14159265358979323846f / h));
    m.scale = e.scale;
    double inv[16];
    inverse4f(e.to_world, inv);
    for (int r = 0; r < 3; r++) {
        m.to_world[r] = make_float4(e.to_world[4 * r], e.to_world[4 * r + 1], e.to_world[4 * r + 2], 0.f);
        m.to_local[r] = make_float4((float)inv[4 * r], (float)inv[4 * r + 1], (float)inv[4 * r + 2], 0.f);
    }
    return PT_OK;
}

int build_scene(pt_scene *s, const pt_scene_desc *d) {
    int st = validate(d);
    if (st != PT_OK) return st;
    s->desc_shallow = *d;
    s->desc_shallow.meshes = nullptr;
    s->desc_shallow.spheres = nullptr;
    s->desc_shallow.materials = nullptr;
    s->desc_shallow.instances = nullptr;
    s->desc_shallow.curves = nullptr;

    std::vector<float4> vpos, vnrm, prims;
    std::vector<float2> vuv;
    std::vector<uint32_t> tri_vidx, prim_inst;
    std::vector<DevInstance> insts(d->num_instances);
    s->mesh_num_vertices.resize(d->num_meshes);
    s->total_mesh_vertices = 0;
    for (uint32_t i = 0; i < d->num_meshes; i++) {
        s->mesh_num_vertices[i] = d->meshes[i].num_vertices;
        s->total_mesh_vertices += d->meshes[i].num_vertices;
    }

    float mag = 0.f;
    uint32_t ntri = 0;
    // triangles first, in instance order
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        DevInstance &in = insts[ii];
        memset(&in, 0, sizeof(in));
        in.material = id.material;
        in.flags = id.flags & (PT_INST_FLIP_NORMALS | PT_INST_FLIP_TEXCOORDS);
        in.emitter_offset = -1;
        double inv[16];
        inverse4f(id.to_world, inv);
        in.inv0 = make_float4((float)inv[0], (float)inv[1], (float)inv[2], (float)inv[3]);
        in.inv1 = make_float4((float)inv[4], (float)inv[5], (float)inv[6], (float)inv[7]);
        in.inv2 = make_float4((float)inv[8], (float)inv[9], (float)inv[10], (float)inv[11]);
        if (id.shape_type != PT_SHAPE_MESH) continue;
        const pt_mesh_desc &m = d->meshes[id.shape_index];
        if (m.normals) in.flags |= ptd::kInstHasNormals;
        if (m.texcoords) in.flags |= ptd::kInstHasUvs;
        uint32_t voff = (uint32_t)vpos.size();
        in.prim_offset = ntri;
        MeshInstanceRef ref{ii, id.shape_index, voff, ntri, {}};
        memcpy(ref.to_world, id.to_world, sizeof(ref.to_world));
        s->mesh_instances.push_back(ref);
        float nm[9];
        normal_matrix(inv, nm);
        for (uint32_t v = 0; v < m.num_vertices; v++) {
            H3 p = xform_point(id.to_world, h3(m.positions[3 * v], m.positions[3 * v + 1], m.positions[3 * v + 2]));
            vpos.push_back(make_float4(p.x, p.y, p.z, 0.f));
            mag = std::max({mag, fabsf(p.x), fabsf(p.y), fabsf(p.z)});
            if (m.normals) {
                H3 n = xform_vec(nm, h3(m.normals[3 * v], m.normals[3 * v + 1], m.normals[3 * v + 2]));
                vnrm.push_back(make_float4(n.x, n.y, n.z, 0.f));
            } else {
                vnrm.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
            }
            vuv.push_back(m.texcoords ? make_float2(m.texcoords[2 * v], m.texcoords[2 * v + 1]) : make_float2(0.f, 0.f));
        }
        for (uint32_t t = 0; t < m.num_triangles; t++) {
            uint32_t pid = ntri + t;
            uint32_t a = voff + m.indices[3 * t], b = voff + m.indices[3 * t + 1], c = voff + m.indices[3 * t + 2];
            tri_vidx.push_back(a);
            tri_vidx.push_back(b);
            tri_vidx.push_back(c);
            prim_inst.push_back(ii);
            float4 pa = vpos[a], pb = vpos[b], pc = vpos[c];
            int32_t ip = (int32_t)pid;
            float idf;
            memcpy(&idf, &ip, 4);
            prims.push_back(make_float4(pa.x, pa.y, pa.z, idf));
            prims.push_back(make_float4(pb.x, pb.y, pb.z, 0.f));
            prims.push_back(make_float4(pc.x, pc.y, pc.z, 0.f));
        }
        ntri += m.num_triangles;
    }
    // spheres after all triangles
    uint32_t nsph = 0;
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (id.shape_type != PT_SHAPE_SPHERE) continue;
        DevInstance &in = insts[ii];
        const pt_sphere_desc &sp = d->spheres[id.shape_index];
        H3 c = h3(sp.center[0], sp.center[1], sp.center[2]);
        H3 cw = xform_point(id.to_world, c);
        H3 pw = xform_point(id.to_world, h3(c.x + sp.radius, c.y, c.z));
        float r = hlen(sub(cw, pw));  // world/emitter.cpp:231-237
        uint32_t pid = ntri + nsph;
        in.flags |= ptd::kInstSphere;
        in.prim_offset = pid;
        in.sphere = make_float4(cw.x, cw.y, cw.z, r);
        in.obj_center = make_float4(c.x, c.y, c.z, 0.f);
        prim_inst.push_back(ii);
        uint32_t bits = pid | 0x80000000u;
        float idf;
        memcpy(&idf, &bits, 4);
        prims.push_back(make_float4(cw.x, cw.y, cw.z, idf));
        prims.push_back(make_float4(r, 0.f, 0.f, 0.f));
        prims.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
        mag = std::max({mag, fabsf(cw.x) + r, fabsf(cw.y) + r, fabsf(cw.z) + r});
        nsph++;
    }
    // round-cone pieces of the curve segments after the spheres
    uint32_t nseg = 0, npiece = 0;
    std::vector<uint32_t> curve_seg;
    std::vector<float4> curve_cp;
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (id.shape_type != PT_SHAPE_CURVES) continue;
        DevInstance &in = insts[ii];
        const pt_curves_desc &cv = d->curves[id.shape_index];
        in.flags |= ptd::kInstCurve | (cv.type << ptd::kInstCurveTypeShift);
        in.prim_offset = ntri + nsph + npiece;
        const float *m = id.to_world;
        const float scale = hlen(h3(m[0], m[4], m[8]));  // length of the transformed x axis
        const uint32_t deg = ptd::curve_degree(cv.type);
        for (uint32_t i = 0; i < cv.num_segments; i++, nseg++) {
            const uint32_t first = cv.segments[i];
            float4 q[4] = {};
            float rmax = 0.f;
            for (uint32_t j = 0; j <= deg; j++) {
                const uint32_t v = first + j;
                H3 p = xform_point(m, h3(cv.positions[3 * v], cv.positions[3 * v + 1], cv.positions[3 * v + 2]));
                q[j] = make_float4(p.x, p.y, p.z, cv.radii[v] * scale);
                rmax = std::max(rmax, q[j].w);
            }
            for (int j = 0; j < 4; j++) curve_cp.push_back(q[j]);
            if (!(rmax > 0.f)) continue;  // an invisible segment gets no pieces
            const bool strand_first = i == 0 || cv.segments[i - 1] + 1 != first;
            const bool strand_last = i + 1 == cv.num_segments || cv.segments[i + 1] != first + 1;
            const ptd::CurveSeg sg = ptd::curve_segment(cv.type, q);
            const uint32_t np = ptd::curve_piece_count(sg, rmax);
            if ((uint64_t)ntri + nsph + npiece + np > ptd::kMaxPrimitives) {
                pt_set_error("scene has more than %u primitives (curve pieces included)", ptd::kMaxPrimitives);
                return PT_ERR_UNSUPPORTED;
            }
            for (uint32_t k = 0; k < np; k++) {
                const float u0 = (float)k / (float)np, u1 = (float)(k + 1) / (float)np;
                const float4 p0 = ptd::curve_pos(sg, u0), p1 = ptd::curve_pos(sg, u1);
                int kind = ptd::kPieceCurve;
                if (cv.type == PT_CURVE_LINEAR) {  // round caps at every vertex, one sphere per vertex
                    kind |= ptd::kPieceSphere0;
                    if (strand_last) kind |= ptd::kPieceSphere1;
                } else {  // smooth joints; open ends at the strand's ends
                    if (k > 0 || !strand_first) kind |= ptd::kPieceSphere0;
                    kind |= ptd::kPieceClampU;
                }
                const float r0 = std::max(p0.w, 0.f), r1 = std::max(p1.w, 0.f);
                const uint32_t bits = (ntri + nsph + npiece) | 0x80000000u;
                float idf, kindf;
                memcpy(&idf, &bits, 4);
                memcpy(&kindf, &kind, 4);
                prims.push_back(make_float4(p0.x, p0.y, p0.z, idf));
                prims.push_back(make_float4(r0, r1, u0, kindf));
                prims.push_back(make_float4(p1.x, p1.y, p1.z, u1));
                prim_inst.push_back(ii);
                curve_seg.push_back(nseg);
                mag = std::max({mag, fabsf(p0.x) + r0, fabsf(p0.y) + r0, fabsf(p0.z) + r0, fabsf(p1.x) + r1,
                                fabsf(p1.y) + r1, fabsf(p1.z) + r1});
                npiece++;
            }
        }
    }
    s->num_tris = ntri;
    s->num_spheres = nsph;
    s->num_curve_segments = nseg;
    s->num_curve_pieces = npiece;
    s->num_prims = ntri + nsph + npiece;
    s->num_vertices = (uint32_t)vpos.size();
    s->scene_mag = std::max(mag, 1e-6f);

    // materials with the host precompute (optix_material.cpp:87-132)
    std::vector<DevMaterial> mats(d->num_materials);
    for (uint32_t i = 0; i < d->num_materials; i++) {
        const pt_material_desc &m = d->materials[i];
        DevMaterial &dm = mats[i];
        memset(&dm, 0, sizeof(dm));
        dm.type = m.type;
        dm.twosided = m.twosided ? 1 : 0;
        dm.nonlinear = m.nonlinear ? 1 : 0;
        dm.eta = m.int_ior / m.ext_ior;
        if (m.type == PT_MAT_PLASTIC || m.type == PT_MAT_ROUGH_PLASTIC) {
            float dl = luminance(tex_average(m.tex[0]));
            float sl = luminance(tex_average(m.tex[1]));
            dm.spec_weight = sl / (sl + dl);
            dm.int_fdr = diffuse_reflectance(1.f / dm.eta);
        }
        for (int k = 0; k < 4; k++) {
            dm.tex[k] = to_dev(m.tex[k]);
            if (m.tex[k].type == PT_TEX_BITMAP) {
                cudaTextureObject_t obj = 0;
                const pt_texture_desc &t = m.tex[k];
                int st = bitmap_texture(s, t.pixels, t.width, t.height, t.address_mode, t.filter, &obj);
                if (st != PT_OK) return st;
                dm.tex[k].obj = static_cast<unsigned long long>(obj);
            }
        }
    }

    // emissive instances in instance order (world/emitter.cpp:169-263)
    std::vector<DevTexture> emit_tex;
    s->emitter_sources.clear();
    s->has_emissive_mesh = false;
    uint32_t n_area = 0;
    for (uint32_t ii = 0; ii < d->num_instances; ii++) {
        const pt_instance_desc &id = d->instances[ii];
        if (!id.is_emitter) continue;
        DevInstance &in = insts[ii];
        in.emitter_offset = (int32_t)n_area;
        EmitterSource src;
        memcpy(src.radiance, id.radiance, sizeof(src.radiance));
        if (id.radiance_textured) {
            const pt_texture_desc &t = id.radiance_tex;
            DevTexture dt = to_dev(t);
            if (t.type == PT_TEX_BITMAP) {
                cudaTextureObject_t obj = 0;
                int st = bitmap_texture(s, t.pixels, t.width, t.height, t.address_mode, t.filter, &obj);
                if (st != PT_OK) return st;
                dt.obj = static_cast<unsigned long long>(obj);
            }
            src.tex = (int32_t)emit_tex.size();
            emit_tex.push_back(dt);
            src.weight = emitter_weight(t);
        } else {
            src.weight = std::max(std::max(id.radiance[0], id.radiance[1]), id.radiance[2]);
        }
        if (id.shape_type == PT_SHAPE_MESH) {
            const pt_mesh_desc &m = d->meshes[id.shape_index];
            if (m.texcoords) src.uvs.assign(m.texcoords, m.texcoords + 2ull * m.num_vertices);
            double inv[16];
            inverse4f(id.to_world, inv);
            normal_matrix(inv, src.nm);
            for (auto &r : s->mesh_instances)
                if (r.instance == ii) src.vertex_offset = r.vertex_offset;
            src.indices.assign(m.indices, m.indices + 3ull * m.num_triangles);
            if (m.normals) src.normals.assign(m.normals, m.normals + 3ull * m.num_vertices);
            n_area += m.num_triangles;
            s->has_emissive_mesh = true;
        } else {
            src.sphere = true;
            src.center[0] = in.sphere.x;
            src.center[1] = in.sphere.y;
            src.center[2] = in.sphere.z;
            src.radius = in.sphere.w;
            n_area += 1;
        }
        s->emitter_sources.push_back(std::move(src));
    }
    s->has_env = d->env.type != PT_ENV_NONE;
    s->env_type = d->env.type;
    memcpy(s->env_radiance, d->env.radiance, sizeof(s->env_radiance));
    if (d->env.type == PT_ENV_MAP) {
        int st = build_env_map(s, d->env);
        if (st != PT_OK) return st;
    }

    int e;
    if ((e = upload(s->prims_world, prims)) != PT_OK) return e;
    if ((e = upload(s->tri_vidx, tri_vidx)) != PT_OK) return e;
    if ((e = upload(s->vpos, vpos)) != PT_OK) return e;
    if ((e = upload(s->vnrm, vnrm)) != PT_OK) return e;
    if ((e = upload(s->vuv, vuv)) != PT_OK) return e;
    if ((e = upload(s->prim_inst, prim_inst)) != PT_OK) return e;
    if ((e = upload(s->curve_seg, curve_seg)) != PT_OK) return e;
    if ((e = upload(s->curve_cp, curve_cp)) != PT_OK) return e;
    if ((e = upload(s->inst, insts)) != PT_OK) return e;
    if ((e = upload(s->mats, mats)) != PT_OK) return e;
    if ((e = upload(s->emitter_tex, emit_tex)) != PT_OK) return e;
    s->h_prims_world = std::move(prims);

    ptd::DevScene &dv = s->dev;
    dv.tri_vidx = s->tri_vidx.as<uint32_t>();
    dv.vpos = s->vpos.as<float4>();
    dv.vnrm = s->vnrm.as<float4>();
    dv.vuv = s->vuv.as<float2>();
    dv.prim_inst = s->prim_inst.as<uint32_t>();
    dv.curve_seg = s->curve_seg.as<uint32_t>();
    dv.curve_cp = s->curve_cp.as<float4>();
    dv.curve_prim0 = ntri + nsph;
    dv.inst = s->inst.as<DevInstance>();
    dv.mats = s->mats.as<DevMaterial>();
    dv.emit_tex = s->emitter_tex.as<DevTexture>();
    dv.num_tris = ntri;
    if ((e = pt_rebuild_emitters(s, vpos.data())) != PT_OK) return e;
    dv.width_px = d->width;
    dv.height_px = d->height;
    dv.max_depth = d->max_depth;
    set_camera(s, d->camera);
    return PT_OK;
}

}  // namespace

// Emitter table (world/emitter.cpp:169-243) and selection probabilities
// (EmitterHelper::ComputeProbability, world/emitter.cpp:321-337), from the
// current world vertices: host_vpos when the caller holds them, else a copy
// of each emissive mesh instance's vertex range from the device.
int pt_rebuild_emitters(pt_scene *s, const float4 *host_vpos) {
    std::vector<DevEmitter> ems;
    std::vector<float> weights;  // Emitter::weight = GetWeight(radiance) * area
    std::vector<float4> fetched;
    for (const EmitterSource &src : s->emitter_sources) {
        H3 rad = h3(src.radiance[0], src.radiance[1], src.radiance[2]);
        const float w = src.weight;  // GetWeight (emitter.cpp:77-101)
        // textured radiance: 1 + texture index in rad.w (rad.xyz unused)
        float texw = 0.f;
        if (src.tex >= 0) {
            const uint32_t bits = (uint32_t)src.tex + 1u;
            memcpy(&texw, &bits, 4);
            rad = h3(0.f, 0.f, 0.f);
        }
        if (!src.sphere) {
            const float4 *vp;
            if (host_vpos) {
                vp = host_vpos + src.vertex_offset;
            } else {
                uint32_t nv = 0;
                for (uint32_t i : src.indices) nv = std::max(nv, i + 1);
                fetched.resize(std::max<uint32_t>(nv, 1));
                PT_CUDA_TRY(cudaMemcpy(fetched.data(), s->vpos.as<float4>() + src.vertex_offset, 16ull * nv,
                                       cudaMemcpyDeviceToHost));
                vp = fetched.data();
            }
            for (size_t t = 0; 3 * t < src.indices.size(); t++) {
                DevEmitter e{};
                H3 P[3], N[3];
                for (int k = 0; k < 3; k++) {
                    float4 p = vp[src.indices[3 * t + k]];
                    P[k] = h3(p.x, p.y, p.z);
                }
                for (int k = 0; k < 3; k++) {
                    uint32_t vi = src.indices[3 * t + k];
                    H3 nw = !src.normals.empty()
                                ? xform_vec(src.nm, h3(src.normals[3 * vi], src.normals[3 * vi + 1], src.normals[3 * vi + 2]))
                                : hcross(sub(P[1], P[0]), sub(P[2], P[0]));
                    float len = sqrtf(nw.x * nw.x + nw.y * nw.y + nw.z * nw.z);  // TransformNormal normalises
                    N[k] = h3(nw.x / len, nw.y / len, nw.z / len);
                }
                float area = hlen(hcross(sub(P[1], P[0]), sub(P[2], P[0]))) * 0.5f;
                uint32_t type = ptd::kEmitTri;
                float tf;
                memcpy(&tf, &type, 4);
                e.a = make_float4(tf, 0.f, area, 0.f);  // type, select probability, area, radius
                weights.push_back(w * area);
                e.rad = make_float4(rad.x, rad.y, rad.z, texw);
                // vertex texture coordinates, as the reference reads them
                // (mesh.texcoords, without flip_tex_coords; world/emitter.cpp:169-217)
                float U[3] = {0.f, 0.f, 0.f}, V[3] = {0.f, 0.f, 0.f};
                if (!src.uvs.empty())
                    for (int k = 0; k < 3; k++) {
                        const uint32_t vi = src.indices[3 * t + k];
                        U[k] = src.uvs[2 * vi];
                        V[k] = src.uvs[2 * vi + 1];
                    }
                e.p0 = make_float4(P[0].x, P[0].y, P[0].z, U[0]);
                e.p1 = make_float4(P[1].x, P[1].y, P[1].z, U[1]);
                e.p2 = make_float4(P[2].x, P[2].y, P[2].z, U[2]);
                e.n0 = make_float4(N[0].x, N[0].y, N[0].z, V[0]);
                e.n1 = make_float4(N[1].x, N[1].y, N[1].z, V[1]);
                e.n2 = make_float4(N[2].x, N[2].y, N[2].z, V[2]);
                ems.push_back(e);
            }
        } else {
            DevEmitter e{};
            float r = src.radius;
            float area = 4 * 3.14159265358979323846f * r * r;
            uint32_t type = ptd::kEmitSphere;
            float tf;
            memcpy(&tf, &type, 4);
            e.a = make_float4(tf, 0.f, area, r);
            weights.push_back(w * area);
            e.rad = make_float4(rad.x, rad.y, rad.z, texw);
            e.p0 = make_float4(src.center[0], src.center[1], src.center[2], 0.f);
            ems.push_back(e);
        }
    }
    float wsum = 0.f;
    for (float w : weights) wsum += w;
    size_t n_emit = (s->has_env ? 1 : 0) + ems.size();
    std::vector<float> cdf;
    float acc = 0.f;
    for (size_t i = 0; i < ems.size(); i++) {
        float p = weights[i] / wsum * (float)ems.size();
        p = p / (float)n_emit;
        ems[i].a.y = p;
        cdf.push_back(acc + p);  // the running sums SelectOneEmiiter compares against
        acc += p;
    }
    DevEmitter env{};
    if (s->has_env) {
        uint32_t type = s->env_type == PT_ENV_MAP ? ptd::kEmitEnvMap : ptd::kEmitConstEnv;
        float tf;
        memcpy(&tf, &type, 4);
        env.a = make_float4(tf, 1.f / (float)n_emit, 0.f, 0.f);
        env.rad = make_float4(s->env_radiance[0], s->env_radiance[1], s->env_radiance[2], 0.f);
    }
    int e;
    if ((e = upload(s->emitters, ems)) != PT_OK) return e;
    if ((e = upload(s->emitter_cdf, cdf)) != PT_OK) return e;
    ptd::DevScene &dv = s->dev;
    dv.emitters = s->emitters.as<DevEmitter>();
    dv.emitter_cdf = s->emitter_cdf.as<float>();
    dv.num_emitters = (uint32_t)ems.size();
    dv.has_env = s->has_env ? 1 : 0;
    dv.env = env;
    return PT_OK;
}

// Entry points start by clearing the runtime's last-error state, so that an
// error left behind by some other call in the process is not reported here.
static inline void clear_stale_cuda_error() { (void)cudaGetLastError(); }

void pt_set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int DevBuf::ensure(size_t n) {
    if (n <= bytes && ptr) return PT_OK;
    release();
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        pt_set_error("cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
    bytes = n;
    return PT_OK;
}
void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

pt_scene::~pt_scene() {
    DevBuf *all[] = {&prims_world, &prims_bvh, &nodes, &cnodes, &tri_vidx, &vpos, &vnrm, &vuv, &prim_inst, &inst, &mats, &curve_seg, &curve_cp,
                     &emitters, &emitter_cdf, &emitter_tex, &mesh_obj_pos, &bvh_scratch, &bvh_order, &sah_scratch, &xform_table, &all_obj_pos, &ws.ray_o, &ws.ray_d, &ws.hit, &ws.thr,
                     &ws.rad, &ws.rng, &ws.meta, &ws.q0, &ws.q1, &ws.sh_o, &ws.sh_d, &ws.sh_c, &ws.mat_key,
                     &ws.counters, &ws.sort_tmp, &ws.bin_blocks};
    for (DevBuf *b : all) b->release();
    env_row_cdf.release();
    env_col_cdf.release();
    env_row_weight.release();
    for (auto &b : bitmaps) {
        if (b.obj) cudaDestroyTextureObject(b.obj);
        if (b.array) cudaFreeArray(b.array);
    }
    if (ws.exec) cudaGraphExecDestroy(ws.exec);
    if (ws.ev_in) cudaEventDestroy(ws.ev_in);
    if (ws.ev_out) cudaEventDestroy(ws.ev_out);
    if (ws.stream) cudaStreamDestroy(ws.stream);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

// C++ exceptions (a host allocation that fails while a large scene's tables
// are built, for instance) must not cross the C ABI: they become statuses.
template <class F>
static int no_throw(const char *where, F &&f) noexcept {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        pt_set_error("%s: out of host memory", where);
        return PT_ERR_OOM;
    } catch (const std::exception &e) {
        pt_set_error("%s: %s", where, e.what());
        return PT_ERR_INVALID;
    } catch (...) {
        pt_set_error("%s: unexpected C++ exception", where);
        return PT_ERR_INVALID;
    }
}

extern "C" {

int pt_api_version(void) { return PT_API_VERSION; }

int pt_last_error(char *buf, size_t n) {
    if (!buf || n == 0) return PT_ERR_INVALID;
    size_t k = std::min(n - 1, g_last_error.size());
    memcpy(buf, g_last_error.data(), k);
    buf[k] = 0;
    return PT_OK;
}

int pt_context_create(const pt_device_opts *opts, pt_context **out) {
    clear_stale_cuda_error();
    if (!out) { pt_set_error("out is NULL"); return PT_ERR_INVALID; }
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        pt_set_error("no CUDA device available (%s)", cudaGetErrorString(e));
        return PT_ERR_UNSUPPORTED;
    }
    int dev = opts ? opts->device : 0;
    if (dev < 0 || dev >= count) { pt_set_error("device %d out of range", dev); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(dev));
    auto c = std::make_unique<pt_context>();
    c->device = dev;
    PT_CUDA_TRY(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev));
    PT_CUDA_TRY(cudaDeviceGetAttribute(&c->max_smem_per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    *out = c.release();
    return PT_OK;
}

int pt_context_destroy(pt_context *ctx) {
    delete ctx;
    return PT_OK;
}

int pt_scene_upload(pt_context *ctx, const pt_scene_desc *desc, pt_scene **out) {
    clear_stale_cuda_error();
    if (!ctx || !out) { pt_set_error("context or out is NULL"); return PT_ERR_INVALID; }
    *out = nullptr;
    PT_CUDA_TRY(cudaSetDevice(ctx->device));
    auto s = std::make_unique<pt_scene>();
    s->ctx = ctx;
    s->device = ctx->device;
    s->num_sms = ctx->num_sms;
    s->max_smem_per_block = ctx->max_smem_per_block;
    int st = no_throw("pt_scene_upload", [&] { return build_scene(s.get(), desc); });
    if (st != PT_OK) return st;
    PT_CUDA_TRY(cudaEventCreate(&s->ev0));
    PT_CUDA_TRY(cudaEventCreate(&s->ev1));
    *out = s.release();
    return PT_OK;
}

int pt_scene_destroy(pt_scene *scene) {
    if (scene) {
        cudaSetDevice(scene->device);
        delete scene;
        clear_stale_cuda_error();
    }
    return PT_OK;
}

int pt_scene_set_camera(pt_scene *scene, const pt_camera_desc *camera) {
    if (!scene || !camera) { pt_set_error("scene or camera is NULL"); return PT_ERR_INVALID; }
    set_camera(scene, *camera);
    return PT_OK;
}

int pt_scene_num_prims(const pt_scene *scene, uint32_t *nt, uint32_t *ns) {
    if (!scene) { pt_set_error("scene is NULL"); return PT_ERR_INVALID; }
    if (nt) *nt = scene->num_tris;
    if (ns) *ns = scene->num_spheres;
    return PT_OK;
}

int pt_scene_num_curves(const pt_scene *scene, uint32_t *num_segments, uint32_t *num_pieces) {
    if (!scene) { pt_set_error("scene is NULL"); return PT_ERR_INVALID; }
    if (num_segments) *num_segments = scene->num_curve_segments;
    if (num_pieces) *num_pieces = scene->num_curve_pieces;
    return PT_OK;
}

int pt_scene_update_vertices(pt_scene *scene, uint32_t mesh, const float *positions, uint32_t num_vertices) {
    clear_stale_cuda_error();
    if (!scene || !positions) { pt_set_error("scene or positions is NULL"); return PT_ERR_INVALID; }
    if (mesh >= scene->mesh_num_vertices.size() || num_vertices != scene->mesh_num_vertices[mesh]) {
        pt_set_error("mesh %u: expected %u vertices", mesh, mesh < scene->mesh_num_vertices.size() ? scene->mesh_num_vertices[mesh] : 0);
        return PT_ERR_INVALID;
    }
    for (uint64_t v = 0; v < 3ull * num_vertices; v++)
        if (!std::isfinite(positions[v])) { pt_set_error("non-finite vertex coordinate"); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    int st = scene->mesh_obj_pos.ensure(std::max<size_t>(12ull * num_vertices, 16));
    if (st != PT_OK) return st;
    PT_CUDA_TRY(cudaMemcpy(scene->mesh_obj_pos.ptr, positions, 12ull * num_vertices, cudaMemcpyHostToDevice));
    st = pt_update_world_vertices(scene, mesh, scene->mesh_obj_pos.as<float>(), num_vertices, 0);
    if (st != PT_OK || !scene->has_emissive_mesh) return st;
    PT_CUDA_TRY(cudaDeviceSynchronize());
    return no_throw("pt_scene_update_vertices", [&] { return pt_rebuild_emitters(scene, nullptr); });
}

int pt_scene_update_all_vertices(pt_scene *scene, const float *positions, int on_device, void *stream) {
    clear_stale_cuda_error();
    if (!scene || !positions) { pt_set_error("scene or positions is NULL"); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    const float *src = positions;
    if (!on_device) {
        size_t n = 3 * scene->total_mesh_vertices;
        for (size_t v = 0; v < n; v++)
            if (!std::isfinite(positions[v])) { pt_set_error("non-finite vertex coordinate"); return PT_ERR_INVALID; }
        int st = scene->all_obj_pos.ensure(std::max<size_t>(4 * n, 16));
        if (st != PT_OK) return st;
        PT_CUDA_TRY(cudaMemcpyAsync(scene->all_obj_pos.ptr, positions, 4 * n, cudaMemcpyHostToDevice,
                                    static_cast<cudaStream_t>(stream)));
        src = scene->all_obj_pos.as<float>();
    }
    int st = pt_update_all_world_vertices(scene, src, static_cast<cudaStream_t>(stream));
    if (st != PT_OK || !scene->has_emissive_mesh) return st;
    // Light triangles moved: the emitter table is rebuilt from the new world
    // vertices once the update kernels on `stream` have finished.
    PT_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return no_throw("pt_scene_update_all_vertices", [&] { return pt_rebuild_emitters(scene, nullptr); });
}

int pt_bvh_build(pt_scene *scene, const pt_bvh_opts *opts, void *stream) {
    clear_stale_cuda_error();
    if (!scene) { pt_set_error("scene is NULL"); return PT_ERR_INVALID; }
    pt_bvh_opts o{4, 4, 0, 0};
    if (opts) o = *opts;
    if (o.width != 2 && o.width != 4 && o.width != 8) { pt_set_error("BVH width must be 2, 4 or 8"); return PT_ERR_INVALID; }
    if (o.max_leaf_size < 1 || o.max_leaf_size > 15) { pt_set_error("max_leaf_size must be in 1..15"); return PT_ERR_INVALID; }
    if (o.flags & ~(uint32_t)PT_BVH_FAST_BUILD) { pt_set_error("unknown BVH flags 0x%x", o.flags); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    return no_throw("pt_bvh_build", [&] { return pt_bvh_build_impl(scene, &o, static_cast<cudaStream_t>(stream)); });
}

int pt_bvh_refit(pt_scene *scene, void *stream) {
    clear_stale_cuda_error();
    if (!scene) { pt_set_error("scene is NULL"); return PT_ERR_INVALID; }
    if (!scene->bvh_built) { pt_set_error("pt_bvh_refit before pt_bvh_build"); return PT_ERR_STATE; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    return pt_bvh_refit_impl(scene, static_cast<cudaStream_t>(stream));
}

int pt_bvh_get_stats(const pt_scene *scene, pt_bvh_stats *out) {
    if (!scene || !out) { pt_set_error("scene or out is NULL"); return PT_ERR_INVALID; }
    *out = scene->bvh_stats;
    return PT_OK;
}

int pt_render(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, void *stream) {
    clear_stale_cuda_error();
    if (!scene || !params || !fb || !fb->accum) { pt_set_error("scene, params, buffers or accum is NULL"); return PT_ERR_INVALID; }
    if (!scene->bvh_built) { pt_set_error("pt_render before pt_bvh_build"); return PT_ERR_STATE; }
    if (params->rng != PT_RNG_REF_LCG && params->rng != PT_RNG_PCG32) { pt_set_error("unknown rng mode"); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    return no_throw("pt_render", [&] { return pt_render_impl(scene, params, fb, static_cast<cudaStream_t>(stream)); });
}

int pt_render_batch(pt_context *ctx, pt_scene *const *scenes, const pt_render_params *params,
                    const pt_frame_buffers *fbs, uint32_t n, void *stream) {
    clear_stale_cuda_error();
    if (!ctx || !params || (n && (!scenes || !fbs))) { pt_set_error("context, scenes, params or buffers is NULL"); return PT_ERR_INVALID; }
    if (params->rng != PT_RNG_REF_LCG && params->rng != PT_RNG_PCG32) { pt_set_error("unknown rng mode"); return PT_ERR_INVALID; }
    for (uint32_t k = 0; k < n; k++) {
        const pt_scene *s = scenes[k];
        if (!s || !fbs[k].accum) { pt_set_error("scene %u or its accum buffer is NULL", k); return PT_ERR_INVALID; }
        if (s->device != ctx->device) { pt_set_error("scene %u lives on another device", k); return PT_ERR_INVALID; }
        if (!s->bvh_built) { pt_set_error("pt_render_batch: scene %u has no BVH", k); return PT_ERR_STATE; }
        if (s->dev.width != scenes[0]->dev.width) {
            pt_set_error("pt_render_batch: scene %u has BVH width %u, scene 0 has %u", k, s->dev.width, scenes[0]->dev.width);
            return PT_ERR_INVALID;
        }
    }
    PT_CUDA_TRY(cudaSetDevice(ctx->device));
    return no_throw("pt_render_batch",
                    [&] { return pt_render_batch_impl(ctx, scenes, params, fbs, n, static_cast<cudaStream_t>(stream)); });
}

int pt_render_batch_get_stats(const pt_context *ctx, pt_render_stats *out) {
    if (!ctx || !out) { pt_set_error("context or out is NULL"); return PT_ERR_INVALID; }
    return pt_render_batch_stats(ctx, out);
}

int pt_autotune(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, pt_tune_result *out,
                void *stream) {
    clear_stale_cuda_error();
    if (!scene || !params || !fb || !fb->accum) { pt_set_error("scene, params, buffers or accum is NULL"); return PT_ERR_INVALID; }
    if (!scene->bvh_built) { pt_set_error("pt_autotune before pt_bvh_build"); return PT_ERR_STATE; }
    if (params->rng != PT_RNG_REF_LCG && params->rng != PT_RNG_PCG32) { pt_set_error("unknown rng mode"); return PT_ERR_INVALID; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    return no_throw("pt_autotune", [&] { return pt_autotune_impl(scene, params, fb, out, static_cast<cudaStream_t>(stream)); });
}

int pt_render_get_stats(const pt_scene *scene, pt_render_stats *out) {
    if (!scene || !out) { pt_set_error("scene or out is NULL"); return PT_ERR_INVALID; }
    *out = scene->render_stats;
    return PT_OK;
}

int pt_trace_rays(pt_scene *scene, const float *rays, float *hits, uint32_t n, int anyhit, void *stream) {
    clear_stale_cuda_error();
    if (!scene || (n && (!rays || !hits))) { pt_set_error("scene, rays or hits is NULL"); return PT_ERR_INVALID; }
    if (!scene->bvh_built) { pt_set_error("pt_trace_rays before pt_bvh_build"); return PT_ERR_STATE; }
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    return no_throw("pt_trace_rays",
                    [&] { return pt_trace_rays_impl(scene, rays, hits, n, anyhit, static_cast<cudaStream_t>(stream)); });
}

int pt_bsdf_eval_batch(const float *bsdf, const float *wo, const float *wi, float *f, float *pdf, uint32_t n, void *stream) {
    clear_stale_cuda_error();
    if (n && (!bsdf || !wo || !wi || !f || !pdf)) { pt_set_error("NULL buffer"); return PT_ERR_INVALID; }
    return pt_bsdf_eval_impl(bsdf, wo, wi, f, pdf, n, static_cast<cudaStream_t>(stream));
}

int pt_bsdf_sample_batch(const float *bsdf, const float *wo, uint32_t *rng, float *wi, float *f, float *pdf,
                         uint32_t *type, uint32_t n, void *stream) {
    clear_stale_cuda_error();
    if (n && (!bsdf || !wo || !rng || !wi || !f || !pdf || !type)) { pt_set_error("NULL buffer"); return PT_ERR_INVALID; }
    return pt_bsdf_sample_impl(bsdf, wo, rng, wi, f, pdf, type, n, static_cast<cudaStream_t>(stream));
}

int pt_trig_eval(uint32_t fn, const float *x, const float *y, float *out, float *out_platform, uint32_t n, void *stream) {
    clear_stale_cuda_error();
    if (fn > 3) { pt_set_error("unknown function %u", fn); return PT_ERR_INVALID; }
    if (n && (!x || !out || (fn == 2 && !y))) { pt_set_error("NULL buffer"); return PT_ERR_INVALID; }
    return pt_trig_eval_impl(fn, x, y, out, out_platform, n, static_cast<cudaStream_t>(stream));
}

// util::Camera::GetSampleToCameraMatrix (framework/util/camera.cpp:7-20):
// sample_to_camera = transpose(inverse(P * T(1,1,0) * S(0.5,0.5,1))) where P is
// DirectXMath's row-vector XMMatrixPerspectiveFovRH; computed in double here.
int pt_camera_make(float fov_y_deg, float aspect, float near_clip, float far_clip, const float to_world[16],
                   pt_camera_desc *out) {
    if (!out || !to_world || !(aspect > 0.f) || !(fov_y_deg > 0.f) || near_clip == far_clip) {
        pt_set_error("invalid camera parameters");
        return PT_ERR_INVALID;
    }
    double fov = (double)(fov_y_deg / 180.f * 3.14159265358979323846f);
    double h = cos(0.5 * fov) / sin(0.5 * fov);
    double w = h / aspect;
    double range = (double)far_clip / ((double)near_clip - (double)far_clip);
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
    inverse4(A, Ainv);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out->sample_to_camera[4 * r + c] = (float)Ainv[4 * c + r];
    memcpy(out->camera_to_world, to_world, 16 * sizeof(float));
    return PT_OK;
}

}  // extern "C"
