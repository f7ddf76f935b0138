// scene.cpp -- mitsuba3-style scene loader (see scene.h).
//
// Follows the reference loader's semantics: resource/scene.cpp:27-226
// (integrator, sensor with fov_axis conversion and the Mitsuba -> Pupil axis
// flip), resource/material.cpp:18-190 (BSDF defaults), resource/shape.cpp
// (rectangle / cube / sphere / obj shapes) and resource/xml/util_loader.cpp:
// 128-210 (transforms: matrix of 16 or 9 values, lookat, or scale then rotate
// then translate, each left-multiplied).
#include "scene.h"
#include "image.h"

#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>

#include "xml.h"

namespace Pupil::resource {

namespace {

constexpr double kPi = 3.14159265358979323846;

void identity(float m[16]) {
    for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.f : 0.f;
}
void mul(const float a[16], const float b[16], float out[16]) {  // out = a * b (row-major)
    float r[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double acc = 0.0;
            for (int k = 0; k < 4; k++) acc += (double)a[4 * i + k] * b[4 * k + j];
            r[4 * i + j] = (float)acc;
        }
    memcpy(out, r, sizeof(r));
}

std::vector<float> numbers(const std::string &s) {
    std::vector<float> v;
    std::string t = s;
    for (char &c : t)
        if (c == ',') c = ' ';
    std::istringstream is(t);
    float x;
    while (is >> x) v.push_back(x);
    return v;
}

// Named dielectric indices of refraction (Hecht, Optics; values at ~589 nm).
bool dielectric_ior(const std::string &name, float &out) {
    static const std::pair<const char *, float> table[] = {
        {"vacuum", 1.0f}, {"helium", 1.000036f}, {"hydrogen", 1.000132f}, {"air", 1.000277f},
        {"carbon dioxide", 1.00045f}, {"water", 1.3330f}, {"acetone", 1.36f}, {"ethanol", 1.361f},
        {"carbon tetrachloride", 1.461f}, {"glycerol", 1.4729f}, {"benzene", 1.501f}, {"silicone oil", 1.52045f},
        {"bromine", 1.661f}, {"water ice", 1.31f}, {"fused quartz", 1.458f}, {"pyrex", 1.470f},
        {"acrylic glass", 1.49f}, {"polypropylene", 1.49f}, {"bk7", 1.5046f}, {"sodium chloride", 1.544f},
        {"amber", 1.55f}, {"pet", 1.5750f}, {"diamond", 2.419f}};
    for (auto &e : table)
        if (name == e.first) {
            out = e.second;
            return true;
        }
    return false;
}

// RGB-averaged complex IORs of a few metals (published measured data).
bool conductor_ior(const std::string &name, float eta[3], float k[3]) {
    struct E {
        const char *n;
        float eta[3], k[3];
    };
    static const E table[] = {
        {"Au", {0.143f, 0.374f, 1.442f}, {3.983f, 2.385f, 1.603f}},
        {"Ag", {0.155f, 0.117f, 0.138f}, {4.828f, 3.122f, 2.147f}},
        {"Cu", {0.200f, 0.924f, 1.102f}, {3.912f, 2.452f, 2.142f}},
        {"Al", {1.657f, 0.880f, 0.521f}, {9.224f, 6.270f, 4.837f}},
    };
    for (auto &e : table)
        if (name == e.n) {
            memcpy(eta, e.eta, sizeof(e.eta));
            memcpy(k, e.k, sizeof(e.k));
            return true;
        }
    return false;
}

pt_texture_desc rgb(float r, float g, float b) {
    pt_texture_desc t{};
    t.type = PT_TEX_RGB;
    t.color0[0] = r;
    t.color0[1] = g;
    t.color0[2] = b;
    const float uv[8] = {1, 0, 0, 0, 0, 1, 0, 0};
    memcpy(t.uv_transform, uv, sizeof(uv));
    return t;
}

}  // namespace

struct Loader {
    Scene &s;
    std::string &err;

    bool fail(const xml::Node *n, const std::string &m) {
        if (err.empty()) err = (n ? "line " + std::to_string(n->line) + ": " : std::string()) + m;
        return false;
    }
    std::string value(const xml::Node *n, const char *key = "value") {
        std::string v = n->attr_or(key, "");
        if (!v.empty() && v[0] == '$') {
            auto it = s.m_defaults.find(v.substr(1));
            if (it != s.m_defaults.end()) return it->second;
        }
        return v;
    }
    const xml::Node *prop(const xml::Node *n, const char *tag, const char *name) {
        for (auto &c : n->children)
            if (c->name == tag && c->attr_or("name", "") == name) return c.get();
        return nullptr;
    }
    bool get_float(const xml::Node *n, const char *name, float &out) {
        const xml::Node *p = prop(n, "float", name);
        if (!p) p = prop(n, "integer", name);
        if (!p) return false;
        auto v = numbers(value(p));
        if (v.size() != 1) return fail(p, std::string("float ") + name + " needs one value");
        out = v[0];
        return true;
    }
    bool get_int(const xml::Node *n, const char *name, uint32_t &out) {
        const xml::Node *p = prop(n, "integer", name);
        if (!p) return false;
        auto v = numbers(value(p));
        if (v.size() != 1 || v[0] < 0) return fail(p, std::string("integer ") + name + " needs one value >= 0");
        out = (uint32_t)v[0];
        return true;
    }
    std::string get_string(const xml::Node *n, const char *name, const std::string &fallback) {
        const xml::Node *p = prop(n, "string", name);
        return p ? value(p) : fallback;
    }
    bool get_bool(const xml::Node *n, const char *name, bool fallback) {
        const xml::Node *p = prop(n, "boolean", name);
        return p ? value(p) == "true" : fallback;
    }
    bool get_point(const xml::Node *n, const char *name, float out[3]) {
        const xml::Node *p = prop(n, "point", name);
        if (!p) return false;
        if (p->attr("value")) {
            auto v = numbers(value(p));
            if (v.size() != 3) return fail(p, "point needs 3 values");
            for (int i = 0; i < 3; i++) out[i] = v[i];
        } else {
            out[0] = std::stof(p->attr_or("x", "0"));
            out[1] = std::stof(p->attr_or("y", "0"));
            out[2] = std::stof(p->attr_or("z", "0"));
        }
        return true;
    }
    // the scale of a texture's to_uv transform
    void uv_scale(const xml::Node *c, pt_texture_desc &out) {
        for (auto &t : c->children)
            if (t->name == "transform" && t->attr_or("name", "") == "to_uv") {
                for (auto &sc : t->children)
                    if (sc->name == "scale") {
                        float x = 1.f, y = 1.f;
                        if (sc->attr("value")) {
                            auto v = numbers(value(sc.get()));
                            x = v.empty() ? 1.f : v[0];
                            y = v.size() > 1 ? v[1] : x;
                        } else {
                            x = std::stof(sc->attr_or("x", "1"));
                            y = std::stof(sc->attr_or("y", "1"));
                        }
                        out.uv_transform[0] = x;
                        out.uv_transform[5] = y;
                    }
            }
    }
    std::string m_root_path(const std::string &file) {
        if (file.empty() || file[0] == '/' || s.m_root.empty()) return file;
        return s.m_root + "/" + file;
    }
    // rgb / float / checkerboard texture (LoadTextureOrRGB)
    bool get_texture(const xml::Node *n, const char *name, pt_texture_desc &out, pt_texture_desc fallback) {
        out = fallback;
        for (auto &c : n->children) {
            if (c->attr_or("name", "") != name) continue;
            if (c->name == "rgb" || c->name == "spectrum") {
                auto v = numbers(value(c.get()));
                if (v.size() == 1) v = {v[0], v[0], v[0]};
                if (v.size() != 3) return fail(c.get(), std::string("rgb ") + name + " needs 1 or 3 values");
                out = rgb(v[0], v[1], v[2]);
                return true;
            }
            if (c->name == "float") {
                auto v = numbers(value(c.get()));
                if (v.size() != 1) return fail(c.get(), "float needs one value");
                out = rgb(v[0], v[0], v[0]);
                return true;
            }
            if (c->name == "texture" && c->attr_or("type", "") == "bitmap") {  // scene.cpp:143-166
                const xml::Node *fn = prop(c.get(), "string", "filename");
                if (!fn) return fail(c.get(), "bitmap texture without a filename");
                std::vector<float> px;
                uint32_t w = 0, h = 0;
                std::string e;
                if (!util::LoadImageRGBA(m_root_path(value(fn)), px, w, h, e)) return fail(c.get(), e);
                s.images.push_back(std::move(px));
                out = rgb(0.f, 0.f, 0.f);
                out.type = PT_TEX_BITMAP;
                out.pixels = s.images.back().data();
                out.width = w;
                out.height = h;
                const xml::Node *ft = prop(c.get(), "string", "filter_type");
                out.filter = (ft && value(ft) == "bilinear") ? PT_TEX_FILTER_LINEAR : PT_TEX_FILTER_POINT;
                const xml::Node *wm = prop(c.get(), "string", "wrap_mode");
                const std::string mode = wm ? value(wm) : "repeat";
                out.address_mode = mode == "mirror" ? PT_TEX_ADDRESS_MIRROR
                                   : mode == "clamp" ? PT_TEX_ADDRESS_CLAMP
                                                     : PT_TEX_ADDRESS_WRAP;
                uv_scale(c.get(), out);
                return true;
            }
            if (c->name == "texture") {
                std::string type = c->attr_or("type", "");
                if (type != "checkerboard") return fail(c.get(), "texture type '" + type + "' is not supported");
                out = rgb(0.4f, 0.4f, 0.4f);
                out.type = PT_TEX_CHECKERBOARD;
                pt_texture_desc c0, c1;
                if (!get_texture(c.get(), "color0", c0, rgb(0.4f, 0.4f, 0.4f))) return false;
                if (!get_texture(c.get(), "color1", c1, rgb(0.2f, 0.2f, 0.2f))) return false;
                memcpy(out.color0, c0.color0, sizeof(out.color0));
                memcpy(out.color1, c1.color0, sizeof(out.color1));
                uv_scale(c.get(), out);
                return true;
            }
        }
        return true;
    }
    bool get_ior(const xml::Node *n, const char *name, float &out, float fallback) {
        out = fallback;
        const xml::Node *p = prop(n, "float", name);
        if (p) {
            auto v = numbers(value(p));
            if (v.size() != 1) return fail(p, "ior needs one value");
            out = v[0];
            return true;
        }
        p = prop(n, "string", name);
        if (p && !dielectric_ior(value(p), out)) return fail(p, "unknown IOR name '" + value(p) + "'");
        return true;
    }

    // util_loader.cpp:128-191
    bool transform(const xml::Node *t, float m[16]) {
        identity(m);
        for (auto &c : t->children)
            if (c->name == "matrix") {
                auto v = numbers(value(c.get()));
                if (v.size() == 16) {
                    for (int i = 0; i < 16; i++) m[i] = v[i];
                } else if (v.size() == 9) {
                    for (int r = 0; r < 3; r++)
                        for (int col = 0; col < 3; col++) m[4 * r + col] = v[3 * r + col];
                } else {
                    return fail(c.get(), "matrix needs 9 or 16 values");
                }
                return true;
            }
        for (auto &c : t->children)
            if (c->name == "lookat") {
                auto o = numbers(c->attr_or("origin", "1, 0, 0"));
                auto tg = numbers(c->attr_or("target", "0, 0, 0"));
                auto up = numbers(c->attr_or("up", "0, 1, 0"));
                if (o.size() != 3 || tg.size() != 3 || up.size() != 3) return fail(c.get(), "lookat needs 3-vectors");
                // inverse of a right-handed look-at view matrix (camera looks down -Z) ...
                double z[3] = {o[0] - tg[0], o[1] - tg[1], o[2] - tg[2]};
                double zl = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
                for (double &x : z) x /= zl;
                double x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
                double xl = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                for (double &v : x) v /= xl;
                double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
                for (int r = 0; r < 3; r++) {
                    // ... with the Mitsuba -> Pupil flip of the X and Z columns (util_loader.cpp:159-165)
                    m[4 * r + 0] = (float)-x[r];
                    m[4 * r + 1] = (float)y[r];
                    m[4 * r + 2] = (float)-z[r];
                    m[4 * r + 3] = o[r];
                }
                return true;
            }
        float S[16], R[16], T[16];
        identity(S);
        identity(R);
        identity(T);
        for (auto &c : t->children) {
            if (c->name == "scale") {
                float x = 1, y = 1, z = 1;
                if (c->attr("value")) {
                    auto v = numbers(value(c.get()));
                    if (v.size() == 1) x = y = z = v[0];
                    else if (v.size() == 3) x = v[0], y = v[1], z = v[2];
                    else return fail(c.get(), "scale needs 1 or 3 values");
                } else {
                    x = std::stof(c->attr_or("x", "1"));
                    y = std::stof(c->attr_or("y", "1"));
                    z = std::stof(c->attr_or("z", "1"));
                }
                S[0] = x, S[5] = y, S[10] = z;
            } else if (c->name == "rotate") {  // quaternion rotation, util/transform.cpp:7-50
                double ax, ay, az;
                if (c->attr("value")) {
                    auto v = numbers(value(c.get()));
                    if (v.size() != 3) return fail(c.get(), "rotate value needs 3 values");
                    ax = v[0], ay = v[1], az = v[2];
                } else {
                    ax = std::stod(c->attr_or("x", "0"));
                    ay = std::stod(c->attr_or("y", "0"));
                    az = std::stod(c->attr_or("z", "0"));
                }
                double len = std::sqrt(ax * ax + ay * ay + az * az);
                if (len == 0) return fail(c.get(), "rotate axis is zero");
                ax /= len, ay /= len, az /= len;
                double th = std::stod(c->attr_or("angle", "0")) / 180.0 * kPi;
                double a = std::cos(0.5 * th), b = std::sin(0.5 * th) * ax, cc = std::sin(0.5 * th) * ay,
                       d = std::sin(0.5 * th) * az;
                const double r[9] = {1 - 2 * cc * cc - 2 * d * d, 2 * b * cc - 2 * a * d,     2 * a * cc + 2 * b * d,
                                     2 * b * cc + 2 * a * d,     1 - 2 * b * b - 2 * d * d, 2 * cc * d - 2 * a * b,
                                     2 * b * d - 2 * a * cc,     2 * a * b + 2 * cc * d,     1 - 2 * b * b - 2 * cc * cc};
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) R[4 * i + j] = (float)r[3 * i + j];
            } else if (c->name == "translate") {
                if (c->attr("value")) {
                    auto v = numbers(value(c.get()));
                    if (v.size() != 3) return fail(c.get(), "translate needs 3 values");
                    T[3] = v[0], T[7] = v[1], T[11] = v[2];
                } else {
                    T[3] = std::stof(c->attr_or("x", "0"));
                    T[7] = std::stof(c->attr_or("y", "0"));
                    T[11] = std::stof(c->attr_or("z", "0"));
                }
            }
        }
        float RS[16];
        mul(R, S, RS);
        mul(T, RS, m);
        return true;
    }

    // resource/material.cpp:18-157
    bool bsdf(const xml::Node *b, pt_material_desc &m) {
        memset(&m, 0, sizeof(m));
        for (auto &t : m.tex) t = rgb(0, 0, 0);
        std::string type = b->attr_or("type", "");
        if (type == "twosided") {
            const xml::Node *inner = nullptr;
            for (auto &c : b->children)
                if (c->name == "bsdf") inner = c.get();
            if (!inner) return fail(b, "twosided needs a nested bsdf");
            if (!bsdf(inner, m)) return false;
            m.twosided = 1;
            return true;
        }
        const pt_texture_desc one = rgb(1, 1, 1), half = rgb(0.5f, 0.5f, 0.5f), alpha = rgb(0.1f, 0.1f, 0.1f);
        if (type == "diffuse") {
            m.type = PT_MAT_DIFFUSE;
            return get_texture(b, "reflectance", m.tex[0], half);
        }
        if (type == "dielectric" || type == "roughdielectric") {
            m.type = type == "dielectric" ? PT_MAT_DIELECTRIC : PT_MAT_ROUGH_DIELECTRIC;
            return get_ior(b, "int_ior", m.int_ior, 1.5046f) && get_ior(b, "ext_ior", m.ext_ior, 1.000277f) &&
                   get_texture(b, "specular_reflectance", m.tex[0], one) &&
                   get_texture(b, "specular_transmittance", m.tex[1], one) &&
                   (m.type == PT_MAT_DIELECTRIC || get_texture(b, "alpha", m.tex[2], alpha));
        }
        if (type == "conductor" || type == "roughconductor") {
            m.type = type == "conductor" ? PT_MAT_CONDUCTOR : PT_MAT_ROUGH_CONDUCTOR;
            float eta[3] = {0, 0, 0}, k[3] = {1, 1, 1};
            std::string metal = get_string(b, "material", "");
            if (!metal.empty() && !conductor_ior(metal, eta, k)) {
                eta[0] = eta[1] = eta[2] = 0.f;  // unknown name: the reference's default (material.cpp:73-78)
                k[0] = k[1] = k[2] = 1.f;
            }
            return get_texture(b, "specular_reflectance", m.tex[0], one) &&
                   get_texture(b, "eta", m.tex[1], rgb(eta[0], eta[1], eta[2])) &&
                   get_texture(b, "k", m.tex[2], rgb(k[0], k[1], k[2])) &&
                   (m.type == PT_MAT_CONDUCTOR || get_texture(b, "alpha", m.tex[3], alpha));
        }
        if (type == "plastic" || type == "roughplastic") {
            m.type = type == "plastic" ? PT_MAT_PLASTIC : PT_MAT_ROUGH_PLASTIC;
            m.nonlinear = get_bool(b, "nonlinear", false) ? 1 : 0;
            return get_ior(b, "int_ior", m.int_ior, 1.49f) && get_ior(b, "ext_ior", m.ext_ior, 1.000277f) &&
                   get_texture(b, "diffuse_reflectance", m.tex[0], half) &&
                   get_texture(b, "specular_reflectance", m.tex[1], one) &&
                   (m.type == PT_MAT_PLASTIC || get_texture(b, "alpha", m.tex[2], alpha));
        }
        return fail(b, "unknown bsdf '" + type + "'");
    }

    uint32_t add_mesh(Mesh &&mesh) {
        s.meshes.push_back(std::move(mesh));
        return (uint32_t)s.meshes.size() - 1;
    }

    // Built-in shapes (resource/shape.cpp:19-69): rectangle XY [-1,1]^2 with +Z
    // normal, cube [-1,1]^3 with 24 vertices and face normals.
    static Mesh rectangle() {
        Mesh m;
        m.positions = {-1, -1, 0, 1, -1, 0, 1, 1, 0, -1, 1, 0};
        m.normals = {0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1};
        m.texcoords = {0, 0, 1, 0, 1, 1, 0, 1};
        m.indices = {0, 1, 2, 0, 2, 3};
        return m;
    }
    static Mesh cube() {
        // Faces in the reference's order (-X, -Z, +X, +Z, +Y, -Y), each with
        // its four corners counter-clockwise seen from outside, uv (0,0) (1,0)
        // (1,1) (0,1) and triangles (0,1,2) (0,2,3): the vertex order, and so
        // the quad diagonals, primitive ids, barycentrics and uvs, are the
        // reference's built-in cube's.
        struct Face {
            float n[3];
            float c[4][3];
        };
        static const Face faces[6] = {
            {{-1, 0, 0}, {{-1, -1, -1}, {-1, -1, 1}, {-1, 1, 1}, {-1, 1, -1}}},
            {{0, 0, -1}, {{1, -1, -1}, {-1, -1, -1}, {-1, 1, -1}, {1, 1, -1}}},
            {{1, 0, 0}, {{1, -1, 1}, {1, -1, -1}, {1, 1, -1}, {1, 1, 1}}},
            {{0, 0, 1}, {{-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}}},
            {{0, 1, 0}, {{-1, 1, 1}, {1, 1, 1}, {1, 1, -1}, {-1, 1, -1}}},
            {{0, -1, 0}, {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1}}},
        };
        static const float uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        Mesh m;
        for (const Face &f : faces) {
            const uint32_t base = (uint32_t)m.positions.size() / 3;
            for (int k = 0; k < 4; k++) {
                m.positions.insert(m.positions.end(), f.c[k], f.c[k] + 3);
                m.normals.insert(m.normals.end(), f.n, f.n + 3);
                m.texcoords.insert(m.texcoords.end(), uv[k], uv[k] + 2);
            }
            for (uint32_t i : {0u, 1u, 2u, 0u, 2u, 3u}) m.indices.push_back(base + i);
        }
        return m;
    }

    bool shape(const xml::Node *n) {
        ShapeInstance ins;
        ins.id = n->attr_or("id", "");
        identity(ins.to_world);
        std::string type = n->attr_or("type", "");
        for (auto &c : n->children)
            if (c->name == "transform" && c->attr_or("name", "to_world") == "to_world")
                if (!transform(c.get(), ins.to_world)) return false;
        if (get_bool(n, "flip_normals", false)) ins.flags |= PT_INST_FLIP_NORMALS;
        if (type == "rectangle") {
            ins.shape_index = add_mesh(rectangle());
        } else if (type == "cube") {
            ins.shape_index = add_mesh(cube());
        } else if (type == "obj") {
            std::string file = get_string(n, "filename", "");
            Mesh mesh;
            std::string e;
            std::string path = (file.size() && file[0] == '/') ? file : m_root_join(file);
            if (!LoadObj(path, mesh, e)) return fail(n, e);
            if (get_bool(n, "face_normals", false)) mesh.normals.clear();
            if (get_bool(n, "flip_tex_coords", true)) ins.flags |= PT_INST_FLIP_TEXCOORDS;
            ins.shape_index = add_mesh(std::move(mesh));
        } else if (type == "sphere") {
            pt_sphere_desc sp{};
            float c[3] = {0, 0, 0};
            get_point(n, "center", c);
            float r = 1.f;
            get_float(n, "radius", r);
            memcpy(sp.center, c, sizeof(c));
            sp.radius = r;
            s.spheres.push_back(sp);
            ins.shape_type = PT_SHAPE_SPHERE;
            ins.shape_index = (uint32_t)s.spheres.size() - 1;
        } else if (type == "hair") {  // resource/shape.cpp:153-181
            std::string file = get_string(n, "filename", "");
            std::string path = (file.size() && file[0] == '/') ? file : m_root_join(file);
            std::string sm = get_string(n, "spline_mode", "cubic");
            uint32_t mode = PT_CURVE_CUBIC_BSPLINE;
            if (sm == "linear") mode = PT_CURVE_LINEAR;
            else if (sm == "quadratic") mode = PT_CURVE_QUADRATIC_BSPLINE;
            else if (sm == "catrom") mode = PT_CURVE_CATMULL_ROM;
            float radius = 0.f;
            get_float(n, "radius", radius);
            Curves cv;
            std::string e;
            if (!LoadCyHair(path, radius, get_bool(n, "tapered", false), mode, cv, e)) return fail(n, e);
            s.curves.push_back(std::move(cv));
            ins.shape_type = PT_SHAPE_CURVES;
            ins.shape_index = (uint32_t)s.curves.size() - 1;
        } else {
            return fail(n, "shape type '" + type + "' is not supported");
        }
        bool has_bsdf = false;
        for (auto &c : n->children) {
            if (c->name == "ref") {
                auto it = s.m_named_bsdf.find(c->attr_or("id", ""));
                if (it == s.m_named_bsdf.end()) return fail(c.get(), "unknown bsdf id '" + c->attr_or("id", "") + "'");
                ins.material = it->second;
                has_bsdf = true;
            } else if (c->name == "bsdf") {
                pt_material_desc m;
                if (!bsdf(c.get(), m)) return false;
                s.materials.push_back(m);
                ins.material = (uint32_t)s.materials.size() - 1;
                has_bsdf = true;
            } else if (c->name == "emitter") {
                std::string et = c->attr_or("type", "");
                if (et != "area") return fail(c.get(), "shape emitter '" + et + "' is not supported");
                pt_texture_desc rad;
                if (!get_texture(c.get(), "radiance", rad, rgb(1, 1, 1))) return false;
                ins.is_emitter = true;
                if (rad.type == PT_TEX_RGB) {
                    memcpy(ins.radiance, rad.color0, sizeof(ins.radiance));
                } else {  // checkerboard or bitmap radiance (AreaEmitter, resource/emitter.h:17-19)
                    ins.radiance_textured = true;
                    ins.radiance_tex = rad;
                }
            }
        }
        if (!has_bsdf) {  // the reference's default material: diffuse 0.5
            pt_material_desc m{};
            for (auto &t : m.tex) t = rgb(0, 0, 0);
            m.type = PT_MAT_DIFFUSE;
            m.tex[0] = rgb(0.5f, 0.5f, 0.5f);
            s.materials.push_back(m);
            ins.material = (uint32_t)s.materials.size() - 1;
        }
        s.shape_instances.push_back(ins);
        return true;
    }

    std::string m_root_join(const std::string &f) { return s.m_root.empty() ? f : s.m_root + "/" + f; }

    // resource/scene.cpp:96-139
    bool sensor(const xml::Node *n) {
        if (n->attr_or("type", "") != "perspective") return fail(n, "only perspective sensors are supported");
        Sensor &se = s.sensor;
        se.fov = 90.f;
        get_float(n, "fov", se.fov);
        get_float(n, "near_clip", se.near_clip);
        get_float(n, "far_clip", se.far_clip);
        for (auto &c : n->children)
            if (c->name == "film") {
                get_int(c.get(), "width", se.width);
                get_int(c.get(), "height", se.height);
            }
        std::string axis = get_string(n, "fov_axis", "x");
        if (axis == "x" || axis == "X") {
            float aspect = (float)se.height / (float)se.width;
            float radian = se.fov * 3.14159265358979323846f / 180.f * 0.5f;
            float t = std::tan(radian) * aspect;
            se.fov = 2.f * std::atan(t) * 180.f / 3.14159265358979323846f;
        } else if (axis != "y" && axis != "Y") {
            return fail(n, "fov_axis must be x or y");
        }
        identity(se.to_world);
        for (auto &c : n->children)
            if (c->name == "transform")
                if (!transform(c.get(), se.to_world)) return false;
        // Mitsuba 3: +X left, +Z view; Pupil: +X right, +Z -view (scene.cpp:130-138).
        // A lookat transform was flipped once already, so it ends up unflipped,
        // exactly as in the reference.
        for (int r = 0; r < 3; r++) {
            se.to_world[4 * r + 0] *= -1.f;
            se.to_world[4 * r + 2] *= -1.f;
        }
        return true;
    }

    bool load(const xml::Node *root) {
        if (root->name != "scene") return fail(root, "root element must be <scene>");
        for (auto &c : root->children)
            if (c->name == "default") s.m_defaults[c->attr_or("name", "")] = c->attr_or("value", "");
        for (auto &c : root->children) {
            const xml::Node *n = c.get();
            if (n->name == "integrator") {
                uint32_t d = 1;
                get_int(n, "max_depth", d);
                s.max_depth = d;
            } else if (n->name == "sensor") {
                if (!sensor(n)) return false;
            } else if (n->name == "bsdf") {
                pt_material_desc m;
                if (!bsdf(n, m)) return false;
                s.materials.push_back(m);
                std::string id = n->attr_or("id", "");
                if (!id.empty()) s.m_named_bsdf[id] = (uint32_t)s.materials.size() - 1;
            } else if (n->name == "shape") {
                if (!shape(n)) return false;
            } else if (n->name == "emitter") {
                std::string et = n->attr_or("type", "");
                if (et == "constant") {
                    pt_texture_desc r;
                    if (!get_texture(n, "radiance", r, rgb(1, 1, 1))) return false;
                    s.has_env = true;
                    memcpy(s.env_radiance, r.color0, sizeof(s.env_radiance));
                } else if (et == "envmap") {  // scene.cpp:208-221
                    const xml::Node *fn = prop(n, "string", "filename");
                    if (!fn) return fail(n, "envmap emitter without a filename");
                    std::vector<float> px;
                    uint32_t w = 0, h = 0;
                    std::string e;
                    if (!util::LoadImageRGBA(m_root_path(value(fn)), px, w, h, e)) return fail(n, e);
                    s.images.push_back(std::move(px));
                    s.env_map.on = true;
                    s.env_map.image = s.images.size() - 1;
                    s.env_map.width = w;
                    s.env_map.height = h;
                    s.env_map.scale = 1.f;
                    if (const xml::Node *sc = prop(n, "float", "scale")) {
                        auto v = numbers(value(sc));
                        if (v.size() == 1) s.env_map.scale = v[0];
                    }
                    for (auto &t : n->children)
                        if (t->name == "transform" && !transform(t.get(), s.env_map.to_world)) return false;
                    s.has_env = true;
                } else if (et == "point") {
                    // Parsed by the reference (resource/scene.cpp:194-202) but never
                    // placed in its emitter tables (world/emitter.cpp:314-315 leaves
                    // the Point case as a TODO), so it lights nothing there: accepted
                    // and dropped here the same way.
                    continue;
                } else {
                    return fail(n, "emitter '" + et + "' is not supported");
                }
            } else if (n->name == "default" || n->name == "texture") {
                continue;
            }
        }
        return err.empty();
    }
};

bool Scene::LoadFromString(const std::string &text, const std::string &root_dir) {
    *this = Scene();
    m_root = root_dir;
    std::string perr;
    auto root = xml::Parse(text, perr);
    if (!root) {
        m_error = perr;
        return false;
    }
    Loader l{*this, m_error};
    // malformed or out-of-range numbers surface as std::stof / std::stod
    // exceptions; they end the load with an error instead of leaving the library
    try {
        return l.load(root.get());
    } catch (const std::invalid_argument &) {
        m_error = "malformed number in the scene description";
    } catch (const std::out_of_range &) {
        m_error = "number out of range in the scene description";
    } catch (const std::exception &e) {
        m_error = std::string("scene load failed: ") + e.what();
    }
    return false;
}

bool Scene::LoadFromXML(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        m_error = "cannot open " + path;
        return false;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    size_t slash = path.find_last_of('/');
    return LoadFromString(ss.str(), slash == std::string::npos ? "" : path.substr(0, slash));
}

const pt_scene_desc &Scene::Desc() {
    m_mesh_descs.clear();
    for (auto &m : meshes) {
        pt_mesh_desc d{};
        d.positions = m.positions.data();
        d.normals = m.normals.empty() ? nullptr : m.normals.data();
        d.texcoords = m.texcoords.empty() ? nullptr : m.texcoords.data();
        d.indices = m.indices.data();
        d.num_vertices = (uint32_t)m.positions.size() / 3;
        d.num_triangles = (uint32_t)m.indices.size() / 3;
        m_mesh_descs.push_back(d);
    }
    m_inst_descs.clear();
    for (auto &s : shape_instances) {
        pt_instance_desc d{};
        d.shape_type = s.shape_type;
        d.shape_index = s.shape_index;
        d.material = s.material;
        d.flags = s.flags;
        memcpy(d.to_world, s.to_world, sizeof(d.to_world));
        d.is_emitter = s.is_emitter ? 1 : 0;
        memcpy(d.radiance, s.radiance, sizeof(d.radiance));
        d.radiance_textured = s.radiance_textured ? 1u : 0u;
        d.radiance_tex = s.radiance_tex;
        m_inst_descs.push_back(d);
    }
    m_desc = pt_scene_desc{};
    m_desc.meshes = m_mesh_descs.data();
    m_desc.num_meshes = (uint32_t)m_mesh_descs.size();
    m_desc.spheres = spheres.data();
    m_desc.num_spheres = (uint32_t)spheres.size();
    m_desc.materials = materials.data();
    m_desc.num_materials = (uint32_t)materials.size();
    m_desc.instances = m_inst_descs.data();
    m_desc.num_instances = (uint32_t)m_inst_descs.size();
    m_curve_descs.clear();
    for (auto &c : curves) {
        pt_curves_desc d{};
        d.positions = c.positions.data();
        d.radii = c.radii.data();
        d.segments = c.segments.data();
        d.num_points = (uint32_t)c.radii.size();
        d.num_segments = (uint32_t)c.segments.size();
        d.type = c.type;
        m_curve_descs.push_back(d);
    }
    m_desc.curves = m_curve_descs.data();
    m_desc.num_curves = (uint32_t)m_curve_descs.size();
    m_desc.env.type = has_env ? PT_ENV_CONST : PT_ENV_NONE;
    memcpy(m_desc.env.radiance, env_radiance, sizeof(env_radiance));
    if (env_map.on) {
        m_desc.env.type = PT_ENV_MAP;
        m_desc.env.pixels = images[env_map.image].data();
        m_desc.env.width = env_map.width;
        m_desc.env.height = env_map.height;
        m_desc.env.scale = env_map.scale;
        memcpy(m_desc.env.to_world, env_map.to_world, sizeof(env_map.to_world));
    }
    m_desc.camera = Camera();
    m_desc.width = sensor.width;
    m_desc.height = sensor.height;
    m_desc.max_depth = max_depth;
    return m_desc;
}

pt_camera_desc Scene::Camera() const {
    pt_camera_desc c{};
    pt_camera_make(sensor.fov, (float)sensor.width / (float)sensor.height, sensor.near_clip, sensor.far_clip,
                   sensor.to_world, &c);
    return c;
}

bool LoadObj(const std::string &path, Mesh &out, std::string &error) {
    std::ifstream f(path);
    if (!f) {
        error = "cannot open " + path;
        return false;
    }
    std::vector<float> P, N, T;
    std::map<std::tuple<long, long, long>, uint32_t> remap;
    out = Mesh();
    bool any_vn = false, any_vt = false, all_vn = true;
    std::string line;
    int lineno = 0;
    std::vector<uint32_t> poly;
    auto resolve = [](long i, size_t n) -> long { return i > 0 ? i - 1 : (long)n + i; };
    while (std::getline(f, line)) {
        lineno++;
        std::istringstream is(line);
        std::string tag;
        if (!(is >> tag)) continue;
        if (tag == "v") {
            float x, y, z;
            is >> x >> y >> z;
            P.insert(P.end(), {x, y, z});
        } else if (tag == "vn") {
            float x, y, z;
            is >> x >> y >> z;
            N.insert(N.end(), {x, y, z});
        } else if (tag == "vt") {
            float u, v;
            is >> u >> v;
            T.insert(T.end(), {u, v});
        } else if (tag == "f") {
            poly.clear();
            std::string tok;
            while (is >> tok) {
                long vi = 0, ti = 0, ni = 0;
                size_t a = tok.find('/');
                try {
                    vi = std::stol(tok.substr(0, a));
                    if (a != std::string::npos) {
                        size_t b = tok.find('/', a + 1);
                        std::string ts = tok.substr(a + 1, b == std::string::npos ? std::string::npos : b - a - 1);
                        if (!ts.empty()) ti = std::stol(ts);
                        if (b != std::string::npos && b + 1 < tok.size()) ni = std::stol(tok.substr(b + 1));
                    }
                } catch (const std::exception &) {
                    error = path + ":" + std::to_string(lineno) + ": malformed face index '" + tok + "'";
                    return false;
                }
                long rv = resolve(vi, P.size() / 3), rt = ti ? resolve(ti, T.size() / 2) : -1,
                     rn = ni ? resolve(ni, N.size() / 3) : -1;
                if (rv < 0 || rv >= (long)P.size() / 3 || (ti && (rt < 0 || rt >= (long)T.size() / 2)) ||
                    (ni && (rn < 0 || rn >= (long)N.size() / 3))) {
                    error = path + ":" + std::to_string(lineno) + ": face index out of range";
                    return false;
                }
                auto key = std::make_tuple(rv, rt, rn);
                auto it = remap.find(key);
                uint32_t id;
                if (it == remap.end()) {
                    id = (uint32_t)out.positions.size() / 3;
                    remap[key] = id;
                    out.positions.insert(out.positions.end(), {P[3 * rv], P[3 * rv + 1], P[3 * rv + 2]});
                    if (rn >= 0) {
                        any_vn = true;
                        out.normals.insert(out.normals.end(), {N[3 * rn], N[3 * rn + 1], N[3 * rn + 2]});
                    } else {
                        all_vn = false;
                        out.normals.insert(out.normals.end(), {0.f, 0.f, 0.f});
                    }
                    if (rt >= 0) {
                        any_vt = true;
                        out.texcoords.insert(out.texcoords.end(), {T[2 * rt], T[2 * rt + 1]});
                    } else {
                        out.texcoords.insert(out.texcoords.end(), {0.f, 0.f});
                    }
                } else {
                    id = it->second;
                }
                poly.push_back(id);
            }
            for (size_t k = 1; k + 1 < poly.size(); k++) out.indices.insert(out.indices.end(), {poly[0], poly[k], poly[k + 1]});
        }
    }
    if (!any_vn || !all_vn) out.normals.clear();  // partial normals: use geometric normals throughout
    if (!any_vt) out.texcoords.clear();
    if (out.indices.empty()) {
        error = path + ": no faces";
        return false;
    }
    return true;
}

}  // namespace Pupil::resource
