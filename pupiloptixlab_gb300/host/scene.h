// scene.h -- mitsuba3-style scene loading into the tracer's scene descriptor.
//
// The host-side counterpart of resource::Scene (framework/resource/scene.h:
// 39-57): integrator, perspective sensor + film, shapes (obj, rectangle,
// cube, sphere, hair) with to_world transforms, the seven BSDFs plus
// `twosided`, bitmap and checkerboard textures, area emitters on shapes, the
// constant environment and the environment map.  `$name` values are
// substituted from <default> entries and <ref id=...> resolves named BSDFs,
// as in framework/resource/xml/visitor.h.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "pt_api.h"

namespace Pupil::resource {

struct Mesh {
    std::vector<float> positions, normals, texcoords;
    std::vector<uint32_t> indices;
};

// Curve strands (resource::Shape _hair): control points, per-point radii,
// first control point of every segment, PT_CURVE_* type.
struct Curves {
    std::vector<float> positions, radii;
    std::vector<uint32_t> segments;
    uint32_t type = PT_CURVE_CUBIC_BSPLINE;
};

struct ShapeInstance {
    std::string id;
    uint32_t shape_type = PT_SHAPE_MESH;
    uint32_t shape_index = 0;
    uint32_t material = 0;
    uint32_t flags = 0;
    float to_world[16];
    bool is_emitter = false;
    float radiance[3] = {0, 0, 0};
    bool radiance_textured = false;  // radiance from radiance_tex (checkerboard or bitmap)
    pt_texture_desc radiance_tex{};
};

struct Sensor {
    float fov = 90.f;  // vertical, degrees (after the fov_axis conversion)
    float near_clip = 0.01f;
    float far_clip = 10000.f;
    float to_world[16];  // Pupil convention: +X right, +Y up, +Z away from the view
    uint32_t width = 768, height = 576;
};

class Scene {
public:
    uint32_t max_depth = 1;
    Sensor sensor;
    std::vector<Mesh> meshes;
    std::vector<pt_sphere_desc> spheres;
    std::vector<Curves> curves;
    std::vector<pt_material_desc> materials;
    std::vector<ShapeInstance> shape_instances;
    bool has_env = false;
    float env_radiance[3] = {0, 0, 0};
    // decoded bitmap images (RGBA float); textures and the environment map point into them
    std::vector<std::vector<float>> images;
    struct EnvMap {
        bool on = false;
        size_t image = 0;
        uint32_t width = 0, height = 0;
        float scale = 1.f;
        float to_world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    } env_map;

    bool LoadFromXML(const std::string &path);
    bool LoadFromString(const std::string &text, const std::string &root_dir);
    const std::string &error() const { return m_error; }

    // Descriptor pointing into this object (valid until the scene changes).
    const pt_scene_desc &Desc();
    pt_camera_desc Camera() const;

private:
    std::string m_error;
    std::string m_root;
    std::map<std::string, std::string> m_defaults;
    std::map<std::string, uint32_t> m_named_bsdf;
    std::vector<pt_mesh_desc> m_mesh_descs;
    std::vector<pt_instance_desc> m_inst_descs;
    std::vector<pt_curves_desc> m_curve_descs;
    pt_scene_desc m_desc{};
    friend struct Loader;
};

// Wavefront OBJ (v / vt / vn / f, polygons fan-triangulated).
bool LoadObj(const std::string &path, Mesh &out, std::string &error);

// Cem Yuksel's HAIR file as curve strands (hair.cpp): radius 0 keeps the
// file's thickness, tapered strands fall to zero radius at the tip, mode is
// the PT_CURVE_* type.
bool LoadCyHair(const std::string &path, float radius, bool tapered, uint32_t mode, Curves &out, std::string &error);

}  // namespace Pupil::resource
