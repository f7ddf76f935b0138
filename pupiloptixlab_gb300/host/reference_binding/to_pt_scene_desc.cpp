// to_pt_scene_desc.cpp -- resource::Scene -> pt_scene_desc (see the header).
#include "to_pt_scene_desc.h"

#include <cstring>

namespace Pupil::pt {

pt_texture_desc ToPtTexture(const util::Texture &t) {
    pt_texture_desc d;
    std::memset(&d, 0, sizeof(d));
    switch (t.type) {
        case util::ETextureType::RGB:
            d.type = PT_TEX_RGB;
            for (int i = 0; i < 3; i++) d.color0[i] = t.rgb.color.e[i];
            break;
        case util::ETextureType::Checkerboard:
            d.type = PT_TEX_CHECKERBOARD;
            for (int i = 0; i < 3; i++) {
                d.color0[i] = t.checkerboard.patch1.e[i];
                d.color1[i] = t.checkerboard.patch2.e[i];
            }
            break;
        case util::ETextureType::Bitmap:
            d.type = PT_TEX_BITMAP;
            d.pixels = t.bitmap.data;  // RGBA floats, w * h
            d.width = (uint32_t)t.bitmap.w;
            d.height = (uint32_t)t.bitmap.h;
            // the values of cudaTextureAddressMode / cudaTextureFilterMode, as
            // framework/cuda/texture.cpp:82-84 casts them
            d.address_mode = (uint32_t)t.bitmap.address_mode;
            d.filter = (uint32_t)t.bitmap.filter_mode;
            break;
    }
    // the first two rows of the row-major uv transform
    std::memcpy(d.uv_transform, t.transform.matrix.e, sizeof(d.uv_transform));
    return d;
}

namespace {

pt_material_desc ToPtMaterial(const resource::Material &m) {
    pt_material_desc d;
    std::memset(&d, 0, sizeof(d));
    d.type = (uint32_t)m.type;  // EMatType and pt_material_type share their values
    d.twosided = m.twosided ? 1u : 0u;
    const pt_texture_desc unused = ToPtTexture(util::Texture{});  // black RGB, identity uv transform
    for (pt_texture_desc &t : d.tex) t = unused;
    switch (m.type) {  // texture slots per type: include/pt_api.h
        case EMatType::Diffuse:
            d.tex[0] = ToPtTexture(m.diffuse.reflectance);
            break;
        case EMatType::Dielectric:
            d.int_ior = m.dielectric.int_ior;
            d.ext_ior = m.dielectric.ext_ior;
            d.tex[0] = ToPtTexture(m.dielectric.specular_reflectance);
            d.tex[1] = ToPtTexture(m.dielectric.specular_transmittance);
            break;
        case EMatType::RoughDielectric:
            d.int_ior = m.rough_dielectric.int_ior;
            d.ext_ior = m.rough_dielectric.ext_ior;
            d.tex[0] = ToPtTexture(m.rough_dielectric.specular_reflectance);
            d.tex[1] = ToPtTexture(m.rough_dielectric.specular_transmittance);
            d.tex[2] = ToPtTexture(m.rough_dielectric.alpha);
            break;
        case EMatType::Conductor:
            d.tex[0] = ToPtTexture(m.conductor.specular_reflectance);
            d.tex[1] = ToPtTexture(m.conductor.eta);
            d.tex[2] = ToPtTexture(m.conductor.k);
            break;
        case EMatType::RoughConductor:
            d.tex[0] = ToPtTexture(m.rough_conductor.specular_reflectance);
            d.tex[1] = ToPtTexture(m.rough_conductor.eta);
            d.tex[2] = ToPtTexture(m.rough_conductor.k);
            d.tex[3] = ToPtTexture(m.rough_conductor.alpha);
            break;
        case EMatType::Plastic:
            d.int_ior = m.plastic.int_ior;
            d.ext_ior = m.plastic.ext_ior;
            d.nonlinear = m.plastic.nonlinear ? 1u : 0u;
            d.tex[0] = ToPtTexture(m.plastic.diffuse_reflectance);
            d.tex[1] = ToPtTexture(m.plastic.specular_reflectance);
            break;
        case EMatType::RoughPlastic:
            d.int_ior = m.rough_plastic.int_ior;
            d.ext_ior = m.rough_plastic.ext_ior;
            d.nonlinear = m.rough_plastic.nonlinear ? 1u : 0u;
            d.tex[0] = ToPtTexture(m.rough_plastic.diffuse_reflectance);
            d.tex[1] = ToPtTexture(m.rough_plastic.specular_reflectance);
            d.tex[2] = ToPtTexture(m.rough_plastic.alpha);
            break;
        default:
            break;
    }
    return d;
}

void set_error(std::string *error, const std::string &msg) {
    if (error) *error = msg;
}

}  // namespace

bool ToPtSceneDesc(const resource::Scene &scene, const pt_camera_desc &camera, PtSceneDesc &out, std::string *error) {
    out = PtSceneDesc{};
    std::unordered_map<const resource::Shape *, uint32_t> shape_index;
    for (size_t i = 0; i < scene.shape_instances.size(); i++) {
        const resource::ShapeInstance &ins = scene.shape_instances[i];
        const resource::Shape *shape = ins.shape;
        if (!shape) {
            set_error(error, "shape instance " + std::to_string(i) + " (" + ins.name + ") has no shape");
            return false;
        }
        pt_instance_desc d;
        std::memset(&d, 0, sizeof(d));
        auto known = shape_index.find(shape);
        switch (shape->type) {
            case resource::EShapeType::_obj:
            case resource::EShapeType::_cube:
            case resource::EShapeType::_rectangle: {
                const resource::Mesh &m = shape->mesh;
                d.shape_type = PT_SHAPE_MESH;
                if (known == shape_index.end()) {
                    pt_mesh_desc md;
                    std::memset(&md, 0, sizeof(md));
                    md.positions = m.positions;
                    // face_normals: the geometric normal (framework/render/geometry.h:82-90)
                    md.normals = (m.face_normals || !m.normals) ? nullptr : m.normals;
                    md.texcoords = m.texcoords;
                    md.indices = m.indices;
                    md.num_vertices = m.vertex_num;
                    md.num_triangles = m.face_num;
                    known = shape_index.emplace(shape, (uint32_t)out.meshes.size()).first;
                    out.meshes.push_back(md);
                }
                d.flags = (m.flip_normals ? (uint32_t)PT_INST_FLIP_NORMALS : 0u) |
                          (m.flip_tex_coords ? (uint32_t)PT_INST_FLIP_TEXCOORDS : 0u);
                break;
            }
            case resource::EShapeType::_sphere: {
                // the shared unit sphere: centre and radius are in the instance
                // transform (framework/resource/shape.cpp:113-133; the render
                // object uses centre 0, radius 1, world/render_object.cpp:30-35)
                d.shape_type = PT_SHAPE_SPHERE;
                if (known == shape_index.end()) {
                    known = shape_index.emplace(shape, (uint32_t)out.spheres.size()).first;
                    out.spheres.push_back(pt_sphere_desc{{0.f, 0.f, 0.f}, 1.f});
                }
                d.flags = shape->sphere.flip_normals ? (uint32_t)PT_INST_FLIP_NORMALS : 0u;
                break;
            }
            case resource::EShapeType::_hair: {
                const resource::Hair &h = shape->hair;
                d.shape_type = PT_SHAPE_CURVES;
                if (known == shape_index.end()) {
                    pt_curves_desc cd;
                    std::memset(&cd, 0, sizeof(cd));
                    cd.positions = h.positions;
                    cd.radii = h.widths;  // OptiX curve "widths" are radii
                    cd.segments = h.segments_index;
                    cd.num_points = h.point_num;
                    cd.num_segments = h.segments_num;
                    cd.type = h.flags & 3u;
                    known = shape_index.emplace(shape, (uint32_t)out.curves.size()).first;
                    out.curves.push_back(cd);
                }
                break;
            }
            default:
                set_error(error, "shape instance " + std::to_string(i) + " (" + ins.name + ") has an unknown shape type");
                return false;
        }
        d.shape_index = known->second;
        d.material = (uint32_t)out.materials.size();  // every ShapeInstance carries its own Material
        out.materials.push_back(ToPtMaterial(ins.mat));
        std::memcpy(d.to_world, ins.transform.matrix.e, sizeof(d.to_world));
        if (ins.is_emitter && ins.emitter.type == resource::EEmitterType::Area) {
            const util::Texture &r = ins.emitter.area.radiance;
            d.is_emitter = 1;
            if (r.type == util::ETextureType::RGB) {
                for (int k = 0; k < 3; k++) d.radiance[k] = r.rgb.color.e[k];
            } else {  // checkerboard or bitmap radiance
                d.radiance_textured = 1;
                d.radiance_tex = ToPtTexture(r);
            }
        }
        out.instances.push_back(d);
    }
    pt_env_desc env;
    std::memset(&env, 0, sizeof(env));
    env.type = PT_ENV_NONE;
    for (const resource::Emitter &e : scene.emitters) {
        if (e.type == resource::EEmitterType::ConstEnv) {
            env.type = PT_ENV_CONST;
            for (int k = 0; k < 3; k++) env.radiance[k] = e.const_env.radiance.e[k];
        } else if (e.type == resource::EEmitterType::EnvMap) {
            env.type = PT_ENV_MAP;
            env.pixels = e.env_map.radiance.bitmap.data;
            env.width = (uint32_t)e.env_map.radiance.bitmap.w;
            env.height = (uint32_t)e.env_map.radiance.bitmap.h;
            env.scale = e.env_map.scale;
            std::memcpy(env.to_world, e.env_map.transform.matrix.e, sizeof(env.to_world));
        }
    }
    pt_scene_desc &s = out.desc;
    std::memset(&s, 0, sizeof(s));
    s.meshes = out.meshes.data();
    s.num_meshes = (uint32_t)out.meshes.size();
    s.spheres = out.spheres.data();
    s.num_spheres = (uint32_t)out.spheres.size();
    s.curves = out.curves.data();
    s.num_curves = (uint32_t)out.curves.size();
    s.materials = out.materials.data();
    s.num_materials = (uint32_t)out.materials.size();
    s.instances = out.instances.data();
    s.num_instances = (uint32_t)out.instances.size();
    s.env = env;
    s.camera = camera;
    s.width = (uint32_t)scene.sensor.film.w;
    s.height = (uint32_t)scene.sensor.film.h;
    s.max_depth = (uint32_t)scene.integrator.max_depth;
    return true;
}

}  // namespace Pupil::pt
