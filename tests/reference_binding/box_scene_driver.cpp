// Test driver for the reference-side binding (pupiloptixlab_gb300/host/
// reference_binding/): builds tests/scenes/box.xml in the reference's own data
// model (resource::Scene with ShapeInstances sharing the built-in rectangle
// and cube shapes, per-instance Materials, an area emitter, the sensor after
// the mitsuba -> Pupil flip), then
//   dump            converts it with ToPtSceneDesc and prints the descriptor,
//                   expanded per instance, as one JSON object (float bits as
//                   integers) for comparison with the library's XML loader;
//   run FRAMES OUT  puts it into a World, dispatches the SceneLoad event to a
//                   WavefrontPTPass, calls OnRun FRAMES times and writes the
//                   "final result" buffer (float4 per pixel) to OUT.
// Test infrastructure only.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "system/buffer.h"
#include "system/system.h"
#include "to_pt_scene_desc.h"
#include "util/event.h"
#include "wavefront_pass.h"
#include "world/world.h"

using namespace Pupil;

namespace {

// the reference's built-in shapes (framework/resource/shape.cpp:19-69)
float rect_p[] = {-1, -1, 0, 1, -1, 0, 1, 1, 0, -1, 1, 0};
float rect_n[] = {0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1};
float rect_t[] = {0, 0, 1, 0, 1, 1, 0, 1};
uint32_t rect_i[] = {0, 1, 2, 0, 2, 3};
float cube_p[] = {-1, -1, -1, -1, -1, 1, -1, 1, 1, -1, 1, -1, 1, -1, -1, -1, -1, -1, -1, 1, -1, 1, 1, -1,
                  1, -1, 1, 1, -1, -1, 1, 1, -1, 1, 1, 1, -1, -1, 1, 1, -1, 1, 1, 1, 1, -1, 1, 1,
                  -1, 1, 1, 1, 1, 1, 1, 1, -1, -1, 1, -1, -1, -1, -1, 1, -1, -1, 1, -1, 1, -1, -1, 1};
float cube_n[] = {-1, 0, 0, -1, 0, 0, -1, 0, 0, -1, 0, 0, 0, 0, -1, 0, 0, -1, 0, 0, -1, 0, 0, -1,
                  1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1,
                  0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, -1, 0, 0, -1, 0, 0, -1, 0, 0, -1, 0};
float cube_t[] = {0, 0, 1, 0, 1, 1, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1,
                  0, 0, 1, 0, 1, 1, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1};
uint32_t cube_i[] = {0, 1, 2, 0, 2, 3, 4, 5, 6, 4, 6, 7, 8, 9, 10, 8, 10, 11,
                     12, 13, 14, 12, 14, 15, 16, 17, 18, 16, 18, 19, 20, 21, 22, 20, 22, 23};

// util::Transform's operations (framework/util/transform.cpp): each one
// left-multiplies the matrix, in float
util::Mat4 mul(const util::Mat4 &a, const util::Mat4 &b) {
    util::Mat4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float s = 0.f;
            for (int k = 0; k < 4; k++) s += a.re[i][k] * b.re[k][j];
            r.re[i][j] = s;
        }
    return r;
}
void scale(util::Transform &t, float x, float y, float z) {
    t.matrix = mul(util::Mat4(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1), t.matrix);
}
void translate(util::Transform &t, float x, float y, float z) {
    t.matrix = mul(util::Mat4(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1), t.matrix);
}
void rotate(util::Transform &t, float ux, float uy, float uz, float angle) {
    float len = std::sqrt(ux * ux + uy * uy + uz * uz);
    ux /= len, uy /= len, uz /= len;
    float theta = angle / 180.f * 3.14159265358979323846f;
    float a = std::cos(0.5f * theta), b = std::sin(0.5f * theta) * ux, c = std::sin(0.5f * theta) * uy,
          d = std::sin(0.5f * theta) * uz;
    util::Mat4 r(1.f - 2.f * c * c - 2.f * d * d, 2.f * b * c - 2.f * a * d, 2.f * a * c + 2.f * b * d, 0.f,
                 2.f * b * c + 2.f * a * d, 1.f - 2.f * b * b - 2.f * d * d, 2.f * c * d - 2.f * a * b, 0.f,
                 2.f * b * d - 2.f * a * c, 2.f * a * b + 2.f * c * d, 1.f - 2.f * b * b - 2.f * c * c, 0.f,
                 0.f, 0.f, 0.f, 1.f);
    t.matrix = mul(r, t.matrix);
}

resource::Shape make_mesh_shape(resource::EShapeType type, float *p, float *n, float *t, uint32_t *i, uint32_t nv,
                                uint32_t nf) {
    resource::Shape s;
    s.type = type;
    s.mesh = resource::Mesh{false, false, false, nv, nf, p, n, t, i};
    return s;
}

resource::Material diffuse(float r, float g, float b) {
    resource::Material m;
    m.type = EMatType::Diffuse;
    m.twosided = true;
    m.diffuse.reflectance.type = util::ETextureType::RGB;
    m.diffuse.reflectance.rgb.color = util::Float3(r, g, b);
    return m;
}

void build_box(resource::Scene &s, resource::Shape &rect, resource::Shape &cube) {
    s.integrator.max_depth = 5;
    s.sensor.fov = 40.f;  // fov_axis y: kept as is
    s.sensor.film = resource::Film{48, 48};
    util::Mat4 m(-1, 0, 0, 0, 0, 1, 0, 1, 0, 0, -1, 3.8f, 0, 0, 0, 1);
    for (int r = 0; r < 3; r++) m.re[r][0] *= -1, m.re[r][2] *= -1;  // mitsuba -> Pupil (resource/scene.cpp:130-137)
    s.sensor.transform.matrix = m;
    auto add = [&](const char *name, resource::Shape *shape, resource::Material mat, util::Transform t) {
        resource::ShapeInstance ins;
        ins.name = name;
        ins.shape = shape;
        ins.mat = mat;
        ins.transform = t;
        s.shape_instances.push_back(ins);
        return &s.shape_instances.back();
    };
    const resource::Material white = diffuse(0.73f, 0.73f, 0.73f), red = diffuse(0.65f, 0.05f, 0.05f),
                             green = diffuse(0.12f, 0.45f, 0.15f), black = diffuse(0.f, 0.f, 0.f);
    s.shape_instances.reserve(8);
    util::Transform t;
    rotate(t, 1, 0, 0, -90), translate(t, 0, 0, 0);
    add("floor", &rect, white, t);
    t = util::Transform();
    rotate(t, 1, 0, 0, 90), translate(t, 0, 2, 0);
    add("ceiling", &rect, white, t);
    t = util::Transform();
    translate(t, 0, 1, -1);
    add("back", &rect, white, t);
    t = util::Transform();
    rotate(t, 0, 1, 0, 90), translate(t, -1, 1, 0);
    add("left", &rect, red, t);
    t = util::Transform();
    rotate(t, 0, 1, 0, -90), translate(t, 1, 1, 0);
    add("right", &rect, green, t);
    t = util::Transform();
    scale(t, 0.3f, 0.6f, 0.3f), rotate(t, 0, 1, 0, 15), translate(t, -0.33f, 0.6f, -0.29f);
    add("tall", &cube, white, t);
    t = util::Transform();
    scale(t, 0.3f, 0.3f, 0.3f), rotate(t, 0, 1, 0, -18), translate(t, 0.33f, 0.3f, 0.37f);
    add("short", &cube, white, t);
    t = util::Transform();
    scale(t, 0.125f, 0.125f, 0.125f), rotate(t, 1, 0, 0, 90), translate(t, 0, 1.98f, 0);
    resource::ShapeInstance *lamp = add("lamp", &rect, black, t);
    lamp->is_emitter = true;
    lamp->emitter.type = resource::EEmitterType::Area;
    lamp->emitter.area.radiance.type = util::ETextureType::RGB;
    lamp->emitter.area.radiance.rgb.color = util::Float3(17.f, 12.f, 4.f);
}

unsigned bits(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}
void floats(std::string &o, const char *key, const float *p, size_t n) {
    o += "\"";
    o += key;
    o += "\": [";
    for (size_t i = 0; i < n; i++) o += (i ? "," : "") + std::to_string(p ? bits(p[i]) : 0u);
    o += "], ";
}
void uints(std::string &o, const char *key, const uint32_t *p, size_t n) {
    o += "\"";
    o += key;
    o += "\": [";
    for (size_t i = 0; i < n; i++) o += (i ? "," : "") + std::to_string(p ? p[i] : 0u);
    o += "], ";
}

}  // namespace

int main(int argc, char **argv) {
    resource::Shape rect = make_mesh_shape(resource::EShapeType::_rectangle, rect_p, rect_n, rect_t, rect_i, 4, 2);
    resource::Shape cube = make_mesh_shape(resource::EShapeType::_cube, cube_p, cube_n, cube_t, cube_i, 24, 12);
    const std::string mode = argc > 1 ? argv[1] : "dump";
    pt_camera_desc cam{};
    if (mode == "dump") {
        resource::Scene s;
        build_box(s, rect, cube);
        pt_camera_make(s.sensor.fov, (float)s.sensor.film.w / (float)s.sensor.film.h, s.sensor.near_clip,
                       s.sensor.far_clip, s.sensor.transform.matrix.e, &cam);
        pt::PtSceneDesc d;
        std::string err;
        if (!pt::ToPtSceneDesc(s, cam, d, &err)) {
            std::fprintf(stderr, "ToPtSceneDesc: %s\n", err.c_str());
            return 2;
        }
        const pt_scene_desc &sd = d.desc;
        std::string o = "{";
        o += "\"width\": " + std::to_string(sd.width) + ", \"height\": " + std::to_string(sd.height) +
             ", \"max_depth\": " + std::to_string(sd.max_depth) + ", \"env_type\": " + std::to_string(sd.env.type) +
             ", \"num_meshes\": " + std::to_string(sd.num_meshes) + ", ";
        floats(o, "camera", sd.camera.sample_to_camera, 32);
        o += "\"instances\": [";
        for (uint32_t i = 0; i < sd.num_instances; i++) {
            const pt_instance_desc &in = sd.instances[i];
            const pt_mesh_desc &m = sd.meshes[in.shape_index];
            const pt_material_desc &mt = sd.materials[in.material];
            o += i ? ", {" : "{";
            o += "\"shape_type\": " + std::to_string(in.shape_type) + ", \"flags\": " + std::to_string(in.flags) +
                 ", \"is_emitter\": " + std::to_string(in.is_emitter) + ", ";
            floats(o, "radiance", in.radiance, 3);
            floats(o, "to_world", in.to_world, 16);
            floats(o, "positions", m.positions, 3ull * m.num_vertices);
            floats(o, "normals", m.normals, m.normals ? 3ull * m.num_vertices : 0);
            floats(o, "texcoords", m.texcoords, m.texcoords ? 2ull * m.num_vertices : 0);
            uints(o, "indices", m.indices, 3ull * m.num_triangles);
            o += "\"material\": {\"type\": " + std::to_string(mt.type) + ", \"twosided\": " +
                 std::to_string(mt.twosided) + ", \"nonlinear\": " + std::to_string(mt.nonlinear) + ", ";
            floats(o, "ior", &mt.int_ior, 2);
            o += "\"tex\": [";
            for (int k = 0; k < 4; k++) {
                const pt_texture_desc &t = mt.tex[k];
                o += k ? ", {" : "{";
                o += "\"type\": " + std::to_string(t.type) + ", ";
                floats(o, "color0", t.color0, 3);
                floats(o, "color1", t.color1, 3);
                floats(o, "uv", t.uv_transform, 8);
                o += "\"wh\": [" + std::to_string(t.width) + "," + std::to_string(t.height) + "]}";
            }
            o += "]}}";
        }
        o += "]}";
        std::puts(o.c_str());
        return 0;
    }
    if (mode == "run" && argc > 3) {
        // World with the scene and a device copy of its optix::Camera
        auto *world = util::Singleton<world::World>::instance();
        world->scene = std::make_unique<resource::Scene>();
        build_box(*world->scene, rect, cube);
        const resource::Sensor &sn = world->scene->sensor;
        pt_camera_make(sn.fov, (float)sn.film.w / (float)sn.film.h, sn.near_clip, sn.far_clip, sn.transform.matrix.e,
                       &cam);
        void *dcam = nullptr;
        cudaMalloc(&dcam, sizeof(cam));
        cudaMemcpy(dcam, &cam, sizeof(cam), cudaMemcpyHostToDevice);
        world->camera = std::make_unique<world::CameraHelper>();
        world->camera->m_camera_cuda_memory = reinterpret_cast<unsigned long long>(dcam);
        pt::WavefrontPTPass pass;
        EventDispatcher<ESystemEvent::SceneLoad>(world);  // System::SetScene's event (system.cpp)
        const int frames = std::atoi(argv[2]);
        for (int f = 0; f < frames; f++) pass.Run();
        if (pass.last_status() != PT_OK) return 3;
        Buffer *out = util::Singleton<BufferManager>::instance()->GetBuffer("final result");
        std::vector<float> img(4ull * sn.film.w * sn.film.h);
        cudaMemcpy(img.data(), reinterpret_cast<void *>(out->cuda_ptr), img.size() * 4, cudaMemcpyDeviceToHost);
        FILE *f = std::fopen(argv[3], "wb");
        if (!f) return 4;
        std::fwrite(img.data(), 4, img.size(), f);
        std::fclose(f);
        std::printf("%u frames\n", pass.sample_count());
        cudaFree(dcam);
        return 0;
    }
    std::fprintf(stderr, "usage: %s dump | run FRAMES OUT\n", argv[0]);
    return 1;
}
