// Declaration subset of framework/resource/shape.h:31-97: shape kinds, the
// mesh / sphere / hair payloads, Shape and ShapeInstance.
#pragma once
#include <cstdint>
#include <string>
#include "material.h"
#include "emitter.h"
#include "util/transform.h"

namespace Pupil::resource {
enum class EShapeType : unsigned int { _unknown = 0, _obj, _sphere, _cube, _rectangle, _hair, _count };

struct Mesh {
    bool face_normals;
    bool flip_normals;
    bool flip_tex_coords;
    uint32_t vertex_num;
    uint32_t face_num;
    float *positions;
    float *normals;
    float *texcoords;
    uint32_t *indices;
};
struct Sphere {
    bool flip_normals = false;
    float radius;
    util::Float3 center{};
};
struct Hair {
    uint32_t segments_num;
    uint32_t point_num;
    uint32_t strands_num;
    uint32_t flags;  // bits 0-1: 0 linear, 1 quadratic B-spline, 2 cubic B-spline, 3 Catmull-Rom; bit 2: tapered
    float *positions;
    float *widths;
    uint32_t *segments_index;
    uint32_t *strands_index;
};
struct Shape {
    uint32_t id;
    std::string file_path;
    EShapeType type = EShapeType::_unknown;
    union {
        Mesh mesh;
        Sphere sphere{};
        Hair hair;
    };
};
struct ShapeInstance {
    std::string name = "";
    Shape *shape = nullptr;
    Material mat{};
    bool is_emitter = false;
    Emitter emitter{};
    util::Transform transform{};
};
}  // namespace Pupil::resource
