// Declaration subset of framework/resource/scene.h:16-57: integrator, film,
// perspective sensor and the loaded scene (shape instances and emitters).
#pragma once
#include <vector>
#include "shape.h"
#include "emitter.h"

namespace Pupil::resource {
struct Integrator { int max_depth = 1; };
struct Film {
    int w = 768;
    int h = 576;
};
struct Sensor {
    float fov = 90.f;
    float near_clip = 0.01f;
    float far_clip = 10000.f;
    util::Transform transform{};
    Film film{};
};
class Scene {
public:
    Integrator integrator;
    Sensor sensor;
    std::vector<ShapeInstance> shape_instances;
    std::vector<Emitter> emitters;
};
}  // namespace Pupil::resource
