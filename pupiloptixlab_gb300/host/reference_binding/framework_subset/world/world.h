// Declaration subset of framework/world/world.h:15-66: world events and the
// World singleton's scene and camera helper.
#pragma once
#include <memory>
#include "resource/scene.h"
#include "util/util.h"
#include "camera.h"

namespace Pupil {
enum class EWorldEvent {
    CameraChange, CameraMove, CameraFovChange, CameraViewChange, RenderInstanceTransform, RenderInstanceUpdate,
    RenderInstanceRemove
};
namespace world {
class World : public util::Singleton<World> {
public:
    std::unique_ptr<resource::Scene> scene = nullptr;
    std::unique_ptr<CameraHelper> camera = nullptr;
};
}  // namespace world
}  // namespace Pupil
