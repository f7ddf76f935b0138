// Declaration subset of framework/world/camera.h:10-40: the camera helper
// whose GetCudaMemory() returns the device copy of optix::Camera
// {sample_to_camera, camera_to_world} (framework/render/camera.h:7-10),
// refreshed when the camera changed.
#pragma once

namespace Pupil::world {
class CameraHelper {
public:
    unsigned long long GetCudaMemory() noexcept { return m_camera_cuda_memory; }
    unsigned long long m_camera_cuda_memory = 0;  // set by the owner outside the tree
};
}  // namespace Pupil::world
