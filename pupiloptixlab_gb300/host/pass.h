// pass.h -- headless mirror of PupilOptixLab's pass / system API over the
// tracer's C-ABI (include/pt_api.h).
//
//   Pupil::Pass              framework/system/pass.h:22-43 (name, OnRun, Inspector, timed Run)
//   Pupil::BufferManager     framework/system/buffer.h:44-63 (named device buffers)
//   Pupil::System            framework/system/system.h:22-41 (Init, AddPass, SetScene, Run, Destroy)
//   Pupil::pt::WavefrontPTPass  the drop-in for pt::PTPass (example/path_tracer/pt_pass.h:21-41):
//                            one frame (1 spp) per OnRun, sample count and seed advanced per
//                            frame, accumulation restarted when the camera or scene changes.
// There is no GUI thread: System::Run(frames) runs the passes on the calling thread.
#pragma once

#include <atomic>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <vector>

#include "event.h"
#include "pt_api.h"
#include "scene.h"

namespace Pupil {

enum class EPassTag : unsigned { None = 0, Pre = 1 << 0, Post = 1 << 1 };

class Pass {
public:
    Pass(std::string_view name, EPassTag tag = EPassTag::None) noexcept;
    virtual ~Pass() noexcept = default;
    virtual void OnRun() noexcept = 0;
    virtual void Inspector() noexcept {}
    void Run() noexcept;  // OnRun, timed, skipped while disabled (pass.cpp:6-13)

    // enable switch (pass.h:37-39; the reference's spelling of SetEnablility kept)
    void Toggle() noexcept { m_enable = !m_enable; }
    void SetEnablility(bool enable) noexcept { m_enable = enable; }
    bool IsEnabled() const noexcept { return m_enable; }

    const std::string name;
    const EPassTag tag;
    double last_exec_ms = 0.0;

protected:
    bool m_enable = true;
};

class BufferManager {
public:
    struct Buffer {
        std::string name;
        void *device = nullptr;
        size_t bytes = 0;
    };
    // BufferDesc (buffer.h:25-31): width * height * stride_in_byte bytes; the
    // flag (DX12 sharing) has no meaning without a display and is ignored
    struct BufferDesc {
        const char *name = nullptr;
        uint32_t flag = 0;
        uint32_t width = 1;
        uint32_t height = 1;
        uint32_t stride_in_byte = 1;
    };
    static constexpr std::string_view DEFAULT_FINAL_RESULT_BUFFER_NAME = "final result";

    Buffer *AllocBuffer(const std::string &name, size_t bytes);  // zero-filled; reused if big enough
    Buffer *AllocBuffer(const BufferDesc &desc);
    Buffer *GetBuffer(const std::string &name);
    const std::vector<std::string> &GetBufferNameList() const { return m_names; }  // in allocation order
    void Destroy();
    ~BufferManager() { Destroy(); }

private:
    std::map<std::string, std::unique_ptr<Buffer>> m_buffers;
    std::vector<std::string> m_names;
};

// Payloads of the events System dispatches.
struct SceneLoadEvent {  // ESystemEvent::SceneLoad (the reference passes its world::World *)
    resource::Scene *scene;
    pt_context *ctx;
    BufferManager *buffers;
};
struct InstanceUpdateEvent {  // EWorldEvent::RenderInstanceUpdate
    const float *positions;    // every mesh's object-space vertices, in mesh order (pt_scene_update_all_vertices)
    int on_device;             // positions in device memory
    bool rebuild;              // rebuild the BVH (PT_BVH_FAST_BUILD) instead of refitting it
};

class System {
public:
    // system.h:26-27: the render loop runs the passes only while render_flag
    // is set (the GUI's pause); quit_flag is kept for callers that poll it
    bool render_flag = true;
    bool quit_flag = false;

    static System *Instance();
    bool Init(int device = 0);
    void AddPass(Pass *pass);
    bool SetScene(const std::string &xml_path);
    // System::SetScene (system.cpp:136-173): the "final result" buffer, then
    // ESystemEvent::SceneLoad to every pass that subscribed
    bool SetScene(std::unique_ptr<resource::Scene> scene);
    // the world's camera moved (EWorldEvent::CameraChange, payload pt_camera_desc *)
    void SetCamera(const pt_camera_desc &camera);
    // instances changed (EWorldEvent::RenderInstanceUpdate; world.cpp:45-59)
    void UpdateInstances(const float *positions, bool on_device, bool rebuild = false);
    void Run(uint32_t frames);
    void Destroy();

    pt_context *context() const { return m_ctx; }
    resource::Scene *scene() const { return m_scene.get(); }
    BufferManager &buffers() { return m_buffers; }
    const std::string &error() const { return m_error; }

private:
    pt_context *m_ctx = nullptr;
    std::unique_ptr<resource::Scene> m_scene;
    std::vector<Pass *> m_passes, m_pre_passes;
    BufferManager m_buffers;
    std::string m_error;
};

namespace pt {

class WavefrontPTPass : public Pass {
public:
    explicit WavefrontPTPass(std::string_view name = "Path Tracing") noexcept;
    ~WavefrontPTPass() noexcept override;
    void OnRun() noexcept override;
    void Inspector() noexcept override;

    // SceneLoad event: upload the scene, build the BVH, allocate the pass buffers.
    bool SetScene(resource::Scene *scene, pt_context *ctx, BufferManager &buffers) noexcept;
    // RenderInstanceUpdate event: new vertices, refit or rebuild, restart accumulation.
    bool UpdateInstances(const InstanceUpdateEvent &e) noexcept;
    // Progressive resume (the reference keeps its accumulation only in device
    // memory): the accumulation buffer, sample count, seed, camera and render
    // settings to a file, and back into a pass whose scene has the same size;
    // the frames rendered after LoadProgress continue the saved sequence exactly.
    bool SaveProgress(const std::string &path) noexcept;
    bool LoadProgress(const std::string &path) noexcept;
    // CameraChange event: restart accumulation with the new camera.
    void SetCamera(const pt_camera_desc &camera) noexcept;
    void SetMaxDepth(uint32_t depth) noexcept;
    void SetAccumulate(bool on) noexcept;
    void SetRng(uint32_t mode) noexcept { m_params.rng = mode; }
    void SetBvhOptions(const pt_bvh_opts &opts) noexcept { m_bvh = opts; }
    // Frees the device scene (System::Destroy calls it before destroying the context).
    void ReleaseScene() noexcept;

    int last_status() const { return m_status; }
    const std::string &last_error() const { return m_error; }
    uint32_t sample_count() const { return m_params.sample_cnt; }
    pt_scene *handle() const { return m_scene; }

private:
    pt_scene *m_scene = nullptr;
    pt_render_params m_params{};
    pt_frame_buffers m_fb{};
    pt_bvh_opts m_bvh{4, 4, 0, 0};
    pt_camera_desc m_camera{};
    std::atomic_bool m_dirty{true};
    bool m_accumulate = true;
    int m_status = PT_OK;
    std::string m_error;
    uint32_t m_width = 0, m_height = 0;
    uint64_t m_ev_scene = 0, m_ev_camera = 0, m_ev_update = 0;  // event subscriptions
};

}  // namespace pt
}  // namespace Pupil
