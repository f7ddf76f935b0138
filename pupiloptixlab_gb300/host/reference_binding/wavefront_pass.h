// wavefront_pass.h -- the reference-side pass a PupilOptixLab maintainer adds
// in place of pt::PTPass (example/path_tracer/pt_pass.h:21-41): same events,
// same named buffers, same one-frame-per-OnRun accumulation, with the OptiX
// pipeline replaced by this library's C-ABI (include/pt_api.h).
//
// It compiles inside the PupilOptixLab tree against its framework headers, or
// here against framework_subset/ (tests/test_reference_binding_cpu.py; the
// GPU test runs it end to end).
#pragma once

#include <atomic>
#include <string_view>

#include <cuda_runtime.h>

#include "pt_api.h"
#include "system/pass.h"
#include "world/world.h"

namespace Pupil::pt {

class WavefrontPTPass : public Pass {
public:
    WavefrontPTPass(std::string_view name = "Path Tracing (GB300)") noexcept;
    ~WavefrontPTPass() noexcept override;
    void OnRun() noexcept override;      // replaces PTPass::OnRun (pt_pass.cpp:39-57)
    void Inspector() noexcept override;  // the reference draws ImGui here; nothing to draw headless
    void SetScene(world::World *world) noexcept;  // replaces PTPass::SetScene (pt_pass.cpp:127-240)

    int last_status() const noexcept { return m_status; }
    unsigned sample_count() const noexcept { return m_params.sample_cnt; }

private:
    void Fail(const char *where) noexcept;

    pt_context *m_ctx = nullptr;
    pt_scene *m_scene = nullptr;
    world::World *m_world = nullptr;
    pt_render_params m_params{};
    pt_frame_buffers m_fb{};
    cudaStream_t m_stream = nullptr;
    std::atomic_bool m_dirty = true;
    int m_status = PT_OK;
};

}  // namespace Pupil::pt
