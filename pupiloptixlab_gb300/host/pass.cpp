// pass.cpp -- headless Pass / System / WavefrontPTPass (see pass.h).
#include "pass.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

namespace Pupil {

namespace {
std::string pt_error() {
    char buf[1024];
    pt_last_error(buf, sizeof(buf));
    return buf;
}
}  // namespace

Pass::Pass(std::string_view n, EPassTag t) noexcept : name(n), tag(t) {}

void Pass::Run() noexcept {
    if (!m_enable) return;
    auto t0 = std::chrono::steady_clock::now();
    OnRun();
    last_exec_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

BufferManager::Buffer *BufferManager::AllocBuffer(const std::string &name, size_t bytes) {
    auto &slot = m_buffers[name];
    if (slot && slot->bytes >= bytes) {
        cudaMemset(slot->device, 0, slot->bytes);
        return slot.get();
    }
    const bool is_new = !slot;
    if (slot && slot->device) cudaFree(slot->device);
    slot = std::make_unique<Buffer>();
    slot->name = name;
    if (cudaMalloc(&slot->device, bytes) != cudaSuccess) {
        slot.reset();
        m_buffers.erase(name);
        if (!is_new) m_names.erase(std::find(m_names.begin(), m_names.end(), name));
        return nullptr;
    }
    if (is_new) m_names.push_back(name);
    slot->bytes = bytes;
    cudaMemset(slot->device, 0, bytes);
    return slot.get();
}

BufferManager::Buffer *BufferManager::AllocBuffer(const BufferDesc &desc) {
    if (!desc.name) return nullptr;
    return AllocBuffer(std::string(desc.name), (size_t)desc.width * desc.height * desc.stride_in_byte);
}

BufferManager::Buffer *BufferManager::GetBuffer(const std::string &name) {
    auto it = m_buffers.find(name);
    return it == m_buffers.end() ? nullptr : it->second.get();
}

void BufferManager::Destroy() {
    for (auto &kv : m_buffers)
        if (kv.second && kv.second->device) cudaFree(kv.second->device);
    m_buffers.clear();
    m_names.clear();
}

System *System::Instance() {
    static System s;
    return &s;
}

bool System::Init(int device) {
    if (m_ctx) return true;
    pt_device_opts o{device, 0};
    if (pt_context_create(&o, &m_ctx) != PT_OK) {
        m_error = pt_error();
        return false;
    }
    return true;
}

void System::AddPass(Pass *pass) {
    if (static_cast<unsigned>(pass->tag) & static_cast<unsigned>(EPassTag::Pre)) m_pre_passes.push_back(pass);
    else m_passes.push_back(pass);
}

bool System::SetScene(const std::string &xml_path) {
    auto s = std::make_unique<resource::Scene>();
    if (!s->LoadFromXML(xml_path)) {
        m_error = s->error();
        return false;
    }
    return SetScene(std::move(s));
}

// System::SetScene (framework/system/system.cpp:136-173): allocate the
// "final result" buffer, then the SceneLoad event reaches every pass.
bool System::SetScene(std::unique_ptr<resource::Scene> scene) {
    if (!m_ctx && !Init()) return false;
    m_scene = std::move(scene);
    size_t px = (size_t)m_scene->sensor.width * m_scene->sensor.height;
    if (!m_buffers.AllocBuffer("final result", px * 16)) {
        m_error = "cannot allocate the final result buffer";
        return false;
    }
    for (Pass *p : m_pre_passes) p->Run();
    SceneLoadEvent ev{m_scene.get(), m_ctx, &m_buffers};
    EventDispatcher<ESystemEvent::SceneLoad>(&ev);
    for (Pass *p : m_passes)
        if (auto *pt = dynamic_cast<pt::WavefrontPTPass *>(p); pt && pt->last_status() != PT_OK) {
            m_error = pt->last_error();
            return false;
        }
    return true;
}

void System::SetCamera(const pt_camera_desc &camera) {
    pt_camera_desc c = camera;
    EventDispatcher<EWorldEvent::CameraChange>(&c);
}

void System::UpdateInstances(const float *positions, bool on_device, bool rebuild) {
    InstanceUpdateEvent ev{positions, on_device ? 1 : 0, rebuild};
    EventDispatcher<EWorldEvent::RenderInstanceUpdate>(&ev);
}

void System::Run(uint32_t frames) {
    if (!render_flag) return;
    for (uint32_t f = 0; f < frames; f++)
        for (Pass *p : m_passes) p->Run();
}

void System::Destroy() {
    for (Pass *p : m_passes)
        if (auto *pt = dynamic_cast<pt::WavefrontPTPass *>(p)) pt->ReleaseScene();
    m_passes.clear();
    m_pre_passes.clear();
    m_buffers.Destroy();
    m_scene.reset();
    if (m_ctx) pt_context_destroy(m_ctx);
    m_ctx = nullptr;
}

namespace pt {

// The events PTPass subscribes to (pt_pass.cpp:242-254).
WavefrontPTPass::WavefrontPTPass(std::string_view n) noexcept : Pass(n) {
    m_params.spp = 1;
    m_params.accumulate = 1;
    m_params.rng = PT_RNG_REF_LCG;
    m_ev_scene = EventBinder<ESystemEvent::SceneLoad>([this](void *p) {
        auto *e = static_cast<SceneLoadEvent *>(p);
        SetScene(e->scene, e->ctx, *e->buffers);
    });
    m_ev_camera = EventBinder<EWorldEvent::CameraChange>([this](void *p) {
        if (p) SetCamera(*static_cast<const pt_camera_desc *>(p));
        else m_dirty = true;
    });
    m_ev_update = EventBinder<EWorldEvent::RenderInstanceUpdate>([this](void *p) {
        if (p) UpdateInstances(*static_cast<const InstanceUpdateEvent *>(p));
        else m_dirty = true;
    });
}

WavefrontPTPass::~WavefrontPTPass() noexcept {
    EventUnbind<ESystemEvent::SceneLoad>(m_ev_scene);
    EventUnbind<EWorldEvent::CameraChange>(m_ev_camera);
    EventUnbind<EWorldEvent::RenderInstanceUpdate>(m_ev_update);
    ReleaseScene();
}

void WavefrontPTPass::ReleaseScene() noexcept {
    if (m_scene) pt_scene_destroy(m_scene);
    m_scene = nullptr;
    m_fb = pt_frame_buffers{};
}

bool WavefrontPTPass::SetScene(resource::Scene *scene, pt_context *ctx, BufferManager &buffers) noexcept {
    if (m_scene) pt_scene_destroy(m_scene);
    m_scene = nullptr;
    m_status = PT_OK;
    const pt_scene_desc &d = scene->Desc();
    if ((m_status = pt_scene_upload(ctx, &d, &m_scene)) != PT_OK ||
        (m_status = pt_bvh_build(m_scene, &m_bvh, nullptr)) != PT_OK) {
        m_error = pt_error();
        return false;
    }
    size_t px = (size_t)d.width * d.height;
    auto *accum = buffers.AllocBuffer("pt accum buffer", px * 16);
    auto *albedo = buffers.AllocBuffer("albedo", px * 12);
    auto *normal = buffers.AllocBuffer("normal", px * 12);
    auto *test = buffers.AllocBuffer("test", px * 4);
    auto *final_result = buffers.GetBuffer("final result");
    if (!accum || !albedo || !normal || !test || !final_result) {
        m_status = PT_ERR_OOM;
        m_error = "cannot allocate the pass buffers";
        return false;
    }
    m_fb.accum = static_cast<float *>(accum->device);
    m_fb.frame = static_cast<float *>(final_result->device);
    m_fb.albedo = static_cast<float *>(albedo->device);
    m_fb.normal = static_cast<float *>(normal->device);
    m_fb.test = static_cast<float *>(test->device);
    m_params.max_depth = d.max_depth;
    m_camera = d.camera;
    m_width = d.width;
    m_height = d.height;
    m_dirty = true;
    return true;
}

bool WavefrontPTPass::UpdateInstances(const InstanceUpdateEvent &e) noexcept {
    if (!m_scene) return false;
    m_status = pt_scene_update_all_vertices(m_scene, e.positions, e.on_device, nullptr);
    if (m_status == PT_OK) {
        if (e.rebuild) {
            pt_bvh_opts o = m_bvh;
            o.flags |= 1u;  // PT_BVH_FAST_BUILD: the per-frame rebuild
            m_status = pt_bvh_build(m_scene, &o, nullptr);
        } else {
            m_status = pt_bvh_refit(m_scene, nullptr);
        }
    }
    if (m_status != PT_OK) {
        m_error = pt_error();
        return false;
    }
    m_dirty = true;
    return true;
}

namespace {
constexpr char kProgressMagic[8] = {'P', 'T', 'P', 'R', 'O', 'G', '1', 0};
struct ProgressHeader {
    char magic[8];
    uint32_t width, height, sample_cnt, seed, max_depth, rng, accumulate, reserved;
    pt_camera_desc camera;
};
}  // namespace

bool WavefrontPTPass::SaveProgress(const std::string &path) noexcept {
    if (!m_scene || !m_fb.accum) {
        m_error = "SaveProgress: no scene";
        return false;
    }
    ProgressHeader h{};
    std::memcpy(h.magic, kProgressMagic, 8);
    h.width = m_width;
    h.height = m_height;
    h.sample_cnt = m_dirty ? 0 : m_params.sample_cnt;
    h.seed = m_dirty ? 0 : m_params.seed;
    h.max_depth = m_params.max_depth;
    h.rng = m_params.rng;
    h.accumulate = m_accumulate ? 1 : 0;
    h.camera = m_camera;
    std::vector<float> accum(4ull * m_width * m_height);
    if (cudaMemcpy(accum.data(), m_fb.accum, accum.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
        m_error = "SaveProgress: reading the accumulation buffer failed";
        return false;
    }
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        m_error = "SaveProgress: cannot write " + path;
        return false;
    }
    const bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(accum.data(), 4, accum.size(), f) == accum.size();
    fclose(f);
    if (!ok) m_error = "SaveProgress: write failed";
    return ok;
}

bool WavefrontPTPass::LoadProgress(const std::string &path) noexcept {
    if (!m_scene || !m_fb.accum) {
        m_error = "LoadProgress: no scene";
        return false;
    }
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) {
        m_error = "LoadProgress: cannot read " + path;
        return false;
    }
    ProgressHeader h{};
    std::vector<float> accum;
    bool ok = fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kProgressMagic, 8) == 0;
    if (ok && (h.width != m_width || h.height != m_height)) {
        fclose(f);
        m_error = "LoadProgress: the saved image is " + std::to_string(h.width) + "x" + std::to_string(h.height) +
                  ", the scene's film " + std::to_string(m_width) + "x" + std::to_string(m_height);
        return false;
    }
    if (ok) {
        accum.resize(4ull * h.width * h.height);
        ok = fread(accum.data(), 4, accum.size(), f) == accum.size();
    }
    fclose(f);
    if (!ok) {
        m_error = "LoadProgress: " + path + " is not a progress file of this pass";
        return false;
    }
    if (cudaMemcpy(m_fb.accum, accum.data(), accum.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        m_error = "LoadProgress: writing the accumulation buffer failed";
        return false;
    }
    m_camera = h.camera;
    pt_scene_set_camera(m_scene, &m_camera);
    m_params.sample_cnt = h.sample_cnt;
    m_params.seed = h.seed;
    m_params.max_depth = h.max_depth;
    m_params.rng = h.rng;
    m_accumulate = h.accumulate != 0;
    m_params.accumulate = h.accumulate;
    m_dirty = false;  // continue the saved sequence
    return true;
}

void WavefrontPTPass::SetCamera(const pt_camera_desc &camera) noexcept {
    m_camera = camera;
    m_dirty = true;
}
void WavefrontPTPass::SetMaxDepth(uint32_t depth) noexcept {
    m_params.max_depth = depth;
    m_dirty = true;
}
void WavefrontPTPass::SetAccumulate(bool on) noexcept {
    m_accumulate = on;
    m_dirty = true;
}

// PTPass::OnRun (example/path_tracer/pt_pass.cpp:39-57)
void WavefrontPTPass::OnRun() noexcept {
    if (!m_scene) return;
    if (m_dirty) {
        pt_scene_set_camera(m_scene, &m_camera);
        m_params.accumulate = m_accumulate ? 1 : 0;
        m_params.sample_cnt = 0;
        m_params.seed = 0;
        m_dirty = false;
    }
    m_status = pt_render(m_scene, &m_params, &m_fb, nullptr);
    if (m_status != PT_OK) {
        m_error = pt_error();
        return;
    }
    m_params.sample_cnt += m_params.accumulate;
    ++m_params.seed;
}

void WavefrontPTPass::Inspector() noexcept {
    // The reference draws max depth / accumulate controls with ImGui
    // (pt_pass.cpp:256-268); headless, they are SetMaxDepth / SetAccumulate.
}

}  // namespace pt
}  // namespace Pupil
