// wavefront_pass.cpp -- see the header.
#include "wavefront_pass.h"

#include "system/buffer.h"
#include "system/system.h"
#include "to_pt_scene_desc.h"
#include "util/event.h"
#include "util/log.h"
#include "world/camera.h"

namespace Pupil::pt {

WavefrontPTPass::WavefrontPTPass(std::string_view name) noexcept : Pass(name) {
    pt_device_opts o{};
    o.device = 0;
    if ((m_status = pt_context_create(&o, &m_ctx)) != PT_OK) Fail("pt_context_create");
    cudaStreamCreateWithFlags(&m_stream, cudaStreamNonBlocking);
    // the events PTPass subscribes to (pt_pass.cpp:242-254)
    EventBinder<EWorldEvent::CameraChange>([this](void *) { m_dirty = true; });
    EventBinder<EWorldEvent::RenderInstanceUpdate>([this](void *) { m_dirty = true; });
    EventBinder<ESystemEvent::SceneLoad>([this](void *p) { SetScene(static_cast<world::World *>(p)); });
}

WavefrontPTPass::~WavefrontPTPass() noexcept {
    if (m_scene) pt_scene_destroy(m_scene);
    if (m_ctx) pt_context_destroy(m_ctx);
    if (m_stream) cudaStreamDestroy(m_stream);
}

void WavefrontPTPass::Fail(const char *where) noexcept {
    char msg[512];
    pt_last_error(msg, sizeof(msg));
    Log::Error("{}: {}", where, msg);
}

void WavefrontPTPass::SetScene(world::World *world) noexcept {
    m_world = world;
    if (m_scene) {
        pt_scene_destroy(m_scene);
        m_scene = nullptr;
    }
    pt_camera_desc cam{};
    cudaMemcpy(&cam, reinterpret_cast<const void *>(world->camera->GetCudaMemory()), sizeof(cam),
               cudaMemcpyDeviceToHost);
    PtSceneDesc d;
    std::string error;
    if (!ToPtSceneDesc(*world->scene, cam, d, &error)) {
        Log::Error("ToPtSceneDesc: {}", error.c_str());
        m_status = PT_ERR_INVALID;
        return;
    }
    if ((m_status = pt_scene_upload(m_ctx, &d.desc, &m_scene)) != PT_OK) return Fail("pt_scene_upload");
    pt_bvh_opts b{};
    b.width = 4;
    b.max_leaf_size = 4;
    if ((m_status = pt_bvh_build(m_scene, &b, m_stream)) != PT_OK) return Fail("pt_bvh_build");

    // the named buffers PTPass uses: "final result" comes from System::SetScene,
    // the pass allocates its accumulation and AOV buffers (pt_pass.cpp:144-170)
    auto buf_mngr = util::Singleton<BufferManager>::instance();
    const uint32_t w = (uint32_t)world->scene->sensor.film.w, h = (uint32_t)world->scene->sensor.film.h;
    auto get_or_alloc = [&](const char *name, uint32_t stride) {
        Buffer *b = buf_mngr->GetBuffer(name);
        return b ? b : buf_mngr->AllocBuffer(BufferDesc{name, EBufferFlag::None, w, h, stride});
    };
    Buffer *frame = get_or_alloc(BufferManager::DEFAULT_FINAL_RESULT_BUFFER_NAME.data(), sizeof(float) * 4);
    Buffer *accum = get_or_alloc("pt accum buffer", sizeof(float) * 4);
    Buffer *albedo = get_or_alloc("albedo", sizeof(float) * 3);
    Buffer *normal = get_or_alloc("normal", sizeof(float) * 3);
    Buffer *test = get_or_alloc("test", sizeof(float));
    if (!frame || !accum || !albedo || !normal || !test) {
        Log::Error("buffer allocation failed");
        m_status = PT_ERR_OOM;
        return;
    }
    m_fb.accum = reinterpret_cast<float *>(accum->cuda_ptr);
    m_fb.frame = reinterpret_cast<float *>(frame->cuda_ptr);
    m_fb.albedo = reinterpret_cast<float *>(albedo->cuda_ptr);
    m_fb.normal = reinterpret_cast<float *>(normal->cuda_ptr);
    m_fb.test = reinterpret_cast<float *>(test->cuda_ptr);
    m_params = pt_render_params{};
    m_params.spp = 1;  // one frame per OnRun, as the OptiX launch
    m_params.max_depth = (uint32_t)world->scene->integrator.max_depth;
    m_params.accumulate = 1;
    m_params.rng = PT_RNG_REF_LCG;
    m_dirty = true;
}

void WavefrontPTPass::OnRun() noexcept {
    if (!m_scene) return;
    if (m_dirty) {  // camera or instances changed: restart accumulation (pt_pass.cpp:40-49)
        pt_camera_desc cam{};
        cudaMemcpy(&cam, reinterpret_cast<const void *>(m_world->camera->GetCudaMemory()), sizeof(cam),
                   cudaMemcpyDeviceToHost);
        pt_scene_set_camera(m_scene, &cam);
        m_params.sample_cnt = 0;
        m_params.seed = 0;
        m_dirty = false;
    }
    if ((m_status = pt_render(m_scene, &m_params, &m_fb, m_stream)) != PT_OK) return Fail("pt_render");
    cudaStreamSynchronize(m_stream);
    m_params.sample_cnt += m_params.accumulate;  // pt_pass.cpp:55-56
    ++m_params.seed;
}

void WavefrontPTPass::Inspector() noexcept { Pass::Inspector(); }

}  // namespace Pupil::pt
