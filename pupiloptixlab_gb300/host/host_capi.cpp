// host_capi.cpp -- C entry points of the C++ host layer (libpupil_host.so),
// used by the tests and by non-C++ callers: load a mitsuba-style scene into
// the tracer's descriptor, and run the headless System with the
// WavefrontPTPass for a number of frames.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "pass.h"
#include "scene.h"
#include "image.h"

namespace {
thread_local std::string g_err;
int fail(const std::string &m, int st = PT_ERR_INVALID) {
    g_err = m;
    return st;
}
}  // namespace

extern "C" {

int pupil_host_last_error(char *buf, size_t n) {
    if (!buf || !n) return PT_ERR_INVALID;
    size_t k = std::min(n - 1, g_err.size());
    memcpy(buf, g_err.data(), k);
    buf[k] = 0;
    return PT_OK;
}

// Loads an XML file (or, with is_text != 0, XML text) into a scene handle.
int pupil_scene_load(const char *path_or_text, int is_text, void **out) {
    if (!path_or_text || !out) return fail("NULL argument");
    auto s = std::make_unique<Pupil::resource::Scene>();
    bool ok = is_text ? s->LoadFromString(path_or_text, "") : s->LoadFromXML(path_or_text);
    if (!ok) return fail(s->error());
    *out = s.release();
    return PT_OK;
}

const pt_scene_desc *pupil_scene_desc(void *scene) {
    return scene ? &static_cast<Pupil::resource::Scene *>(scene)->Desc() : nullptr;
}

void pupil_scene_free(void *scene) { delete static_cast<Pupil::resource::Scene *>(scene); }

// Headless System + WavefrontPTPass: load `xml`, run `frames` frames (1 spp
// each, as PTPass::OnRun) and copy the "final result" buffer (float4 per
// pixel) to out_rgba (host, width*height*4 floats, may be NULL).
int pupil_run_scene(const char *xml, int is_text, uint32_t frames, uint32_t rng, float *out_rgba, uint32_t *out_w,
                    uint32_t *out_h) {
    using namespace Pupil;
    auto scene = std::make_unique<resource::Scene>();
    if (!(is_text ? scene->LoadFromString(xml, "") : scene->LoadFromXML(xml))) return fail(scene->error());
    uint32_t w = scene->sensor.width, h = scene->sensor.height;
    System sys;
    if (!sys.Init(0)) return fail(sys.error(), PT_ERR_UNSUPPORTED);
    pt::WavefrontPTPass pass;
    pass.SetRng(rng);
    sys.AddPass(&pass);
    if (!sys.SetScene(std::move(scene))) {
        std::string e = sys.error();
        sys.Destroy();
        return fail(e, PT_ERR_CUDA);
    }
    sys.Run(frames);
    int st = pass.last_status();
    if (st != PT_OK) {
        std::string e = pass.last_error();
        sys.Destroy();
        return fail(e, st);
    }
    if (out_rgba) {
        auto *fr = sys.buffers().GetBuffer("final result");
        cudaMemcpy(out_rgba, fr->device, (size_t)w * h * 16, cudaMemcpyDeviceToHost);
    }
    if (out_w) *out_w = w;
    if (out_h) *out_h = h;
    sys.Destroy();
    return PT_OK;
}

// The same with the world changing in between, through the events the pass
// subscribes to: after `change_after` frames, `positions` (host, every mesh's
// object-space vertices in mesh order; may be NULL) arrive as
// EWorldEvent::RenderInstanceUpdate (refit) and `camera` (may be NULL) as
// EWorldEvent::CameraChange; both restart accumulation.  `resume_from` (may
// be NULL) loads a progress file right after the scene, `save_to` (may be
// NULL) saves one after the last frame.
int pupil_run_scene_ex(const char *xml, int is_text, uint32_t frames, uint32_t rng, const char *resume_from,
                       const char *save_to, uint32_t change_after, const float *positions,
                       const pt_camera_desc *camera, float *out_rgba, uint32_t *out_w, uint32_t *out_h) {
    using namespace Pupil;
    auto scene = std::make_unique<resource::Scene>();
    if (!(is_text ? scene->LoadFromString(xml, "") : scene->LoadFromXML(xml))) return fail(scene->error());
    uint32_t w = scene->sensor.width, h = scene->sensor.height;
    System sys;
    if (!sys.Init(0)) return fail(sys.error(), PT_ERR_UNSUPPORTED);
    pt::WavefrontPTPass pass;
    pass.SetRng(rng);
    sys.AddPass(&pass);
    auto bail = [&](const std::string &e, int st) {
        sys.Destroy();
        return fail(e, st);
    };
    if (!sys.SetScene(std::move(scene))) return bail(sys.error(), PT_ERR_CUDA);
    if (resume_from && !pass.LoadProgress(resume_from)) return bail(pass.last_error(), PT_ERR_INVALID);
    const bool change = positions || camera;
    for (uint32_t f = 0; f < frames; f++) {
        if (change && f == change_after) {
            if (positions) sys.UpdateInstances(positions, false);
            if (camera) sys.SetCamera(*camera);
        }
        sys.Run(1);
        if (pass.last_status() != PT_OK) return bail(pass.last_error(), pass.last_status());
    }
    if (pass.last_status() != PT_OK) return bail(pass.last_error(), pass.last_status());
    if (save_to && !pass.SaveProgress(save_to)) return bail(pass.last_error(), PT_ERR_INVALID);
    if (out_rgba) {
        auto *fr = sys.buffers().GetBuffer("final result");
        cudaMemcpy(out_rgba, fr->device, (size_t)w * h * 16, cudaMemcpyDeviceToHost);
    }
    if (out_w) *out_w = w;
    if (out_h) *out_h = h;
    sys.Destroy();
    return PT_OK;
}

// Portable float map (little endian, bottom row first: row 0 of the frame
// buffer is the bottom of the image, as in the reference's display path).
int pupil_write_pfm(const char *path, const float *rgba, uint32_t w, uint32_t h) {
    FILE *f = fopen(path, "wb");
    if (!f) return fail(std::string("cannot write ") + path);
    fprintf(f, "PF\n%u %u\n-1.0\n", w, h);
    for (size_t i = 0; i < (size_t)w * h; i++) fwrite(rgba + 4 * i, sizeof(float), 3, f);
    fclose(f);
    return PT_OK;
}

// Headless image save (the GUI's screenshot, framework/system/gui.cpp:475-482,
// writes EXR through tinyexr): uncompressed scanline OpenEXR, RGBA floats.
int pupil_write_exr(const char *path, const float *rgba, uint32_t w, uint32_t h) {
    std::string e;
    if (!path || !rgba || !w || !h) return fail("pupil_write_exr: bad arguments");
    if (!Pupil::util::SaveExrRGBA(path, rgba, w, h, e)) return fail(e);
    return PT_OK;
}

}  // extern "C"
