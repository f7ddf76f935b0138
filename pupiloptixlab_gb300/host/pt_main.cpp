// pt_main.cpp -- headless counterpart of example/path_tracer/main.cpp: load a
// mitsuba-style scene, run the WavefrontPTPass for N frames, write the frame
// as PFM or (by the .exr extension) uncompressed OpenEXR.
//   pupil_pt <scene.xml> <out.pfm|out.exr> [frames=64] [rng: lcg|pcg32]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pass.h"

extern "C" int pupil_write_pfm(const char *path, const float *rgba, uint32_t w, uint32_t h);
extern "C" int pupil_write_exr(const char *path, const float *rgba, uint32_t w, uint32_t h);

static int usage(const char *prog) {
    fprintf(stderr, "usage: %s <scene.xml> <out.pfm|out.exr> [frames >= 1] [lcg|pcg32]\n", prog);
    return 2;
}

int main(int argc, char **argv) {
    if (argc < 3 || argc > 5) return usage(argv[0]);
    uint32_t frames = 64;
    if (argc > 3) {
        char *end = nullptr;
        const unsigned long v = strtoul(argv[3], &end, 10);
        if (end == argv[3] || *end != '\0' || argv[3][0] == '-' || v == 0 || v > 0xffffffffUL) return usage(argv[0]);
        frames = (uint32_t)v;
    }
    uint32_t rng = PT_RNG_REF_LCG;
    if (argc > 4) {
        const std::string r = argv[4];
        if (r == "pcg32") rng = PT_RNG_PCG32;
        else if (r != "lcg") return usage(argv[0]);
    }
    Pupil::System *sys = Pupil::System::Instance();
    if (!sys->Init(0)) {
        fprintf(stderr, "%s\n", sys->error().c_str());
        return 1;
    }
    Pupil::pt::WavefrontPTPass pass;
    pass.SetRng(rng);
    sys->AddPass(&pass);
    if (!sys->SetScene(std::string(argv[1]))) {
        fprintf(stderr, "%s\n", sys->error().c_str());
        return 1;
    }
    sys->Run(frames);
    if (pass.last_status() != PT_OK) {
        fprintf(stderr, "render failed: %s\n", pass.last_error().c_str());
        return 1;
    }
    uint32_t w = sys->scene()->sensor.width, h = sys->scene()->sensor.height;
    std::vector<float> img((size_t)w * h * 4);
    if (cudaMemcpy(img.data(), sys->buffers().GetBuffer("final result")->device, img.size() * 4,
                   cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "cannot read the frame back from the device\n");
        return 1;
    }
    const std::string out = argv[2];
    int st;
    if (out.size() > 4 && out.compare(out.size() - 4, 4, ".exr") == 0) {
        // the frame's row 0 is the bottom of the image (PFM order); EXR stores the top first
        std::vector<float> top((size_t)w * h * 4);
        for (uint32_t y = 0; y < h; y++)
            memcpy(&top[(size_t)y * w * 4], &img[(size_t)(h - 1 - y) * w * 4], (size_t)w * 4 * sizeof(float));
        st = pupil_write_exr(argv[2], top.data(), w, h);
    } else {
        st = pupil_write_pfm(argv[2], img.data(), w, h);
    }
    if (st != PT_OK) {
        fprintf(stderr, "cannot write %s\n", argv[2]);
        return 1;
    }
    printf("%s: %ux%u, %u frames, last frame %.2f ms\n", argv[2], w, h, frames, pass.last_exec_ms);
    sys->Destroy();
    return 0;
}
