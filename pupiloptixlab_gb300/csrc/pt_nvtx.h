// pt_nvtx.h -- NVTX ranges around the host-side stages of a render, a BVH
// build and a denoiser step, so that a profiler timeline (Nsight Systems)
// groups the kernels each stage launches.  Without a profiler attached an
// NVTX call returns at once.  Ranges enclose the enqueueing of work; for a
// render replayed from a CUDA graph they enclose the capture and the launch.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace pt_nvtx {
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};
}  // namespace pt_nvtx
