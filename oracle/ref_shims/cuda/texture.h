// Host stand-in for framework/cuda/texture.h, used only by oracle/ref_kat.cpp.
// The reference header pulls in DirectXMath (util/type.h) and the device-only
// tex2D; the BSDF and emitter code only needs a texture whose Sample(uv)
// returns a colour: a constant RGB value, or a bitmap fetched with the CPU
// restatement of a float4 texture fetch (oracle/tex_fetch.h).
#pragma once
#include "cuda/preprocessor.h"
#include "cuda/vec_math.h"
#include "../../tex_fetch.h"

namespace Pupil::cuda {
struct Texture {
    float3 rgb;
    const float *pixels = nullptr;
    unsigned w = 0, h = 0, address = 0, filter = 1;
    float3 Sample(float2 uv) const noexcept {
        if (!pixels) return rgb;
        texfetch::Float4 c = texfetch::fetch(pixels, w, h, address, filter, uv.x, uv.y);
        return make_float3(c.x, c.y, c.z);
    }
};
}// namespace Pupil::cuda
