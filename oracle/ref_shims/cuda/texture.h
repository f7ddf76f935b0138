// Host stand-in for framework/cuda/texture.h, used only by oracle/ref_kat.cpp.
// The reference header pulls in DirectXMath (util/type.h) and the device-only
// tex2D; the BSDF and emitter code only needs a texture whose Sample(uv)
// returns a colour, so this keeps a constant RGB value.
#pragma once
#include "cuda/preprocessor.h"
#include "cuda/vec_math.h"

namespace Pupil::cuda {
struct Texture {
    float3 rgb;
    float3 Sample(float2) const noexcept { return rgb; }
};
}// namespace Pupil::cuda
