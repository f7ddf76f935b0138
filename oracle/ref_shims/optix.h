// Host stand-in for <optix.h>, used only by oracle/ref_kat.cpp to compile the
// reference's render-layer headers (BSDFs, Fresnel, GGX, emitters, sampling
// utilities) for the CPU.  It supplies the standard headers those files get
// transitively from the OptiX SDK and brings the float overloads of the math
// functions into the global namespace, as CUDA's device math does; without
// `using std::abs`, host abs(float) would bind to C's int abs(int).
#pragma once
#include <cstdint>
#include <cmath>
#include <algorithm>
using std::abs;
using std::acos;
using std::atan2;
using std::cos;
using std::max;
using std::min;
using std::sin;
using std::sqrt;

// The trigonometric functions the reference's render layer calls (sin, cos,
// sinf, cosf, atan2, acos, all unqualified inside namespace Pupil::optix) are
// bound to the library's deterministic ones, so that these known-answer
// vectors pin every other step of the reference's arithmetic bit for bit
// while the GPU kernels and the oracle use the same trigonometry.  Unqualified
// lookup inside Pupil::optix finds these before the global overloads.
#include "pt_trig.h"
namespace Pupil::optix {
inline float sin(float x) { return pt_sinf(x); }
inline float cos(float x) { return pt_cosf(x); }
inline float sinf(float x) { return pt_sinf(x); }
inline float cosf(float x) { return pt_cosf(x); }
inline float atan2(float y, float x) { return pt_atan2f(y, x); }
inline float acos(float x) { return pt_acosf(x); }
}  // namespace Pupil::optix
