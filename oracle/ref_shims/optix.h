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
