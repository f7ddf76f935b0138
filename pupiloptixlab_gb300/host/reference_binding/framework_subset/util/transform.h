// Declaration subset of framework/util/transform.h:6-26: the instance /
// texture transform, a row-major Mat4 with the translation in the last column.
#pragma once
#include "type.h"

namespace Pupil::util {
struct Transform {
    Mat4 matrix;
    Transform() noexcept : matrix(1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f) {}
    Transform(const Mat4 &m) noexcept : matrix(m) {}
};
}  // namespace Pupil::util
