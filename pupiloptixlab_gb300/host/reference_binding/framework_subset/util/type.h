// Declaration subset of framework/util/type.h:7-112 without DirectXMath:
// Float3, Float4 and the row-major Mat4 (as e[16] and re[4][4]).
#pragma once

namespace Pupil::util {
struct Float3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        float e[3];
    };
    constexpr Float3(float v = 0.f) noexcept : x(v), y(v), z(v) {}
    constexpr Float3(float x_, float y_, float z_) noexcept : x(x_), y(y_), z(z_) {}
};
struct Float4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        float e[4];
    };
    constexpr Float4(float v = 0.f) noexcept : x(v), y(v), z(v), w(v) {}
    constexpr Float4(float x_, float y_, float z_, float w_) noexcept : x(x_), y(y_), z(z_), w(w_) {}
};
// The reference's Mat4 also names its rows r0..r3 (Float4) and overlays a
// DirectX::XMMATRIX; the binding uses only e[] and re[][].
struct Mat4 {
    union {
        float e[16];
        float re[4][4];
    };
    constexpr Mat4() noexcept : e{} {}
    constexpr Mat4(float m00, float m01, float m02, float m03, float m10, float m11, float m12, float m13,
                   float m20, float m21, float m22, float m23, float m30, float m31, float m32, float m33) noexcept
        : e{m00, m01, m02, m03, m10, m11, m12, m13, m20, m21, m22, m23, m30, m31, m32, m33} {}
};
}  // namespace Pupil::util
