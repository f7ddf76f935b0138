// tex_fetch.h -- CPU restatement of a 2D texture fetch from a float4 CUDA
// texture object with normalized coordinates (TEST INFRASTRUCTURE: used by
// the oracle and by the reference-header shim, never by the library).
//
// Follows the texture-fetching rules of the CUDA C++ Programming Guide
// (appendix "Texture Fetching"):
//   addressing on normalized coordinates x in texel units x * N:
//     wrap   x - floor(x), mirror reflects every other period, clamp to [0, N);
//   point filtering: T[floor(x * N)];
//   linear filtering: x_B = x * N - 0.5, i = floor(x_B), a = frac(x_B) held
//     with 8 fractional bits, result (1-a)(1-b) T[i,j] + a(1-b) T[i+1,j]
//     + (1-a) b T[i,j+1] + a b T[i+1,j+1], the texel indices addressed per mode.
// The hardware's internal rounding of the filtered sum is not specified;
// results agree with the texture unit to within a few units in the last
// place of the weights (the tests compare with tolerances).
#pragma once

#include <cmath>
#include <cstdint>

namespace texfetch {

enum : uint32_t { kWrap = 0, kClamp = 1, kMirror = 2 };
enum : uint32_t { kPoint = 0, kLinear = 1 };

struct Float4 {
    float x, y, z, w;
};

// Texel index i of a dimension with n texels under the address mode.
inline int64_t address(int64_t i, int64_t n, uint32_t mode) {
    if (mode == kWrap) {
        int64_t r = i % n;
        return r < 0 ? r + n : r;
    }
    if (mode == kMirror) {
        const int64_t period = 2 * n;
        int64_t r = i % period;
        if (r < 0) r += period;
        return r < n ? r : period - 1 - r;
    }
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// Normalized coordinate -> texel-space coordinate under the address mode
// (wrap and mirror act on the normalized coordinate before scaling).
inline float coord(float x, uint32_t mode) {
    if (mode == kWrap) return x - std::floor(x);
    if (mode == kMirror) {
        const float f = std::floor(x);
        const float r = x - f;
        return (static_cast<int64_t>(f) & 1) ? 1.f - r : r;
    }
    return x;
}

inline Float4 texel(const float *px, uint32_t w, int64_t x, int64_t y) {
    const float *p = px + 4 * (static_cast<size_t>(y) * w + static_cast<size_t>(x));
    return {p[0], p[1], p[2], p[3]};
}

inline Float4 fetch(const float *px, uint32_t w, uint32_t h, uint32_t addr, uint32_t filter, float u, float v) {
    const float cu = coord(u, addr), cv = coord(v, addr);
    if (filter == kPoint) {
        const int64_t i = address(static_cast<int64_t>(std::floor(cu * w)), w, addr);
        const int64_t j = address(static_cast<int64_t>(std::floor(cv * h)), h, addr);
        return texel(px, w, i, j);
    }
    const float xb = cu * static_cast<float>(w) - 0.5f, yb = cv * static_cast<float>(h) - 0.5f;
    const float fx = std::floor(xb), fy = std::floor(yb);
    const float a = std::nearbyint((xb - fx) * 256.f) / 256.f;  // 8 fractional bits
    const float b = std::nearbyint((yb - fy) * 256.f) / 256.f;
    const int64_t i0 = address(static_cast<int64_t>(fx), w, addr), i1 = address(static_cast<int64_t>(fx) + 1, w, addr);
    const int64_t j0 = address(static_cast<int64_t>(fy), h, addr), j1 = address(static_cast<int64_t>(fy) + 1, h, addr);
    const Float4 t00 = texel(px, w, i0, j0), t10 = texel(px, w, i1, j0), t01 = texel(px, w, i0, j1),
                 t11 = texel(px, w, i1, j1);
    const float w00 = (1.f - a) * (1.f - b), w10 = a * (1.f - b), w01 = (1.f - a) * b, w11 = a * b;
    return {w00 * t00.x + w10 * t10.x + w01 * t01.x + w11 * t11.x, w00 * t00.y + w10 * t10.y + w01 * t01.y + w11 * t11.y,
            w00 * t00.z + w10 * t10.z + w01 * t01.z + w11 * t11.z, w00 * t00.w + w10 * t10.w + w01 * t01.w + w11 * t11.w};
}

}  // namespace texfetch
