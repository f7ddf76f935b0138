// Host stand-in for framework/cuda/random.h, used only by oracle/ref_kat.cpp.
// Same class, interface and algorithm (TEA-4 seeding, LCG A=1664525
// C=1013904223, 24-bit float), with one change: Next2() draws x before y.
// The reference writes make_float2(Next(), Next()), whose argument evaluation
// order C++ leaves unspecified (GCC on x86-64 evaluates right to left), so
// the host build would otherwise swap the two draws.
#pragma once
#include "cuda/preprocessor.h"
#include "cuda/vec_math.h"

namespace Pupil::cuda {
class Random {
private:
    unsigned int m_seed;

public:
    Random() noexcept : m_seed(0) {}
    void Init(unsigned int N, unsigned int val0, unsigned int val1) noexcept {
        unsigned int v0 = val0, v1 = val1, s0 = 0;
        for (unsigned int n = 0; n < N; n++) {
            s0 += 0x9e3779b9u;
            v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
            v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
        }
        m_seed = v0;
    }
    unsigned int GetSeed() const noexcept { return m_seed; }
    void SetSeed(unsigned int seed) noexcept { m_seed = seed; }
    float Next() noexcept {
        m_seed = 1664525u * m_seed + 1013904223u;
        return static_cast<float>(m_seed & 0x00FFFFFFu) / 0x01000000;
    }
    float2 Next2() noexcept {
        float x = Next();
        float y = Next();
        return make_float2(x, y);
    }
};
}// namespace Pupil::cuda
