// Declaration subset of framework/system/pass.h:7-43: pass tags and the
// Pass base class (OnRun per frame, Inspector, enable switch).
#pragma once
#include <cstdint>
#include <string>
#include <string_view>

namespace Pupil {
enum class EPassTag : uint32_t { None = 0, Pre = 1 << 0, Post = 1 << 1, Asyn = 1 << 2 };

class Pass {
protected:
    double m_last_exec_time = 0.;
    bool m_enable = true;

public:
    const std::string name;
    const EPassTag tag;
    Pass(std::string_view name, EPassTag tag = EPassTag::None) noexcept : name(name), tag(tag) {}
    virtual ~Pass() noexcept = default;
    virtual void Run() noexcept { if (m_enable) OnRun(); }
    virtual void Inspector() noexcept {}
    virtual void OnRun() noexcept = 0;
    void Toggle() noexcept { m_enable ^= true; }
    void SetEnablility(bool enable) noexcept { m_enable = enable; }
    bool IsEnabled() const noexcept { return m_enable; }
};
}  // namespace Pupil
