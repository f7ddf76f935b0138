// Declaration subset of framework/util/event.h:8-51: per-enum-value event
// lists, EventBinder (subscribe) and EventDispatcher (respond).
#pragma once
#include <functional>
#include <mutex>
#include <type_traits>
#include <vector>

namespace Pupil {
template<typename ET, ET enum_v>
class Event {
public:
    static void Bind(std::function<void(void *)> &&op) noexcept {
        std::scoped_lock<std::mutex> lock(mutex());
        ops().push_back(std::move(op));
    }
    static void Respond(void *p = nullptr) noexcept {
        for (auto &&op : ops()) op(p);
    }

private:
    static std::mutex &mutex() { static std::mutex m; return m; }
    static std::vector<std::function<void(void *)>> &ops() { static std::vector<std::function<void(void *)>> v; return v; }
};

template<auto enum_v, typename Func>
inline void EventBinder(Func &&f) { Event<decltype(enum_v), enum_v>::Bind(std::forward<Func>(f)); }

template<auto enum_v>
inline void EventDispatcher(void *p = nullptr) { Event<decltype(enum_v), enum_v>::Respond(p); }
}  // namespace Pupil
