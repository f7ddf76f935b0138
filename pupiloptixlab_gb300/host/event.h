// event.h -- the reference's event mechanism (framework/util/event.h:8-51):
// one list of callbacks per enum value, EventBinder subscribes,
// EventDispatcher calls them in subscription order with a void * payload.
// Unlike the reference, whose passes live as long as the program, a binding
// can be removed (EventUnbind with the token EventBinder returns), so that a
// pass that is destroyed leaves no callback behind.
#pragma once

#include <cstdint>
#include <functional>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

namespace Pupil {

template<typename ET, ET enum_v>
class Event {
public:
    static uint64_t Bind(std::function<void(void *)> &&op) {
        std::scoped_lock<std::mutex> lock(mutex());
        const uint64_t token = ++next();
        ops().emplace_back(token, std::move(op));
        return token;
    }
    static void Unbind(uint64_t token) {
        std::scoped_lock<std::mutex> lock(mutex());
        auto &v = ops();
        for (auto it = v.begin(); it != v.end(); ++it)
            if (it->first == token) {
                v.erase(it);
                return;
            }
    }
    static void Respond(void *p) {
        std::vector<std::pair<uint64_t, std::function<void(void *)>>> copy;
        {
            std::scoped_lock<std::mutex> lock(mutex());
            copy = ops();
        }
        for (auto &op : copy) op.second(p);
    }

private:
    static std::mutex &mutex() { static std::mutex m; return m; }
    static uint64_t &next() { static uint64_t n = 0; return n; }
    static std::vector<std::pair<uint64_t, std::function<void(void *)>>> &ops() {
        static std::vector<std::pair<uint64_t, std::function<void(void *)>>> v;
        return v;
    }
};

template<auto enum_v, typename Func>
inline uint64_t EventBinder(Func &&f) {
    return Event<decltype(enum_v), enum_v>::Bind(std::function<void(void *)>(std::forward<Func>(f)));
}
template<auto enum_v>
inline void EventUnbind(uint64_t token) {
    Event<decltype(enum_v), enum_v>::Unbind(token);
}
template<auto enum_v>
inline void EventDispatcher(void *p = nullptr) {
    Event<decltype(enum_v), enum_v>::Respond(p);
}

// framework/system/system.h:13-20 and framework/world/world.h:15-23
enum class ESystemEvent { Quit, Precompute, StartRendering, StopRendering, SceneLoad, FrameFinished };
enum class EWorldEvent {
    CameraChange, CameraMove, CameraFovChange, CameraViewChange, RenderInstanceTransform, RenderInstanceUpdate,
    RenderInstanceRemove
};

}  // namespace Pupil
