// Declaration subset of PupilOptixLab framework/util/util.h:10-23 (the
// Singleton template) for compiling the reference-side binding outside the
// PupilOptixLab tree.  In the tree, the real header is used instead.
#pragma once
#include <memory>

namespace Pupil::util {
template<typename T>
class Singleton {
public:
    static T *instance() {
        static const std::unique_ptr<T> inst = std::make_unique<T>();
        return inst.get();
    }
    Singleton(const Singleton &) = delete;
    Singleton &operator=(const Singleton) = delete;

protected:
    Singleton() {}
};
}  // namespace Pupil::util
