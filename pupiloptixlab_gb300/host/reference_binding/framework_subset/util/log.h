// Declaration subset of framework/util/log.h:12-59: Log::Error/Warn/Info with a
// format string.  Outside the tree the message is written to stderr as is.
#pragma once
#include <cstdio>
#include <string_view>

namespace Pupil {
struct Log {
    template<typename... Args>
    static void Error(std::string_view fmt, Args &&...) noexcept { std::fprintf(stderr, "[error] %.*s\n", (int)fmt.size(), fmt.data()); }
    template<typename... Args>
    static void Warn(std::string_view fmt, Args &&...) noexcept { std::fprintf(stderr, "[warn] %.*s\n", (int)fmt.size(), fmt.data()); }
    template<typename... Args>
    static void Info(std::string_view fmt, Args &&...) noexcept { std::fprintf(stderr, "[info] %.*s\n", (int)fmt.size(), fmt.data()); }
};
}  // namespace Pupil
