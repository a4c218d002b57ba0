// Stand-in for the reference's core/Error.h (test oracle build only).
#pragma once
#include <stdexcept>
#include <string_view>
#include <fmt/format.h>
struct Error : public std::runtime_error {
    template <typename... Args>
    Error(std::string_view f, const Args&... args) : std::runtime_error(fmt::format(f, args...)) {}
};
