// Minimal stand-in for fmt 5.3, used only to compile the reference's octree
// builder (test oracle): replaces each "{...}" field with the next argument.
#pragma once
#include <cstdio>
#include <sstream>
#include <string>
#include <string_view>
namespace fmt {
namespace detail {
inline void put(std::ostringstream& os, std::string_view f) { os << f; }
template <typename T, typename... Rest>
void put(std::ostringstream& os, std::string_view f, const T& v, const Rest&... rest) {
    size_t a = f.find('{');
    if (a == std::string_view::npos) { os << f; return; }
    size_t b = f.find('}', a);
    if (b == std::string_view::npos) { os << f; return; }
    os << f.substr(0, a) << v;
    put(os, f.substr(b + 1), rest...);
}
}
template <typename... Args>
std::string format(std::string_view f, const Args&... args) {
    std::ostringstream os;
    detail::put(os, f, args...);
    return os.str();
}
template <typename... Args>
void print(std::string_view f, const Args&... args) {
    std::string s = format(f, args...);
    std::fwrite(s.data(), 1, s.size(), stderr);
}
}
