// Minimal stand-in for fmt 5.3, used only to compile reference sources for the
// test oracle (the octree builder, the headless.conf parser): replaces each
// "{...}" field with the next argument, written with operator<<.
#pragma once
#include <cstdio>
#include <sstream>
#include <string>
#include <string_view>
#include <vector>
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
template <typename T>
std::string text(const T& v) {
    std::ostringstream os;
    os << v;
    return os.str();
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
// the arguments of a format call, each already written out
struct format_args {
    std::vector<std::string> items;
};
template <typename... Args>
format_args make_format_args(const Args&... args) {
    return format_args{{detail::text(args)...}};
}
struct memory_buffer {
    std::string data;
};
inline void vformat_to(memory_buffer& buf, std::string_view f, const format_args& args) {
    size_t next = 0;
    while (true) {
        size_t a = f.find('{');
        size_t b = a == std::string_view::npos ? a : f.find('}', a);
        if (b == std::string_view::npos) {
            buf.data.append(f);
            return;
        }
        buf.data.append(f.substr(0, a));
        if (next < args.items.size()) buf.data.append(args.items[next++]);
        f = f.substr(b + 1);
    }
}
template <typename... Args>
void format_to(memory_buffer& buf, std::string_view f, const Args&... args) {
    buf.data.append(format(f, args...));
}
inline std::string to_string(const memory_buffer& buf) { return buf.data; }
}
