// Support code of the `xenodon` command line.  The grammars and messages
// follow the reference (src/core/arg_parse.cpp, src/core/Parser.cpp,
// src/core/Config.h, src/camera/ScriptCameraController.cpp) so that scripts
// and configuration files written for it behave the same.
#include "cli_util.h"

#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iostream>
#include <sstream>

namespace cli {

namespace {

std::string dup_error(const std::string& type, const std::string& long_arg, int short_arg) {
    if (short_arg != -1) return "Duplicate specification of " + type + " " + long_arg + "/-" + std::string(1, (char)short_arg);
    return "Duplicate specification of " + type + " " + long_arg;
}

bool matches(const std::string& arg, const std::string& long_arg, int short_arg) {
    return arg == long_arg || (arg.size() == 2 && (unsigned char)arg[1] == short_arg);
}

}  // namespace

void parse_args(const std::vector<std::string>& args, Command& cmd) {
    size_t pos_seen = 0;
    for (size_t i = 0; i < args.size(); ++i) {
        const std::string& arg = args[i];
        if (!arg.empty() && arg[0] == '-') {
            Flag* flag = nullptr;
            for (auto& f : cmd.flags)
                if (matches(arg, f.long_arg, f.short_arg)) { flag = &f; break; }
            if (flag) {
                if (flag->seen) throw Error(dup_error("flag", flag->long_arg, flag->short_arg));
                flag->seen = true;
                *flag->variable = true;
                continue;
            }
            Parameter* param = nullptr;
            for (auto& p : cmd.parameters)
                if (matches(arg, p.long_arg, p.short_arg)) { param = &p; break; }
            if (!param) throw Error("Unrecognized option " + arg);
            ++i;
            if (param->seen) throw Error(dup_error("parameter", param->long_arg, param->short_arg));
            if (i == args.size()) throw Error("Parameter " + arg + " expects argument <" + param->value_name + ">");
            param->seen = true;
            if (!param->action(args[i]))
                throw Error("Invalid value for <" + param->value_name + "> of parameter " + arg);
        } else if (pos_seen == cmd.positional.size()) {
            throw Error("Unexpected positional argument '" + arg + "'");
        } else {
            auto& p = cmd.positional[pos_seen];
            if (!p.action(arg)) throw Error("Invalid value for positional argument <" + p.name + ">");
            ++pos_seen;
        }
    }
    if (pos_seen != cmd.positional.size())
        throw Error("Missing required positional argument <" + cmd.positional[pos_seen].name + ">");
}

// arg_parse.h: only digits, '.' and '-' are accepted, and strtod must consume
// the whole string.
bool parse_float(const std::string& s, double& out) {
    for (char c : s)
        if (!std::isdigit((unsigned char)c) && c != '.' && c != '-') return false;
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end != s.c_str() + s.size()) return false;
    out = v;
    return true;
}

// std::from_chars for an unsigned integer: digits only, whole string.
bool parse_uint(const std::string& s, uint64_t& out) {
    if (s.empty()) return false;
    uint64_t v = 0;
    for (char c : s) {
        if (c < '0' || c > '9') return false;
        uint64_t d = (uint64_t)(c - '0');
        if (v > (UINT64_MAX - d) / 10) return false;
        v = v * 10 + d;
    }
    out = v;
    return true;
}

// ------------------------------------------------------------ headless.conf

namespace {

class Parser {
public:
    explicit Parser(const std::string& text) : s_(text) {}

    int peek() {
        int c = pos_ < s_.size() ? (unsigned char)s_[pos_] : -1;
        if (c == '#') fail_at("Unexpected character '#'");  // comments are an error in multi-line mode
        return c;
    }
    int consume() {
        if (pos_ >= s_.size()) fail_at("Unexpected end of input");
        int c = (unsigned char)s_[pos_++];
        if (c == '\n') {
            ++line_;
            col_ = 0;
        }
        ++col_;
        return c;
    }
    void expect(int e) {
        int a = consume();
        if (a != e) fail_at(std::string("Expected character '") + (char)e + "', found '" + (char)a + "'");
    }
    void optws() {
        while (std::isspace(peek())) consume();
    }
    std::string key() {
        int c = consume();
        if (!std::isalpha(c)) fail_at(std::string("Expected alphabetic key, found '") + (char)c + "'");
        std::string k(1, (char)c);
        while (std::isalpha(peek())) k += (char)consume();
        return k;
    }
    uint64_t number() {
        int c = consume();
        if (c < '0' || c > '9') fail_at(std::string("Expected numeric character, found '") + (char)c + "'");
        uint64_t v = (uint64_t)(c - '0');
        c = peek();
        while (c >= '0' && c <= '9') {
            v = v * 10 + (uint64_t)(c - '0');
            consume();
            c = peek();
        }
        return v;
    }
    std::pair<uint64_t, uint64_t> pair() {
        expect('(');
        optws();
        uint64_t a = number();
        optws();
        expect(',');
        optws();
        uint64_t b = number();
        optws();
        expect(')');
        return {a, b};
    }
    [[noreturn]] void fail_at(const std::string& msg) {
        throw Error("Parse error at line " + std::to_string(line_) + ", col " + std::to_string(col_) + ": " + msg);
    }

private:
    const std::string& s_;
    size_t pos_ = 0;
    size_t line_ = 1, col_ = 1;
};

// cfg::Config::parse: a whitespace-separated list of `key <item>`.
template <class OnKey>
void parse_items(Parser& p, OnKey on_key) {
    p.optws();
    int c = p.peek();
    while (std::isalpha(c)) {
        std::string k = p.key();
        p.optws();
        if (!on_key(k)) p.fail_at("Unexpected key '" + k + "'");
        c = p.peek();
        if (!std::isspace(c)) break;
        p.optws();
        c = p.peek();
    }
    p.optws();
}

}  // namespace

std::vector<HeadlessDevice> parse_headless_config(const std::string& text) {
    Parser p(text);
    std::vector<HeadlessDevice> devices;
    parse_items(p, [&](const std::string& k) {
        if (k != "device") return false;
        p.expect('{');
        HeadlessDevice d;
        bool have_index = false, have_offset = false, have_extent = false;
        parse_items(p, [&](const std::string& kk) {
            bool* seen = kk == "vkindex" ? &have_index : kk == "offset" ? &have_offset : kk == "extent" ? &have_extent : nullptr;
            if (!seen) return false;
            // the value is parsed before a repeated key is refused
            // (src/core/Config.h: accum(item.key, item.parse(*this)))
            p.expect('=');
            p.optws();
            HeadlessDevice v = d;
            if (kk == "vkindex") {
                v.vkindex = p.number();
            } else if (kk == "offset") {
                auto xy = p.pair();
                v.region.x = (int32_t)xy.first;
                v.region.y = (int32_t)xy.second;
            } else {
                auto wh = p.pair();
                v.region.width = (uint32_t)wh.first;
                v.region.height = (uint32_t)wh.second;
            }
            if (*seen) throw Error("Configuration error: Ambiguous key '" + kk + "'");
            *seen = true;
            d = v;
            return true;
        });
        // src/core/Config.h:205 builds the device from the accumulators'
        // get() calls as the arguments of one std::tuple constructor; built
        // with GCC those are evaluated last to first, so of several missing
        // keys the reference reports the last (extent, offset, vkindex)
        if (!have_extent) throw Error("Configuration error: Missing key 'extent'");
        if (!have_offset) throw Error("Configuration error: Missing key 'offset'");
        if (!have_index) throw Error("Configuration error: Missing key 'vkindex'");
        p.expect('}');
        devices.push_back(d);
        return true;
    });
    // src/backend/headless/HeadlessConfig.cpp:23-25 refuses an empty device
    // list before cfg::Config::as (src/core/Config.h:144-151) looks for the
    // end of the input
    if (devices.empty()) throw Error("Configuration error: At least one device entry is required");
    int c = p.peek();
    if (c > 0) p.fail_at(std::string("Expected end of input, found '") + (char)c + "'");
    return devices;
}

Rect rect_union(const Rect& a, const Rect& b) {
    Rect r;
    r.x = std::min(a.x, b.x);
    r.y = std::min(a.y, b.y);
    r.width = std::max((uint32_t)a.x + a.width, (uint32_t)b.x + b.width) - (uint32_t)r.x;
    r.height = std::max((uint32_t)a.y + a.height, (uint32_t)b.y + b.height) - (uint32_t)r.y;
    return r;
}

Rect rect_union_composite(const std::vector<Rect>& rects) {
    if (rects.empty()) return Rect{};
    int64_t bx = rects[0].x, by = rects[0].y;
    int64_t ex = bx + rects[0].width, ey = by + rects[0].height;
    for (size_t i = 1; i < rects.size(); ++i) {
        int64_t cx = rects[i].x, cy = rects[i].y;
        bx = std::min(bx, cx);
        by = std::min(by, cy);
        ex = std::max(ex, cx + (int64_t)rects[i].width);
        ey = std::max(ey, cy + (int64_t)rects[i].height);
    }
    Rect r;
    r.x = (int32_t)bx;
    r.y = (int32_t)bx;  // as the reference: the y origin is taken from x
    r.width = (uint32_t)(ex - bx);
    r.height = (uint32_t)(ey - by);
    return r;
}

// ------------------------------------------------------------ camera script

CameraScript::CameraScript(const std::string& path) {
    auto* f = new std::ifstream(path);
    in_ = f;
    if (!*f) {
        delete f;
        in_ = nullptr;
        throw Error("Failed to open '" + path + "'");
    }
    update();
}

CameraScript::~CameraScript() { delete static_cast<std::ifstream*>(in_); }

bool CameraScript::update() {
    auto& in = *static_cast<std::ifstream*>(in_);
    if (in.eof()) return true;
    float* dst[9] = {&current_.forward[0], &current_.forward[1], &current_.forward[2],
                     &current_.up[0], &current_.up[1], &current_.up[2],
                     &current_.translation[0], &current_.translation[1], &current_.translation[2]};
    for (float* d : dst) in >> *d;
    if (in.fail()) throw Error("Syntax error in camera input file");
    in >> std::ws;
    return false;
}

// ------------------------------------------------------------- formatting

std::string format_frame_name(const std::string& pat, uint64_t frame) {
    std::string out;
    int used = 0;
    for (size_t i = 0; i < pat.size(); ++i) {
        char c = pat[i];
        if (c == '}') {
            if (i + 1 < pat.size() && pat[i + 1] == '}') {
                out += '}';
                ++i;
                continue;
            }
            throw Error("unmatched '}' in format string");
        }
        if (c != '{') {
            out += c;
            continue;
        }
        if (i + 1 < pat.size() && pat[i + 1] == '{') {
            out += '{';
            ++i;
            continue;
        }
        size_t close = pat.find('}', i);
        if (close == std::string::npos) throw Error("missing '}' in format string");
        std::string field = pat.substr(i + 1, close - i - 1);
        i = close;
        std::string index = field, spec;
        size_t colon = field.find(':');
        if (colon != std::string::npos) {
            index = field.substr(0, colon);
            spec = field.substr(colon + 1);
        }
        if (!(index.empty() || index == "0") || (index.empty() && used > 0)) throw Error("argument index out of range");
        ++used;
        // [[fill]align][sign]['#']['0'][width][type]
        char fill = ' ', align = 0, type = 'd';
        size_t k = 0;
        auto is_align = [](char a) { return a == '<' || a == '>' || a == '^'; };
        if (spec.size() >= 2 && is_align(spec[1])) {
            fill = spec[0];
            align = spec[1];
            k = 2;
        } else if (!spec.empty() && is_align(spec[0])) {
            align = spec[0];
            k = 1;
        }
        std::string sign;
        if (k < spec.size() && (spec[k] == '+' || spec[k] == ' ')) {
            sign = spec[k] == '+' ? "+" : " ";
            ++k;
        } else if (k < spec.size() && spec[k] == '-') {
            ++k;
        }
        bool alt = false;
        if (k < spec.size() && spec[k] == '#') {
            alt = true;
            ++k;
        }
        bool zero = false;
        if (k < spec.size() && spec[k] == '0') {
            zero = true;
            ++k;
        }
        size_t width = 0;
        while (k < spec.size() && std::isdigit((unsigned char)spec[k])) width = width * 10 + (size_t)(spec[k++] - '0');
        if (k < spec.size()) type = spec[k++];
        if (k != spec.size()) throw Error("invalid format specifier");
        std::string digits, prefix;
        char buf[80];
        switch (type) {
        case 'd': case 'n': std::snprintf(buf, sizeof buf, "%llu", (unsigned long long)frame); break;
        case 'x': std::snprintf(buf, sizeof buf, "%llx", (unsigned long long)frame); if (alt) prefix = "0x"; break;
        case 'X': std::snprintf(buf, sizeof buf, "%llX", (unsigned long long)frame); if (alt) prefix = "0X"; break;
        case 'o': std::snprintf(buf, sizeof buf, "%llo", (unsigned long long)frame); if (alt && frame) prefix = "0"; break;
        case 'b': {
            std::string b;
            uint64_t v = frame;
            do { b.insert(b.begin(), (char)('0' + (v & 1))); v >>= 1; } while (v);
            std::snprintf(buf, sizeof buf, "%s", b.c_str());
            if (alt) prefix = "0b";
            break;
        }
        default: throw Error("invalid type specifier");
        }
        digits = buf;
        std::string body = sign + prefix + digits;
        if (body.size() < width) {
            size_t pad = width - body.size();
            if (!align && zero) body = sign + prefix + std::string(pad, '0') + digits;
            else if (align == '<') body += std::string(pad, fill);
            else if (align == '^') body = std::string(pad / 2, fill) + body + std::string(pad - pad / 2, fill);
            else body = std::string(pad, fill) + body;  // numbers align right by default
        }
        out += body;
    }
    return out;
}

// "{}" of a double in fmt 5.3.0, the version the reference builds with
// (subprojects/fmt.wrap): without FMT_USE_GRISU that is printf's %g
std::string fmt_double(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%g", v);
    return buf;
}

void Logger::log(const std::string& msg) {
    std::lock_guard<std::mutex> lk(mu);  // the frame-saving thread logs too
    std::time_t t = std::time(nullptr);
    char ts[32];
    std::tm tmv{};
    localtime_r(&t, &tmv);
    std::strftime(ts, sizeof ts, "[%H:%M:%S] ", &tmv);
    std::string line = std::string(ts) + msg;
    if (console) std::cout << line << '\n' << std::flush;
    if (sink) *sink << line << '\n' << std::flush;
}

}  // namespace cli
