// Support code of the `xenodon` command line: argv parsing, the headless
// configuration grammar, camera scripts, fmt-style output names, logging.
#pragma once

#include <cstdint>
#include <functional>
#include <ostream>
#include <stdexcept>
#include <mutex>
#include <string>
#include <vector>

namespace cli {

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ---- argv (the grammar of src/core/arg_parse.cpp:7-84)

struct Flag {
    bool* variable;
    std::string long_arg;
    int short_arg = -1;
    bool seen = false;
};

struct Parameter {
    std::function<bool(const std::string&)> action;
    std::string value_name;
    std::string long_arg;
    int short_arg = -1;
    bool seen = false;
};

struct Positional {
    std::function<bool(const std::string&)> action;
    std::string name;
};

struct Command {
    std::vector<Flag> flags;
    std::vector<Parameter> parameters;
    std::vector<Positional> positional;
};

void parse_args(const std::vector<std::string>& args, Command& cmd);

// Number parsing with the reference's acceptance rules (arg_parse.h).
bool parse_float(const std::string& s, double& out);
bool parse_uint(const std::string& s, uint64_t& out);

// ---- headless.conf (src/core/Config.h, Parser.cpp; HeadlessConfig.cpp:5-28)

struct Rect {
    int32_t x = 0, y = 0;
    uint32_t width = 0, height = 0;
};

struct HeadlessDevice {
    uint64_t vkindex = 0;
    Rect region;
};

std::vector<HeadlessDevice> parse_headless_config(const std::string& text);

// rect_union of two rectangles (src/utility/rect_union.h:11-25)
Rect rect_union(const Rect& a, const Rect& b);
// the iterator form used for the saved composite, including its use of the
// x origin for y (src/utility/rect_union.h:28-60)
Rect rect_union_composite(const std::vector<Rect>& rects);

// ---- camera scripts (src/camera/ScriptCameraController.cpp:17-40)

struct CameraLine {
    float forward[3], up[3], translation[3];
};

class CameraScript {
public:
    explicit CameraScript(const std::string& path);
    ~CameraScript();
    // true when the script is exhausted
    bool update();
    const CameraLine& camera() const { return current_; }

private:
    void* in_;
    CameraLine current_{};
};

// ---- fmt-style formatting of one integer ("out-{}.png", "out-{:0>3}.png")

std::string format_frame_name(const std::string& pattern, uint64_t frame);

// fmt's default "{}" for double as the reference prints it (general format,
// 6 significant digits)
std::string fmt_double(double v);

// ---- logging (src/core/Logger.cpp:20-30): "[HH:MM:SS] message"

struct Logger {
    bool console = true;
    std::ostream* sink = nullptr;  // --log-output file, truncated when opened
    std::mutex mu;
    void log(const std::string& msg);
};

}  // namespace cli
