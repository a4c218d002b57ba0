// `xenodon` command line: the reference's `render --headless` and `convert`
// surface (src/main.cpp, src/main_loop.cpp, src/convert.cpp) over the C ABI.
//
//   xenodon help [topic]
//   xenodon sysinfo
//   xenodon render --headless <config> [options] <volume.tif|volume.svo>
//   xenodon convert [--dag|--rope] [--chan-diff N|--std-dev X] <in.tif> <out.svo>
//
// Rendering runs on one CUDA device: each `device { ... }` block of the
// headless configuration is one output region rendered by one kernel launch,
// all against the union rectangle, so the composite matches a multi-GPU run of
// the reference pixel for pixel.  Errors print "Error: ..." as the reference
// does; the exit status is 1 after an error (the reference always exits 0).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include <xenodon.h>

#include "cli_util.h"

namespace {

const char* HELP_MAIN =
    "Usage: xenodon <command> [arguments]\n"
    "\n"
    "Commands:\n"
    "  help [topic]   Show help on a topic: render, convert, headless-config.\n"
    "  sysinfo        List the CUDA devices this build can render on.\n"
    "  render         Render a volume (a stacked TIFF grid or an .svo octree).\n"
    "  convert        Build a sparse voxel octree from a stacked TIFF.\n";

const char* HELP_RENDER =
    "Usage: xenodon render --headless <config> [options] <volume>\n"
    "\n"
    "Renders <volume> frame by frame and writes each frame to a PNG file.\n"
    "The volume type follows the extension (.tif/.tiff: grid, .svo: octree,\n"
    ".svc: octree in the device layout) unless --volume-type says otherwise.\n"
    "\n"
    "Options:\n"
    "  --headless <config>     Region layout, see 'xenodon help headless-config'.\n"
    "  --backend cuda          The device path (the only one in this build).\n"
    "  --camera <file>         Camera script: one line per frame with nine numbers,\n"
    "                          forward xyz, up xyz, position xyz.\n"
    "  -s, --shader <name>     dda (grids), svo-naive, svo-df, esvo, svo-rope\n"
    "                          (octrees; svo-rope needs a tree made with --rope).\n"
    "  -e, --emission-coeff    Multiplier of the integrated emission (default 1).\n"
    "  -r, --voxel-ratio x:y:z Scale of the volume axes (default 1:1:1).\n"
    "  --repeat <n>            Render every camera line n times.\n"
    "  --output <pattern>      Output file pattern with the frame number in {},\n"
    "                          e.g. 'out-{:0>3}.png' (default 'out-{}.png').\n"
    "  --discard-output        Write no images (for benchmarking).\n"
    "  --stats-output <file>   Per-frame timing statistics.\n"
    "  --volume-type <type>    tiff, tif, svo or svc.\n"
    "  --log-output <file>     Copy of the log.\n"
    "  -q, --quiet             No log on standard output.\n";

const char* HELP_CONVERT =
    "Usage: xenodon convert [options] <source tiff> <destination svo>\n"
    "\n"
    "Builds a sparse voxel octree from a stacked TIFF on the GPU.  A destination\n"
    "ending in .svc receives the device layout (internal nodes only; no 2^32\n"
    "node limit) instead of the XNDN-SVO node array.\n"
    "\n"
    "Options:\n"
    "  --dag             Merge identical subtrees into a directed acyclic graph.\n"
    "  --rope            Store face neighbours in the leaves (for svo-rope).\n"
    "  --chan-diff <n>   Merge a region into one leaf when no colour channel\n"
    "                    varies by more than n (0-255; 0 is lossless).\n"
    "  --std-dev <x>     Merge a region when the standard deviation of its\n"
    "                    colours is at most x.\n"
    "  --lean            (.svc, sparse trees) Build straight into the device\n"
    "                    layout, never holding the node array; not for svo-rope.\n"
    "  --streamed        (.svo, sparse trees) Build one top-level octant of the\n"
    "                    grid at a time on the device, writing its nodes as they\n"
    "                    are done; the same file as the whole-grid build.\n";

const char* HELP_HEADLESS =
    "The headless configuration lists the output regions:\n"
    "\n"
    "device {\n"
    "    vkindex = <index>\n"
    "    offset = (<x>, <y>)\n"
    "    extent = (<width>, <height>)\n"
    "}\n"
    "\n"
    "Each block is one region of the frame; all blocks are rendered on the\n"
    "current CUDA device (vkindex is accepted and not used).\n";

struct Failure {
    std::string msg;
};

std::string read_file(const std::string& path, bool* ok) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        *ok = false;
        return {};
    }
    std::stringstream ss;
    ss << in.rdbuf();
    *ok = true;
    return ss.str();
}

void check(int status) {
    if (status != XN_OK) throw Failure{xn_last_error()};
}

std::string lower_ext(const std::string& path) {
    size_t slash = path.find_last_of('/');
    size_t dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
    return path.substr(dot + 1);
}

enum class FileType { Tiff, Svo, Svc, Unknown };

FileType parse_file_type(const std::string& s) {
    if (s == "tiff" || s == "tif") return FileType::Tiff;
    if (s == "svo") return FileType::Svo;
    if (s == "svc") return FileType::Svc;  // device-layout octree file (xn_volume_save)
    return FileType::Unknown;
}

const char* file_type_name(FileType t) {
    return t == FileType::Tiff ? "tiff" : t == FileType::Svo ? "svo" : t == FileType::Svc ? "svc" : "unknown";
}

struct ShaderOption {
    const char* name;
    FileType type;
    int traversal;
};

// src/main_loop.cpp:37-43
const ShaderOption SHADERS[] = {
    {"dda", FileType::Tiff, XN_DDA},       {"svo-naive", FileType::Svo, XN_SVO_NAIVE},
    {"esvo", FileType::Svo, XN_ESVO},      {"svo-df", FileType::Svo, XN_SVO_DF},
    {"svo-rope", FileType::Svo, XN_SVO_ROPE},
};

struct RenderOptions {
    bool quiet = false, xorg = false, discard = false;
    std::string log_output, headless, output, direct, xorg_multi_gpu, backend = "cuda";
    std::string volume_type, shader, stats_output, camera, volume;
    double emission = 1.0;
    float ratio[3] = {1.f, 1.f, 1.f};
    uint64_t repeat = 1;
};

RenderOptions parse_render_args(const std::vector<std::string>& args) {
    RenderOptions o;
    bool have_output = false;
    auto str = [](std::string* v) { return [v](const std::string& a) { *v = a; return true; }; };
    cli::Command cmd;
    cmd.flags = {{&o.quiet, "--quiet", 'q'}, {&o.xorg, "--xorg"}, {&o.discard, "--discard-output"}};
    cmd.parameters = {
        {str(&o.log_output), "output path", "--log-output"},
        {str(&o.headless), "config path", "--headless"},
        {[&](const std::string& a) { o.output = a; have_output = true; return true; }, "output path", "--output"},
        {str(&o.direct), "config path", "--direct"},
        {str(&o.xorg_multi_gpu), "config path", "--xorg-multi-gpu"},
        {[&](const std::string& a) {
             double v;
             if (!cli::parse_float(a, v) || !(v >= 0.0) || v > 3.4028234663852886e38) return false;
             o.emission = v;
             return true;
         }, "emission coefficient", "--emission-coeff", 'e'},
        {str(&o.volume_type), "volume type", "--volume-type"},
        {str(&o.shader), "shader", "--shader", 's'},
        {[&](const std::string& a) {
             size_t f = a.find(':');
             size_t s = f == std::string::npos ? std::string::npos : a.find(':', f + 1);
             if (f == std::string::npos || s == std::string::npos) return false;
             std::string x = a.substr(0, f), y = a.substr(f + 1, s - f - 1), z = a.substr(s + 1);
             if (x.empty() || y.empty() || z.empty()) return false;
             double v[3];
             if (!cli::parse_float(x, v[0]) || !cli::parse_float(y, v[1]) || !cli::parse_float(z, v[2])) return false;
             if (!(v[0] > 0 && v[1] > 0 && v[2] > 0)) return false;
             for (int i = 0; i < 3; ++i) o.ratio[i] = (float)v[i];
             return true;
         }, "voxel dimension ratio", "--voxel-ratio", 'r'},
        {str(&o.stats_output), "stats output", "--stats-output"},
        {str(&o.camera), "camera", "--camera"},
        {[&](const std::string& a) {
             uint64_t v;
             // the reference accepts 0 and then divides by it; 0 is refused here
             if (!cli::parse_uint(a, v) || v == 0) return false;
             o.repeat = v;
             return true;
         }, "frame repeat", "--repeat"},
        {[&](const std::string& a) {
             if (a != "cuda") return false;
             o.backend = a;
             return true;
         }, "backend", "--backend"},
    };
    cmd.positional = {{str(&o.volume), "volume path"}};
    cli::parse_args(args, cmd);
    int backends = (int)o.xorg + (int)!o.headless.empty() + (int)!o.direct.empty();
    if (backends == 0) throw cli::Error("Missing required backend --xorg, --headless or --direct");
    if (backends > 1) throw cli::Error("--xorg, --headless and --direct are mutually exclusive");
    if (o.headless.empty() && o.discard) throw cli::Error("--dont-save requires --headless");
    if (have_output && o.headless.empty()) throw cli::Error("--output requires --headless");
    if (!have_output) o.output = "out-{}.png";
    else if (o.discard) throw cli::Error("--dont-save and --output are mutually exclusive");
    if (!o.xorg_multi_gpu.empty() && !o.xorg) throw cli::Error("--xorg-multi-gpu requires --xorg");
    return o;
}

struct FrameStats {
    uint64_t total_rays = 0, outputs = 0;
    double total = 0, max = 0, min = 0;
    double mrays() const { return (double)total_rays / (total * 1000.0); }
};

std::string output_name(const std::string& pattern, uint64_t frame) {
    try {
        return cli::format_frame_name(pattern, frame);
    } catch (const cli::Error& e) {
        throw cli::Error(std::string("Failed to format output filename: ") + e.what());
    }
}

// The frames in flight of a headless run: `depth` sets of one xn_output per
// device region, and one thread that composites a finished frame's regions
// into the enclosing rectangle (opaque black where no region is, like
// HeadlessDisplay::save, HeadlessDisplay.cpp:56-92) and writes its PNG.
class FramePipeline {
public:
    FramePipeline(xn_ctx* ctx, const std::vector<cli::HeadlessDevice>& devices, int depth, cli::Rect enclosing,
                  cli::Logger& log)
        : devices_(devices), enclosing_(enclosing), log_(log), busy_(depth, false) {
        outputs_.assign((size_t)depth, std::vector<xn_output*>(devices.size(), nullptr));
        try {
            for (auto& set : outputs_)
                for (size_t i = 0; i < devices.size(); ++i)
                    check(xn_output_create(ctx, (uint64_t)devices[i].region.width * devices[i].region.height, &set[i]));
        } catch (...) {
            for (auto& set : outputs_)
                for (xn_output* o : set) xn_output_destroy(o);
            throw;
        }
        saver_ = std::thread([this] { save_loop(); });
    }
    ~FramePipeline() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        if (saver_.joinable()) saver_.join();
        for (auto& set : outputs_)
            for (xn_output* o : set) xn_output_destroy(o);
    }
    xn_output* output(int set, size_t i) { return outputs_[(size_t)set][i]; }

    // Blocks until the frame last rendered into `set` has been saved.
    void acquire(int set) {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !busy_[(size_t)set]; });
    }

    // Waits for the regions of `frame` (rendered into `set`), returns its
    // stats, and hands the pixels to the saver unless `path` is empty.
    FrameStats finish(uint64_t frame, int set, const std::string& path) {
        FrameStats fs;
        fs.min = 1.7976931348623157e308;
        std::vector<const uint8_t*> px(devices_.size(), nullptr);
        for (size_t i = 0; i < devices_.size(); ++i) {
            float ms = 0;
            int r = xn_output_wait(outputs_[(size_t)set][i], &px[i], &ms);
            if (r == XN_ERR_RAY_LIMIT)
                log_.log("Warning: frame " + std::to_string(frame) + ", device " + std::to_string(i) + ": " +
                         xn_last_error() + "; the frame is saved as rendered");
            else
                check(r);
            fs.total_rays += (uint64_t)devices_[i].region.width * devices_[i].region.height;
            fs.outputs += 1;
            fs.total += ms;
            fs.max = std::max(fs.max, (double)ms);
            fs.min = std::min(fs.min, (double)ms);
        }
        if (!path.empty()) {
            std::lock_guard<std::mutex> lk(mu_);
            busy_[(size_t)set] = true;
            jobs_.push_back(Job{frame, path, std::move(px), set});
            cv_.notify_all();
        }
        return fs;
    }

    // Blocks until every handed-over frame is saved.
    void drain() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] {
            if (!jobs_.empty()) return false;
            for (bool b : busy_)
                if (b) return false;
            return true;
        });
    }

private:
    struct Job {
        uint64_t frame;
        std::string path;
        std::vector<const uint8_t*> pixels;
        int set;
    };

    void save_loop() {
        std::vector<uint8_t> image;
        for (;;) {
            Job job;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || !jobs_.empty(); });
                if (jobs_.empty()) return;
                job = std::move(jobs_.front());
                jobs_.erase(jobs_.begin());
            }
            log_.log("Saving frame " + std::to_string(job.frame) + "...");
            image.assign((size_t)enclosing_.width * enclosing_.height * 4, 0);
            for (size_t q = 0; q < image.size(); q += 4) image[q + 3] = 0xFF;  // 0xFF000000: opaque black
            for (size_t i = 0; i < devices_.size(); ++i) {
                const cli::Rect& rg = devices_[i].region;
                const size_t sx = (size_t)((int64_t)rg.x - enclosing_.x), sy = (size_t)((int64_t)rg.y - enclosing_.y);
                for (uint32_t y = 0; y < rg.height; ++y)
                    std::memcpy(&image[((sy + y) * enclosing_.width + sx) * 4], job.pixels[i] + (size_t)y * rg.width * 4,
                                (size_t)rg.width * 4);
            }
            log_.log("Compressing...");
            if (xn_png_save(job.path.c_str(), image.data(), enclosing_.width, enclosing_.height) != XN_OK)
                log_.log(std::string("Error saving output: ") + xn_last_error());
            else
                log_.log("Saved output to '" + job.path + "'");
            {
                std::lock_guard<std::mutex> lk(mu_);
                busy_[(size_t)job.set] = false;
            }
            cv_.notify_all();
        }
    }

    const std::vector<cli::HeadlessDevice>& devices_;
    cli::Rect enclosing_;
    cli::Logger& log_;
    std::vector<std::vector<xn_output*>> outputs_;
    std::vector<bool> busy_;
    std::vector<Job> jobs_;
    std::mutex mu_;
    std::condition_variable cv_;
    bool stop_ = false;
    std::thread saver_;
};

std::string stats_text(const std::vector<FrameStats>& frames, double wall_s) {
    // RenderStatsAccumulator::save (src/render/RenderStats.cpp:127-158)
    uint64_t rays = 0;
    double total = 0;
    for (auto& f : frames) {
        rays += f.total_rays;
        total += f.total;
    }
    std::string out;
    out += "total rays: " + std::to_string(rays) + "\n";
    out += "total render time: " + cli::fmt_double(total) + "\n";
    out += "total mray/s: " + cli::fmt_double((double)rays / (total * 1000.0)) + "\n";
    out += "average fps: " + cli::fmt_double((double)frames.size() / wall_s) + "\n";
    out += "frames: " + std::to_string(frames.size()) + "\n";
    out += "# Frame number: total rays, outputs, total render time, max render time, min render time, mray/s\n";
    for (size_t i = 0; i < frames.size(); ++i) {
        const auto& f = frames[i];
        out += "frame " + std::to_string(i) + ": " + std::to_string(f.total_rays) + " rays, " +
               std::to_string(f.outputs) + ", " + cli::fmt_double(f.total) + " ms, " + cli::fmt_double(f.max) +
               " ms, " + cli::fmt_double(f.min) + " ms, " + cli::fmt_double(f.mrays()) + " mray/s\n";
    }
    return out;
}

int render(const std::vector<std::string>& args) {
    RenderOptions o;
    try {
        o = parse_render_args(args);
    } catch (const cli::Error& e) {
        std::printf("Error: %s\n", e.what());
        return 1;
    }
    cli::Logger log;
    log.console = !o.quiet;
    std::ofstream log_file;
    if (!o.log_output.empty()) {
        log_file.open(o.log_output);
        log.sink = &log_file;
    }
    std::vector<cli::HeadlessDevice> devices;
    try {
        if (o.xorg || !o.direct.empty())
            throw cli::Error(std::string(o.xorg ? "the X.org" : "the direct") + " backend is not part of this build");
        log.log("Using headless presenting backend");
        bool ok = false;
        std::string text = read_file(o.headless, &ok);
        if (!ok) throw cli::Error("Failed to open config file '" + o.headless + "'");
        try {
            devices = cli::parse_headless_config(text);
        } catch (const cli::Error& e) {
            throw cli::Error("Failed to read config file '" + o.headless + "': " + e.what());
        }
    } catch (const cli::Error& e) {
        std::printf("Error: Failed to initialize backend: %s\n", e.what());
        return 1;
    }

    xn_ctx* ctx = nullptr;
    xn_volume* vol = nullptr;
    try {
        // check_setup (main_loop.cpp:45-68): one output per device block
        std::string setup = "Setup: " + std::to_string(devices.size()) + (devices.size() > 1 ? " devices" : " device") +
                            ", with ";
        for (size_t i = 0; i < devices.size(); ++i) setup += (i ? ", 1" : "1");
        setup += devices.size() > 1 ? " outputs" : " output";
        log.log(setup);

        FileType type = !o.volume_type.empty() ? parse_file_type(o.volume_type) : parse_file_type(lower_ext(o.volume));
        if (type == FileType::Unknown) throw cli::Error("Failed to parse model file type");
        log.log(std::string("Model file type: '") + file_type_name(type) + "'");
        const ShaderOption* shader = nullptr;
        if (!o.shader.empty()) {
            for (const auto& s : SHADERS)
                if (o.shader == s.name) shader = &s;
            if (!shader) throw cli::Error("Invalid shader '" + o.shader + "'");
            if (shader->type != (type == FileType::Svc ? FileType::Svo : type))
                throw cli::Error("Shader '" + o.shader + "' is incompatible with model type '" + file_type_name(type) +
                                 "' (requires '" + file_type_name(shader->type) + "')");
        } else {
            for (const auto& s : SHADERS)
                if (s.type == (type == FileType::Svc ? FileType::Svo : type)) { shader = &s; break; }
        }
        log.log(std::string("Using shader '") + shader->name + "'");

        check(xn_create(0, 0, &ctx));
        uint32_t dim[3];
        if (type == FileType::Tiff) {
            uint8_t* rgba = nullptr;
            if (xn_tiff_load(o.volume.c_str(), &rgba, dim) != XN_OK) throw cli::Error(xn_last_error());
            std::printf("%ux%ux%u = %llu pixels\n", dim[0], dim[1], dim[2], (unsigned long long)dim[0] * dim[1] * dim[2]);
            int r = xn_volume_upload_grid(ctx, rgba, dim[0], dim[1], dim[2], &vol);
            xn_free(rgba);
            check(r);
        } else if (type == FileType::Svc) {
            if (xn_volume_load(ctx, o.volume.c_str(), &vol) != XN_OK) throw cli::Error(xn_last_error());
            xn_volume_info info{};
            check(xn_volume_info_get(vol, &info));
            dim[0] = dim[1] = dim[2] = (uint32_t)info.side;
        } else {
            uint32_t* nodes = nullptr;
            uint64_t n = 0, side = 0;
            if (xn_svo_load(o.volume.c_str(), &nodes, &n, &side) != XN_OK) throw cli::Error(xn_last_error());
            int r = xn_volume_upload_svo(ctx, nodes, n, side, &vol);
            xn_free(nodes);
            check(r);
            dim[0] = dim[1] = dim[2] = (uint32_t)side;
        }
        log.log("Model dimensions: " + std::to_string(dim[0]) + "x" + std::to_string(dim[1]) + "x" + std::to_string(dim[2]));

        std::vector<cli::Rect> regions;
        cli::Rect display = devices[0].region;
        for (const auto& d : devices) {
            regions.push_back(d.region);
            display = cli::rect_union(display, d.region);
        }
        log.log("Total resolution: " + std::to_string(display.width) + "x" + std::to_string(display.height) + " pixels");

        if (o.camera.empty() || o.camera == "orbit")
            throw cli::Error("the interactive orbit camera needs a windowed backend; pass --camera <file>");
        log.log("Reading camera transforms from '" + o.camera + "'");
        cli::CameraScript script(o.camera);

        const cli::Rect enclosing = cli::rect_union_composite(regions);
        for (const auto& d : devices) {
            const cli::Rect& rg = d.region;
            int64_t sx = (int64_t)rg.x - enclosing.x, sy = (int64_t)rg.y - enclosing.y;
            if (sx < 0 || sy < 0 || sx + rg.width > enclosing.width || sy + rg.height > enclosing.height)
                throw cli::Error("the device regions do not fit the composite image");
        }
        // Two sets of outputs: frame n renders into set n % 2 while the saver
        // thread composites and encodes frame n-1 from the other set's pinned
        // read-back (HeadlessDisplay::swap_buffers and save,
        // HeadlessDisplay.cpp:39-92, moved off the render loop).
        // XN_HEADLESS_SERIAL=1 keeps one set: each frame is rendered, waited
        // for and saved before the next is queued, as the reference does.
        const char* serial_env = std::getenv("XN_HEADLESS_SERIAL");
        const int depth = serial_env && serial_env[0] == '1' ? 1 : 2;
        FramePipeline pipe(ctx, devices, depth, enclosing, log);
        std::vector<FrameStats> frames;
        auto start = std::chrono::steady_clock::now();
        auto fps_start = start;
        uint64_t fps_frames = 0, total_frames = 0, frame_no = 0;
        log.log("Starting render loop...");
        for (;;) {
            ++fps_frames;
            ++total_frames;
            const auto& c = script.camera();
            xn_camera cam;
            std::memcpy(cam.forward, c.forward, sizeof cam.forward);
            std::memcpy(cam.up, c.up, sizeof cam.up);
            std::memcpy(cam.translation, c.translation, sizeof cam.translation);
            const int set = (int)(frame_no % (uint64_t)depth);
            pipe.acquire(set);  // its previous frame is saved
            for (size_t i = 0; i < devices.size(); ++i) {
                xn_params p;
                p.output_region = {devices[i].region.x, devices[i].region.y, devices[i].region.width,
                                   devices[i].region.height};
                p.display_region = {display.x, display.y, display.width, display.height};
                for (int k = 0; k < 3; ++k) p.voxel_ratio[k] = o.ratio[k];
                p.emission_coeff = (float)o.emission;
                check(xn_output_render(pipe.output(set, i), vol, shader->traversal, &cam, &p,
                                       o.discard ? XN_OUTPUT_DISCARD : 0));
            }
            // finish the frame before this one (or this one, with one set)
            if (depth == 1) {
                frames.push_back(pipe.finish(frame_no, set, o.discard ? "" : output_name(o.output, frame_no)));
            } else if (frame_no > 0) {
                frames.push_back(pipe.finish(frame_no - 1, 1 - set,
                                             o.discard ? "" : output_name(o.output, frame_no - 1)));
            }
            const bool last = total_frames % o.repeat == 0 && script.update();
            if (last) {
                if (depth == 2) frames.push_back(pipe.finish(frame_no, set, o.discard ? "" : output_name(o.output, frame_no)));
                ++frame_no;
                break;
            }
            ++frame_no;
            auto now = std::chrono::steady_clock::now();
            double dt = std::chrono::duration<double>(now - fps_start).count();
            if (dt > 5.0) {
                log.log("FPS: " + cli::fmt_double((double)fps_frames / dt));
                fps_frames = 0;
                fps_start = now;
            }
        }
        pipe.drain();
        double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        uint64_t rays = 0;
        double total = 0;
        for (auto& f : frames) {
            rays += f.total_rays;
            total += f.total;
        }
        log.log("total rays: " + std::to_string(rays) + ", total render time: " + cli::fmt_double(total) +
                "ms, mray/s: " + cli::fmt_double((double)rays / (total * 1000.0)));
        log.log("frames: " + std::to_string(frames.size()) + ", fps: " + cli::fmt_double((double)frames.size() / wall) +
                ", total time: " + cli::fmt_double(wall) + "s");
        if (!o.stats_output.empty()) {
            std::ofstream f(o.stats_output);
            if (!f) throw cli::Error("Failed to open render stats output path '" + o.stats_output + "'");
            f << stats_text(frames, wall);
            log.log("Saved stats to '" + o.stats_output + "'");
        }
    } catch (const cli::Error& e) {
        std::printf("Error: %s\n", e.what());
        xn_volume_release(vol);
        xn_destroy(ctx);
        return 1;
    } catch (const Failure& e) {
        std::printf("Error: %s\n", e.msg.c_str());
        xn_volume_release(vol);
        xn_destroy(ctx);
        return 1;
    }
    xn_volume_release(vol);
    xn_destroy(ctx);
    return 0;
}

// The streamed build's region reader over a grid in host memory.
struct HostGrid {
    const uint8_t* rgba;
    uint32_t dx, dy, dz;
};

int read_host_region(void* user, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t nx, uint32_t ny, uint32_t nz,
                     uint8_t* out) {
    const HostGrid* g = static_cast<const HostGrid*>(user);
    if ((uint64_t)x0 + nx > g->dx || (uint64_t)y0 + ny > g->dy || (uint64_t)z0 + nz > g->dz) return 1;
    for (uint32_t z = 0; z < nz; ++z)
        for (uint32_t y = 0; y < ny; ++y)
            std::memcpy(out + (((uint64_t)z * ny + y) * nx) * 4,
                        g->rgba + ((((uint64_t)(z0 + z) * g->dy) + (y0 + y)) * g->dx + x0) * 4, (size_t)nx * 4);
    return 0;
}

int convert(const std::vector<std::string>& args) {
    std::string src, dst;
    bool dag = false, rope = false, lean = false, streamed = false;
    int64_t chan = -1;
    double sd = -1;
    cli::Command cmd;
    cmd.flags = {{&dag, "--dag"}, {&rope, "--rope"}, {&lean, "--lean"}, {&streamed, "--streamed"}};
    cmd.parameters = {
        {[&](const std::string& a) {
             uint64_t v;
             if (!cli::parse_uint(a, v) || v > 255) return false;
             chan = (int64_t)v;
             return true;
         }, "channel difference", "--chan-diff"},
        {[&](const std::string& a) {
             double v;
             if (!cli::parse_float(a, v) || !(v >= 0.0)) return false;
             sd = v;
             return true;
         }, "std. dev", "--std-dev"},
    };
    cmd.positional = {{[&](const std::string& a) { src = a; return true; }, "source tiff path"},
                      {[&](const std::string& a) { dst = a; return true; }, "destination svo path"}};
    try {
        cli::parse_args(args, cmd);
    } catch (const cli::Error& e) {
        std::printf("Error: %s\n", e.what());
        return 1;
    }
    if (dag && rope) {
        std::printf("Error: --dag and --rope are mutually exclusive\n");
        return 1;
    }
    if (chan >= 0 && sd >= 0) {
        std::printf("Error: --std-dev and --chan-diff are mutually exclusive\n");
        return 1;
    }
    // a .svc destination gets the device layout (xn_volume_save), built on
    // the device and written from it; --lean never forms the node array
    const bool svc = lower_ext(dst) == "svc";
    if (lean && (!svc || dag || rope)) {
        std::printf("Error: --lean builds a sparse tree into a .svc file (no --dag or --rope)\n");
        return 1;
    }
    if (streamed && (svc || dag || rope || lean)) {
        std::printf("Error: --streamed builds a sparse tree into a .svo file (no --dag, --rope or --lean)\n");
        return 1;
    }
    std::printf("Loading source...\n");
    uint8_t* rgba = nullptr;
    uint32_t dim[3];
    if (xn_tiff_load(src.c_str(), &rgba, dim) != XN_OK) {
        std::printf("Error reading '%s': %s\n", src.c_str(), xn_last_error());
        return 1;
    }
    std::printf("%ux%ux%u = %llu pixels\n", dim[0], dim[1], dim[2], (unsigned long long)dim[0] * dim[1] * dim[2]);
    const uint64_t voxels = (uint64_t)dim[0] * dim[1] * dim[2];
    std::printf("Source grid:\n");
    std::printf(" Dimensions: %ux%ux%u\n", dim[0], dim[1], dim[2]);
    std::printf(" Size: %llu bytes\n", (unsigned long long)(32 + voxels * 4));  // Grid::memory_footprint
    std::printf("Converting to octree...\n");
    std::fflush(stdout);
    xn_ctx* ctx = nullptr;
    uint32_t* nodes = nullptr;
    xn_volume* vol = nullptr;
    xn_build_stats st{};
    int r = xn_create(0, 0, &ctx);
    if (r == XN_OK) {
        const int type = dag ? XN_SVO_DAG : rope ? XN_SVO_ROPE_TREE : XN_SVO_SPARSE;
        const int heur = sd >= 0 ? XN_HEUR_STD_DEV : XN_HEUR_CHANNEL_DIFF;
        const double thr = sd >= 0 ? sd : (double)std::max<int64_t>(chan, 0);
        HostGrid hg{rgba, dim[0], dim[1], dim[2]};
        if (streamed)
            r = xn_build_svo_streamed(ctx, dim[0], dim[1], dim[2], heur, thr, read_host_region, &hg, dst.c_str(), &st);
        else
            r = svc ? xn_build_svo_volume(ctx, rgba, dim[0], dim[1], dim[2], type | (lean ? XN_BUILD_LEAN : 0), heur,
                                          thr, &vol, &st)
                    : xn_build_svo(ctx, rgba, dim[0], dim[1], dim[2], type, heur, thr, &nodes, &st);
    }
    xn_free(rgba);
    if (r != XN_OK) {
        std::printf("Error: %s\n", xn_last_error());
        xn_destroy(ctx);
        return 1;
    }
    // OctreeBuilder::insert reports every millionth unique node
    for (uint64_t k = 1000000; k <= st.n_nodes; k += 1000000) std::printf("%llu nodes...\n", (unsigned long long)k);
    // convert.cpp:88-115, including k_ary_nodes' ipow/(k+1)
    uint64_t z = 1;
    for (uint64_t y = st.depth + 1; --y;) z *= 8;
    const uint64_t perfect = (z - 1) / 9;
    const double total_prop = (double)st.total_nodes / (double)perfect;
    const double unique_prop = (double)st.n_nodes / (double)perfect;
    std::printf("Generated octree:\n");
    std::printf(" Dimensions: %llux%llux%llu\n", (unsigned long long)st.side, (unsigned long long)st.side,
                (unsigned long long)st.side);
    std::printf(" Size: %llu bytes\n", (unsigned long long)(32 + st.n_nodes * 40));  // Octree::memory_footprint
    std::printf(" Perfect tree nodes: %llu\n", (unsigned long long)perfect);
    std::printf(" Total nodes: %llu (%.5f%%)\n", (unsigned long long)st.total_nodes, total_prop * 100);
    std::printf(" Unique nodes: %llu (%.5f%%)\n", (unsigned long long)st.n_nodes, unique_prop * 100);
    std::printf(" Total leaves: %llu\n", (unsigned long long)st.total_leaves);
    std::printf(" Unique leaves: %llu\n", (unsigned long long)st.unique_leaves);
    std::printf(" Depth: %llu\n", (unsigned long long)st.depth);
    int rc = 0;
    if (!streamed &&
        (svc ? xn_volume_save(ctx, vol, dst.c_str()) : xn_svo_save(dst.c_str(), nodes, st.n_nodes, st.side)) != XN_OK) {
        std::printf("Error writing '%s': %s\n", dst.c_str(), xn_last_error());
        rc = 1;
    }
    xn_free(nodes);
    xn_volume_release(vol);
    xn_destroy(ctx);
    return rc;
}

int sysinfo() {
    xn_ctx* ctx = nullptr;
    if (xn_create(0, 0, &ctx) != XN_OK) {
        std::printf("Error: %s\n", xn_last_error());
        return 1;
    }
    uint64_t used = 0, budget = 0;
    xn_ctx_memory(ctx, &used, &budget);
    std::printf("CUDA device 0 is available for rendering.\n");
    xn_destroy(ctx);
    return 0;
}

}  // namespace

int main(int argc, const char* argv[]) {
    if (argc < 2) {
        std::printf("%s", HELP_MAIN);
        return 0;
    }
    std::vector<std::string> args(argv + 2, argv + argc);
    std::string sub = argv[1];
    if (sub == "help") {
        if (args.empty()) {
            std::printf("%s", HELP_MAIN);
            return 0;
        }
        if (args.size() != 1) {
            std::printf("Error: Invalid usage of subcommand 'help', see '%s help'\n", argv[0]);
            return 1;
        }
        const std::string& t = args[0];
        if (t == "help") std::printf("%s", HELP_MAIN);
        else if (t == "render") std::printf("%s", HELP_RENDER);
        else if (t == "convert") std::printf("%s", HELP_CONVERT);
        else if (t == "headless-config") std::printf("%s", HELP_HEADLESS);
        else {
            std::printf("Error: No such topic %s, see '%s help'\n", t.c_str(), argv[0]);
            return 1;
        }
        return 0;
    }
    if (sub == "sysinfo") return sysinfo();
    if (sub == "render") return render(args);
    if (sub == "convert") return convert(args);
    std::printf("Error: Invalid subcommand '%s', see '%s help'\n", sub.c_str(), argv[0]);
    return 1;
}
