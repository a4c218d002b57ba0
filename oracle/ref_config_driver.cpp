// Test-oracle driver around the reference's own headless.conf parser, compiled
// from the reference sources (src/core/Parser.cpp, src/core/Config.h,
// src/backend/headless/HeadlessConfig.cpp) by oracle/Makefile into
// oracle/_ref/.  Used only to check the command line's parser.
//
//   xn_ref_config <headless.conf>
//
// Reads the file as src/backend/headless/headless.cpp:11-22 does and prints
// one line "device <vkindex> <x> <y> <width> <height>" per device entry, or
// "error: <message>" when the parser throws.
#include <cstdio>
#include <fstream>
#include <string>
#include "backend/headless/HeadlessConfig.h"

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s headless.conf\n", argv[0]);
        return 2;
    }
    auto in = std::ifstream(argv[1]);
    if (!in) {
        std::printf("error: cannot open %s\n", argv[1]);
        return 0;
    }
    try {
        HeadlessConfig cfg = cfg::Config(in).as<HeadlessConfig>();
        for (const auto& d : cfg.gpus)
            std::printf("device %u %d %d %u %u\n", d.vulkan_index, d.region.offset.x, d.region.offset.y,
                        d.region.extent.width, d.region.extent.height);
    } catch (const Error& e) {
        std::string m = e.what();
        std::printf("error: ");
        std::fwrite(m.data(), 1, m.size(), stdout);
        std::printf("\n");
    }
    return 0;
}
