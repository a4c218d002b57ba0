// Test-oracle driver around the PNG library the reference writes its frames
// with (subprojects/lodepng, used by src/backend/headless/HeadlessDisplay.cpp),
// compiled from the reference checkout by oracle/Makefile into oracle/_ref/.
// Used only to check that the command line's PNG files decode to their pixels
// with an independent decoder.
//
//   xn_ref_png <in.png> <out.rgba>
//
// Decodes to 8-bit RGBA, writes the pixels raw and prints "ok <w> <h>", or
// prints "error <code> <text>".
#include <cstdio>
#include <fstream>
#include <iterator>
#include <vector>
#include "lodepng.h"

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.png out.rgba\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    std::vector<unsigned char> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    std::vector<unsigned char> px;
    unsigned w = 0, h = 0;
    unsigned e = lodepng::decode(px, w, h, data, LCT_RGBA, 8);
    if (e) {
        std::printf("error %u %s\n", e, lodepng_error_text(e));
        return 0;
    }
    std::ofstream(argv[2], std::ios::binary).write(reinterpret_cast<const char*>(px.data()), (std::streamsize)px.size());
    std::printf("ok %u %u\n", w, h);
    return 0;
}
