// Test-oracle driver around the reference's own rect_union
// (src/utility/rect_union.h, header only), compiled from the reference checkout
// by oracle/Makefile into oracle/_ref/.  Used only to check the command line's
// restatement of both forms.
//
//   xn_ref_rect < lines "n x0 y0 w0 h0 x1 y1 w1 h1 ..."
//
// Prints, per line, "<pair> | <all>": the two-rectangle union of the first two
// rectangles and the iterator form over all n, each as "x y w h".
#include <sys/types.h>
#include <cstdio>
#include <iostream>
#include <vector>
#include "utility/rect_union.h"

int main() {
    size_t n;
    while (std::cin >> n) {
        std::vector<vk::Rect2D> rects(n);
        for (auto& r : rects) std::cin >> r.offset.x >> r.offset.y >> r.extent.width >> r.extent.height;
        vk::Rect2D pair = n >= 2 ? rect_union(rects[0], rects[1]) : vk::Rect2D{};
        vk::Rect2D all = rect_union(rects.begin(), rects.end(), [](const vk::Rect2D& r) { return r; });
        std::printf("%d %d %u %u | %d %d %u %u\n", pair.offset.x, pair.offset.y, pair.extent.width, pair.extent.height,
                    all.offset.x, all.offset.y, all.extent.width, all.extent.height);
    }
    return 0;
}
