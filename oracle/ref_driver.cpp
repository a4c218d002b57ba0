// Test-oracle driver around the reference's own octree builder, compiled from
// the reference sources (src/model/OctreeConstruction.h, Octree.cpp, Grid.cpp)
// by oracle/Makefile into oracle/_ref/.  Used only to produce golden SVO files
// and to check the C restatement in xo_build.c.
//
//   xn_ref_build <raw rgba> <dx> <dy> <dz> <sparse|dag|rope> <chan-diff|std-dev> <value> <out.svo>
//
// Prints "total_leaves unique_leaves total_nodes depth side n_nodes" on stdout.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>
#include "model/Grid.h"
#include "model/Octree.h"
#include "model/OctreeConstruction.h"

int main(int argc, char** argv) {
    if (argc != 9) {
        std::fprintf(stderr, "usage: %s raw dx dy dz type heuristic value out.svo\n", argv[0]);
        return 2;
    }
    size_t dx = std::strtoull(argv[2], nullptr, 10);
    size_t dy = std::strtoull(argv[3], nullptr, 10);
    size_t dz = std::strtoull(argv[4], nullptr, 10);
    std::vector<unsigned char> raw(dx * dy * dz * 4);
    {
        std::ifstream in(argv[1], std::ios::binary);
        in.read(reinterpret_cast<char*>(raw.data()), static_cast<std::streamsize>(raw.size()));
        if (!in) {
            std::fprintf(stderr, "short read\n");
            return 1;
        }
    }
    Grid grid(Vec3Sz(dx, dy, dz));
    for (size_t z = 0; z < dz; ++z)
        for (size_t y = 0; y < dy; ++y)
            for (size_t x = 0; x < dx; ++x) {
                const unsigned char* p = &raw[4 * (x + y * dx + z * dx * dy)];
                grid.set(Vec3Sz(x, y, z), Pixel{p[0], p[1], p[2], p[3]});
            }
    Octree::Type type = Octree::Type::Sparse;
    if (!std::strcmp(argv[5], "dag")) type = Octree::Type::Dag;
    else if (!std::strcmp(argv[5], "rope")) type = Octree::Type::Rope;
    ConstructionStats stats;
    auto build = [&]() {
        if (!std::strcmp(argv[6], "std-dev"))
            return build_octree(grid, stats, StdDevHeuristic{std::strtod(argv[7], nullptr)}, type);
        int cd = std::atoi(argv[7]);
        return build_octree(grid, stats, ChannelDiffHeuristic{static_cast<uint8_t>(cd < 0 ? 0 : cd)}, type);
    };
    Octree octree = build();
    octree.save_svo(argv[8]);
    std::printf("%zu %zu %zu %zu %zu %zu\n", stats.total_leaves, stats.unique_leaves, stats.total_nodes,
                stats.depth, octree.side(), octree.data().size());
    return 0;
}
