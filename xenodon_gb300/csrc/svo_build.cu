// GPU octree build, bit for bit the node array of the reference's recursive
// CPU builder (src/model/OctreeConstruction.h:124-237, src/model/Octree.cpp:116-201).
//
// The reference builds top-down and re-scans every voxel once per ancestor
// level; it inserts nodes in post-order (children 0..7, then the parent),
// reverses the array and rewrites child indices as `end - index`.  Here:
//
//  1. Bottom-up, one kernel per depth d = L-1 .. 0 over the cells of that depth
//     (cell extent e = side >> d):
//       - per-cell channel sums / min / max (ChannelDiff) or exact integer
//         moments (StdDev) reduced from the 8 child cells (from the voxels for
//         d = L-1), over the in-grid part only, like Grid::vol_scan clamps;
//       - the leaf decision of construct(): outside the grid -> black leaf;
//         (!split && fully inside) -> leaf; else internal;
//       - the size of the subtree the cell would root (1 for a leaf).
//  2. Top-down, one kernel per depth: an existing cell with post-order start
//     s and subtree size S gets final index N - s - S (the reversal of
//     build()); internal cells hand their children the starts s, s+S0,
//     s+S0+S1, ... and write their node.  Depth-L cells (single voxels) are
//     written by their parent.
//  3. Ropes (--rope): a leaf's neighbour across a face is the deepest existing
//     cell on the root path of the adjacent cell at the leaf's depth, which is
//     what Octree::find(pos +- extent, depth) returns.
//
// Cells of depth d are stored for the box B_d = min(2^d, 2*ceil(dim/(2e))) per
// axis, x fastest: the in-grid cells plus the outside cells that can be
// children of in-grid ones.
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <new>
#include <vector>

#include <unistd.h>

#include <cuda.h>  // CUcontext / CUresult types; the two driver calls are looked up at run time

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"
#include "xn_scan.cuh"

namespace xn {
namespace {

using namespace scan;

constexpr uint32_t LEAF = 0x80000000u;
constexpr uint64_t NONE = ~0ull;
constexpr uint8_t F_LEAF = 1, F_INSIDE = 2, F_AMBIG = 4;

struct LevelGeom {
    uint32_t bx, by, bz;  // box of stored cells
    uint64_t n;           // bx*by*bz
    uint64_t e;           // cell extent in voxels
};

struct CDStats {  // ChannelDiff: sums, per-channel min and max (packed RGBA)
    unsigned long long sum[4];
    uint32_t mn, mx;
};

struct SDStats {  // StdDev: first and second moments
    unsigned long long s1[4];
    unsigned long long s2[4];
};

struct GridDev {
    const uint32_t* vox;  // packed RGBA8, x fastest
    uint32_t dx, dy, dz;
};

__device__ __forceinline__ uint32_t vox_at(const GridDev& g, uint32_t x, uint32_t y, uint32_t z) {
    return __ldg(g.vox + (uint64_t)x + (uint64_t)g.dx * ((uint64_t)y + (uint64_t)g.dy * z));
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__device__ __forceinline__ uint32_t byte_min4(uint32_t a, uint32_t b) { return __vminu4(a, b); }
__device__ __forceinline__ uint32_t byte_max4(uint32_t a, uint32_t b) { return __vmaxu4(a, b); }

// Voxels of the cell clamped to the grid (Grid::vol_scan's bmin/bmax clamp).
__device__ __forceinline__ uint64_t clamped_count(const GridDev& g, uint64_t ox, uint64_t oy, uint64_t oz, uint64_t e) {
    uint64_t nx = umin64(g.dx, ox + e) - ox;
    uint64_t ny = umin64(g.dy, oy + e) - oy;
    uint64_t nz = umin64(g.dz, oz + e) - oz;
    return nx * ny * nz;
}

struct UpArgs {
    GridDev g;
    LevelGeom cur, child;   // child is unused at the deepest stored level
    int child_is_voxel;     // d + 1 == L
    const void* child_stats;
    void* stats;
    const unsigned long long* child_size;
    unsigned long long* size;
    uint32_t* color;
    uint8_t* flags;
    uint32_t chan_diff;     // ChannelDiff threshold (0..255)
    double stddev;          // StdDev threshold
    unsigned int* ambig_count;
    unsigned long long* ambig_list;
    int lean;               // subtree sizes count internal nodes only (the lean build)
};

__device__ __forceinline__ void cell_coords(uint64_t i, const LevelGeom& L, uint32_t& x, uint32_t& y, uint32_t& z) {
    x = (uint32_t)(i % L.bx);
    uint64_t r = i / L.bx;
    y = (uint32_t)(r % L.by);
    z = (uint32_t)(r / L.by);
}

__device__ __forceinline__ uint64_t cell_index(const LevelGeom& L, uint32_t x, uint32_t y, uint32_t z) {
    return (uint64_t)x + (uint64_t)L.bx * ((uint64_t)y + (uint64_t)L.by * z);
}

// Subtree size of child k of an internal cell (x, y, z) of the current level.
__device__ __forceinline__ uint64_t child_size(const UpArgs& a, uint32_t x, uint32_t y, uint32_t z, int k) {
    if (a.child_is_voxel) return a.lean ? 0 : 1;
    uint32_t cx = 2 * x + ((k >> 2) & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k & 1);
    return a.child_size[cell_index(a.child, cx, cy, cz)];
}

// construct()'s decision (OctreeConstruction.h:141-171) plus the subtree size.
template <int HEUR>
__global__ void up_level_kernel(UpArgs a) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.cur.n) return;
    uint32_t x, y, z;
    cell_coords(i, a.cur, x, y, z);
    const uint64_t e = a.cur.e;
    const uint64_t ox = x * e, oy = y * e, oz = z * e;
    const bool inside = ox < a.g.dx && oy < a.g.dy && oz < a.g.dz;
    if (!inside) {  // OctreeConstruction.h:146-154
        a.size[i] = a.lean ? 0 : 1;
        a.color[i] = 0;
        a.flags[i] = F_LEAF;
        return;
    }
    // the reference names this "partly_in_grid"; it means fully inside
    const bool fully = ox + e <= a.g.dx && oy + e <= a.g.dy && oz + e <= a.g.dz;
    const uint64_t half = e >> 1;
    unsigned long long s[4] = {0, 0, 0, 0};
    unsigned long long q[4] = {0, 0, 0, 0};
    uint32_t mn = 0xFFFFFFFFu, mx = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        uint32_t cx = 2 * x + ((k >> 2) & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k & 1);
        if ((uint64_t)cx * half >= a.g.dx || (uint64_t)cy * half >= a.g.dy || (uint64_t)cz * half >= a.g.dz) continue;
        if (a.child_is_voxel) {
            uint32_t v = vox_at(a.g, cx, cy, cz);
            mn = byte_min4(mn, v);
            mx = byte_max4(mx, v);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                unsigned long long b = (v >> (8 * c)) & 0xFFu;
                s[c] += b;
                q[c] += b * b;
            }
        } else if (HEUR == XN_HEUR_CHANNEL_DIFF) {
            const CDStats& cs = static_cast<const CDStats*>(a.child_stats)[cell_index(a.child, cx, cy, cz)];
            mn = byte_min4(mn, cs.mn);
            mx = byte_max4(mx, cs.mx);
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] += cs.sum[c];
        } else {
            const SDStats& cs = static_cast<const SDStats*>(a.child_stats)[cell_index(a.child, cx, cy, cz)];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                s[c] += cs.s1[c];
                q[c] += cs.s2[c];
            }
        }
    }
    const uint64_t n = clamped_count(a.g, ox, oy, oz, e);
    uint32_t avg = 0;
    bool split;
    bool ambiguous = false;
    if (HEUR == XN_HEUR_CHANNEL_DIFF) {
        CDStats& out = static_cast<CDStats*>(a.stats)[i];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            out.sum[c] = s[c];
            avg |= (uint32_t)(uint8_t)(s[c] / n) << (8 * c);  // Grid.cpp:126-131
        }
        out.mn = mn;
        out.mx = mx;
        // _mm_subs_epu8(max, min), then the largest channel (Grid.cpp:124,135)
        uint32_t d = __vsubus4(mx, mn);
        uint32_t maxdiff = max(max(d & 0xFFu, (d >> 8) & 0xFFu), max((d >> 16) & 0xFFu, d >> 24));
        split = maxdiff > a.chan_diff;
    } else {
        SDStats& out = static_cast<SDStats*>(a.stats)[i];
        const double nd = (double)n;
        unsigned __int128 E = 0;  // n * sum((x - mean)^2), exact
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            out.s1[c] = s[c];
            out.s2[c] = q[c];
            avg |= (uint32_t)(uint8_t)((double)s[c] / nd) << (8 * c);  // Grid.cpp:180-186,208-212
            E += (unsigned __int128)n * q[c] - (unsigned __int128)s[c] * s[c];
        }
        if (E == 0) {
            split = 0.0 > a.stddev;  // every voxel equals the mean: the double sum is exactly 0
        } else {
            // sqrt(sum/n) computed exactly up to double rounding; the
            // reference's sequential double sum differs from the exact value
            // by at most (n + 16) * 2^-52 relative; inside that band the
            // decision is taken from the reference's own loop (stddev_fixup).
            double var = (double)E / (nd * nd);
            double sd = sqrt(var);
            double band = (nd + 16.0) * 2.220446049250313e-16 * sd + 1e-300;
            if (fabs(sd - a.stddev) <= band) ambiguous = true;
            split = sd > a.stddev;
        }
    }
    a.color[i] = avg;
    if (ambiguous) {
        unsigned int slot = atomicAdd(a.ambig_count, 1u);
        a.ambig_list[slot] = i;
    }
    const bool leaf = (!split && fully) || e == 1;
    a.flags[i] = (leaf ? F_LEAF : 0) | F_INSIDE | (ambiguous ? F_AMBIG : 0);
    uint64_t sz = leaf && a.lean ? 0 : 1;
    if (!leaf) {
#pragma unroll
        for (int k = 0; k < 8; ++k) sz += child_size(a, x, y, z, k);
    }
    a.size[i] = sz;
}

// Grid::stddev_scan (Grid.cpp:139-214) run literally -- the sequential double
// loop in z, y, x order -- for the cells whose decision lies inside the
// rounding band of the exact computation.
__global__ void stddev_fixup_kernel(UpArgs a, unsigned int count) {
    unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    uint64_t i = a.ambig_list[j];
    uint32_t x, y, z;
    cell_coords(i, a.cur, x, y, z);
    const uint64_t e = a.cur.e;
    const uint64_t x0 = x * e, y0 = y * e, z0 = z * e;
    const uint64_t x1 = umin64(a.g.dx, x0 + e), y1 = umin64(a.g.dy, y0 + e),
                   z1 = umin64(a.g.dz, z0 + e);
    const SDStats& st = static_cast<const SDStats*>(a.stats)[i];
    const uint64_t n = (x1 - x0) * (y1 - y0) * (z1 - z0);
    const double nd = (double)n;
    double avg[4];
    for (int c = 0; c < 4; ++c) avg[c] = (double)st.s1[c] / nd;
    double s = 0.0;
    for (uint64_t zz = z0; zz < z1; ++zz)
        for (uint64_t yy = y0; yy < y1; ++yy)
            for (uint64_t xx = x0; xx < x1; ++xx) {
                uint32_t v = vox_at(a.g, (uint32_t)xx, (uint32_t)yy, (uint32_t)zz);
                double d0 = (double)(v & 0xFFu) - avg[0];
                double d1 = (double)((v >> 8) & 0xFFu) - avg[1];
                double d2 = (double)((v >> 16) & 0xFFu) - avg[2];
                double d3 = (double)(v >> 24) - avg[3];
                s += ((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3;
            }
    const bool split = sqrt(s / nd) > a.stddev;
    const bool fully = x0 + e <= a.g.dx && y0 + e <= a.g.dy && z0 + e <= a.g.dz;
    const bool leaf = (!split && fully) || e == 1;
    a.flags[i] = (leaf ? F_LEAF : 0) | F_INSIDE;
}

// Recomputes subtree sizes of a level after stddev_fixup changed decisions.
__global__ void resize_level_kernel(UpArgs a) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.cur.n) return;
    if (a.flags[i] & F_LEAF) {
        a.size[i] = a.lean ? 0 : 1;
        return;
    }
    uint32_t x, y, z;
    cell_coords(i, a.cur, x, y, z);
    uint64_t sz = 1;
    for (int k = 0; k < 8; ++k) sz += child_size(a, x, y, z, k);
    a.size[i] = sz;
}

struct DownArgs {
    GridDev g;
    LevelGeom cur, child;
    int child_is_voxel;
    int depth;
    uint64_t n_total;
    const unsigned long long* size;
    const unsigned long long* child_size;
    const uint32_t* color;
    const uint8_t* flags;
    const uint32_t* child_color;  // lean build: the child level's colours and flags
    const uint8_t* child_flags;
    const unsigned long long* start;
    unsigned long long* child_start;
    uint32_t* nodes;  // n_total x 10 words, or null when only the starts are wanted
    unsigned long long* leaves;  // total leaf count
    unsigned int* max_depth;
    unsigned long long* existing;  // [0] existing cells of this level, [1] of them internal
};

__device__ __forceinline__ void write_node(uint32_t* nodes, uint64_t idx, const uint32_t ch[8], uint32_t color,
                                           uint32_t leaf_depth) {
    if (!nodes) return;
    uint2* p = reinterpret_cast<uint2*>(nodes + idx * 10);  // 40-byte nodes are 8-byte aligned
    p[0] = make_uint2(ch[0], ch[1]);
    p[1] = make_uint2(ch[2], ch[3]);
    p[2] = make_uint2(ch[4], ch[5]);
    p[3] = make_uint2(ch[6], ch[7]);
    p[4] = make_uint2(color, leaf_depth);
}

// OctreeBuilder::build (OctreeConstruction.h:92-112) applied to the
// post-order positions: index = N-1-post, post = start + size - 1.
__global__ void down_level_kernel(DownArgs a) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long leaves = 0, exist = 0, internal = 0;
    unsigned int deepest = 0;
    bool active = i < a.cur.n;
    uint64_t st = active ? a.start[i] : NONE;
    if (st != NONE) {
        exist = 1;
        internal = (a.flags[i] & F_LEAF) ? 0 : 1;
        const uint64_t S = a.size[i];
        const uint64_t idx = a.n_total - st - S;
        const uint8_t f = a.flags[i];
        uint32_t ch[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        deepest = (unsigned)a.depth;
        if (f & F_LEAF) {
            leaves = 1;
            write_node(a.nodes, idx, ch, a.color[i], LEAF | (uint32_t)a.depth);
        } else {
            uint32_t x, y, z;
            cell_coords(i, a.cur, x, y, z);
            uint64_t run = st;
            const uint32_t cd = (uint32_t)a.depth + 1;
            for (int k = 0; k < 8; ++k) {
                uint32_t cx = 2 * x + ((k >> 2) & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k & 1);
                if (a.child_is_voxel) {
                    const uint64_t cidx = a.n_total - run - 1;
                    ch[k] = (uint32_t)cidx;
                    uint32_t v = (cx < a.g.dx && cy < a.g.dy && cz < a.g.dz) ? vox_at(a.g, cx, cy, cz) : 0u;
                    const uint32_t zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    write_node(a.nodes, cidx, zero, v, LEAF | cd);
                    run += 1;
                    leaves += 1;
                    deepest = cd;
                } else {
                    const uint64_t ci = cell_index(a.child, cx, cy, cz);
                    const uint64_t cS = a.child_size[ci];
                    a.child_start[ci] = run;
                    ch[k] = (uint32_t)(a.n_total - run - cS);
                    run += cS;
                }
            }
            write_node(a.nodes, idx, ch, a.color[i], (uint32_t)a.depth);
        }
    }
    // block-aggregate the statistics before touching global atomics
    for (int o = 16; o > 0; o >>= 1) {
        leaves += __shfl_down_sync(0xFFFFFFFFu, leaves, o);
        exist += __shfl_down_sync(0xFFFFFFFFu, exist, o);
        internal += __shfl_down_sync(0xFFFFFFFFu, internal, o);
        deepest = max(deepest, __shfl_down_sync(0xFFFFFFFFu, deepest, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (leaves) atomicAdd(a.leaves, leaves);
        if (exist) atomicAdd(a.existing, exist);
        if (internal) atomicAdd(a.existing + 1, internal);
        if (deepest) atomicMax(a.max_depth, deepest);
    }
}

// The lean build's top-down pass: sizes and starts count internal nodes only,
// so index N - start - size is a node's rank among the internal nodes in the
// reference's node order -- the order the device layout (svo_layout.cu) gives
// them.  Every internal cell writes its eight child words (leaf: bit 31 | RGB,
// internal: that child's rank) and its depth; leaves write nothing.
__global__ void lean_down_kernel(DownArgs a, uint32_t* inner, uint32_t* inner_depth) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long leaves = 0, internal = 0;
    unsigned int deepest = 0;
    const uint64_t st = i < a.cur.n ? a.start[i] : NONE;
    if (st != NONE && !(a.flags[i] & F_LEAF)) {
        internal = 1;
        const uint64_t idx = a.n_total - st - a.size[i];
        uint32_t x, y, z;
        cell_coords(i, a.cur, x, y, z);
        uint64_t run = st;
        uint32_t ch[8];
        for (int k = 0; k < 8; ++k) {
            const uint32_t cx = 2 * x + ((k >> 2) & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k & 1);
            if (a.child_is_voxel) {
                const uint32_t v = (cx < a.g.dx && cy < a.g.dy && cz < a.g.dz) ? vox_at(a.g, cx, cy, cz) : 0u;
                ch[k] = LEAF | (v & 0xFFFFFFu);
                ++leaves;
            } else {
                const uint64_t ci = cell_index(a.child, cx, cy, cz);
                if (a.child_flags[ci] & F_LEAF) {
                    ch[k] = LEAF | (a.child_color[ci] & 0xFFFFFFu);
                    ++leaves;
                } else {
                    const uint64_t cS = a.child_size[ci];
                    a.child_start[ci] = run;
                    ch[k] = (uint32_t)(a.n_total - run - cS);
                    run += cS;
                }
            }
        }
        deepest = leaves ? (unsigned)a.depth + 1 : 0;
        uint4* p = reinterpret_cast<uint4*>(inner + idx * 8);
        p[0] = make_uint4(ch[0], ch[1], ch[2], ch[3]);
        p[1] = make_uint4(ch[4], ch[5], ch[6], ch[7]);
        inner_depth[idx] = (uint32_t)a.depth;
    }
    for (int o = 16; o > 0; o >>= 1) {
        leaves += __shfl_down_sync(0xFFFFFFFFu, leaves, o);
        internal += __shfl_down_sync(0xFFFFFFFFu, internal, o);
        deepest = max(deepest, __shfl_down_sync(0xFFFFFFFFu, deepest, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (leaves) atomicAdd(a.leaves, leaves);
        if (internal) atomicAdd(a.existing + 1, internal);
        if (deepest) atomicMax(a.max_depth, deepest);
    }
}

struct LevelDev {
    LevelGeom geom;
    const unsigned long long* size;
    const unsigned long long* start;
    const uint8_t* flags;
};

constexpr int MAX_LEVELS = 40;

struct RopeArgs {
    int L;  // depth of single-voxel cells
    uint64_t n_total;
    LevelDev lv[MAX_LEVELS];
    uint32_t* nodes;
};

// Index of the existing node at (level, cell), or NONE.
__device__ __forceinline__ uint64_t node_at(const RopeArgs& a, int level, uint64_t cx, uint64_t cy, uint64_t cz) {
    if (level < a.L) {
        const LevelDev& d = a.lv[level];
        if (cx >= d.geom.bx || cy >= d.geom.by || cz >= d.geom.bz) return NONE;
        uint64_t i = cell_index(d.geom, (uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
        uint64_t st = d.start[i];
        if (st == NONE) return NONE;
        return a.n_total - st - d.size[i];
    }
    const LevelDev& p = a.lv[a.L - 1];
    uint64_t px = cx >> 1, py = cy >> 1, pz = cz >> 1;
    if (px >= p.geom.bx || py >= p.geom.by || pz >= p.geom.bz) return NONE;
    uint64_t i = cell_index(p.geom, (uint32_t)px, (uint32_t)py, (uint32_t)pz);
    uint64_t st = p.start[i];
    if (st == NONE || (p.flags[i] & F_LEAF)) return NONE;
    uint32_t k = (uint32_t)(((cx & 1) << 2) | ((cy & 1) << 1) | (cz & 1));
    return a.n_total - (st + k) - 1;
}

// Octree::generate_ropes (Octree.cpp:181-201) for one leaf at (level, cell).
__device__ void write_ropes(const RopeArgs& a, int level, uint64_t cx, uint64_t cy, uint64_t cz, uint64_t idx) {
    const uint64_t lim = 1ull << level;
    uint32_t r[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int axis = k >> 1;
        const int64_t s = (k & 1) ? -1 : 1;
        int64_t c[3] = {(int64_t)cx, (int64_t)cy, (int64_t)cz};
        c[axis] += s;
        if (c[axis] < 0 || (uint64_t)c[axis] >= lim) {  // outside the octree: find returns index 0
            r[k] = 0;
            continue;
        }
        uint64_t found = 0;
        for (int l = level; l >= 0; --l) {
            const int sh = level - l;
            uint64_t id = node_at(a, l, (uint64_t)c[0] >> sh, (uint64_t)c[1] >> sh, (uint64_t)c[2] >> sh);
            if (id != NONE) {
                found = id;
                break;
            }
        }
        r[k] = (uint32_t)found;
    }
    uint2* p = reinterpret_cast<uint2*>(a.nodes + idx * 10);
    p[0] = make_uint2(r[0], r[1]);
    p[1] = make_uint2(r[2], r[3]);
    p[2] = make_uint2(r[4], r[5]);
}

__global__ void rope_level_kernel(RopeArgs a, int level) {
    const LevelDev& d = a.lv[level];
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.geom.n) return;
    uint64_t st = d.start[i];
    if (st == NONE) return;
    uint32_t x, y, z;
    cell_coords(i, d.geom, x, y, z);
    if (d.flags[i] & F_LEAF) {
        write_ropes(a, level, x, y, z, a.n_total - st - d.size[i]);
    } else if (level == a.L - 1) {
        for (int k = 0; k < 8; ++k) {
            uint64_t cx = 2ull * x + ((k >> 2) & 1), cy = 2ull * y + ((k >> 1) & 1), cz = 2ull * z + (k & 1);
            write_ropes(a, a.L, cx, cy, cz, a.n_total - (st + k) - 1);
        }
    }
}

// -------------------------------------------------------------------- DAG ---
//
// HashCache (OctreeConstruction.h:19-30): a node equal to one inserted earlier
// (same colour, is_leaf_depth and children) is replaced by the earlier one,
// and the unique nodes are numbered in insertion (post-)order.  With the
// post-order position p(v) of every node of the sparse tree known, the class
// of a node is the smallest position among its equals; equality is decided
// depth by depth, deepest first, since depth is part of is_leaf_depth and an
// internal node's key holds its children's classes.  Keys are compared in
// full (a hash only picks the probe start), so hash collisions cannot merge
// different nodes.

struct DagKey {
    uint32_t color, leaf_depth;
    unsigned long long ch[8];
};

struct DagLevel {
    int depth, L;
    LevelGeom geom;  // depth < L: the cells of this depth; depth == L: the cells of depth L-1
    const unsigned long long* start;
    const unsigned long long* size;
    const uint32_t* color;
    const uint8_t* flags;
    const unsigned long long* child_canon;  // classes of depth+1 (cell-indexed, or 8*i+k for voxels)
    LevelGeom child_geom;
    int child_is_voxel;
    GridDev g;
    unsigned long long* canon;  // class per local id
};

__device__ __forceinline__ uint64_t dag_ids(const DagLevel& a) { return a.depth < a.L ? a.geom.n : 8 * a.geom.n; }

__device__ bool dag_node(const DagLevel& a, uint64_t id, DagKey& k, uint64_t& post) {
    if (a.depth < a.L) {
        const uint64_t st = a.start[id];
        if (st == NONE) return false;
        post = st + a.size[id] - 1;
        k.color = a.color[id];
        const bool leaf = a.flags[id] & F_LEAF;
        k.leaf_depth = (leaf ? LEAF : 0u) | (uint32_t)a.depth;
        uint32_t x, y, z;
        cell_coords(id, a.geom, x, y, z);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            if (leaf) { k.ch[c] = 0; continue; }
            if (a.child_is_voxel) {
                k.ch[c] = a.child_canon[8 * id + c];
            } else {
                uint32_t cx = 2 * x + ((c >> 2) & 1), cy = 2 * y + ((c >> 1) & 1), cz = 2 * z + (c & 1);
                k.ch[c] = a.child_canon[cell_index(a.child_geom, cx, cy, cz)];
            }
        }
        return true;
    }
    const uint64_t i = id >> 3;
    const uint32_t c = (uint32_t)(id & 7);
    const uint64_t st = a.start[i];
    if (st == NONE || (a.flags[i] & F_LEAF)) return false;
    post = st + c;
    uint32_t x, y, z;
    cell_coords(i, a.geom, x, y, z);
    uint32_t vx = 2 * x + ((c >> 2) & 1), vy = 2 * y + ((c >> 1) & 1), vz = 2 * z + (c & 1);
    k.color = (vx < a.g.dx && vy < a.g.dy && vz < a.g.dz) ? vox_at(a.g, vx, vy, vz) : 0u;
    k.leaf_depth = LEAF | (uint32_t)a.L;
#pragma unroll
    for (int j = 0; j < 8; ++j) k.ch[j] = 0;
    return true;
}

__device__ __forceinline__ bool key_eq(const DagKey& a, const DagKey& b) {
    if (a.color != b.color || a.leaf_depth != b.leaf_depth) return false;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (a.ch[j] != b.ch[j]) return false;
    return true;
}

__device__ __forceinline__ uint64_t mix64(uint64_t h) {
    h ^= h >> 30;
    h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 27;
    h *= 0x94d049bb133111ebull;
    h ^= h >> 31;
    return h;
}

__device__ __forceinline__ uint64_t key_hash(const DagKey& k) {
    uint64_t h = mix64(((uint64_t)k.color << 32) | k.leaf_depth);
#pragma unroll
    for (int j = 0; j < 8; ++j) h = mix64(h ^ (k.ch[j] + 0x9e3779b97f4a7c15ull * (j + 1)));
    return h;
}

struct Slot {
    unsigned long long owner;  // local id of the first node that claimed the slot
    unsigned long long rep;    // smallest post-order position of the class
};

__global__ void dag_insert_kernel(DagLevel a, Slot* table, uint64_t mask, unsigned int* overflow) {
    const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= dag_ids(a)) return;
    DagKey k;
    uint64_t post;
    if (!dag_node(a, id, k, post)) return;
    uint64_t slot = key_hash(k) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        unsigned long long o = atomicCAS(&table[slot].owner, NONE, (unsigned long long)id);
        if (o == NONE) {
            atomicMin(&table[slot].rep, (unsigned long long)post);
            return;
        }
        DagKey ko;
        uint64_t po;
        if (dag_node(a, o, ko, po) && key_eq(k, ko)) {
            atomicMin(&table[slot].rep, (unsigned long long)post);
            return;
        }
        slot = (slot + 1) & mask;
    }
    atomicOr(overflow, 1u);
}

__global__ void dag_lookup_kernel(DagLevel a, const Slot* table, uint64_t mask, unsigned int* overflow) {
    const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= dag_ids(a)) return;
    DagKey k;
    uint64_t post;
    if (!dag_node(a, id, k, post)) return;
    uint64_t slot = key_hash(k) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long o = table[slot].owner;
        if (o == NONE) break;
        DagKey ko;
        uint64_t po;
        if (dag_node(a, o, ko, po) && key_eq(k, ko)) {
            a.canon[id] = table[slot].rep;
            return;
        }
        slot = (slot + 1) & mask;
    }
    atomicOr(overflow, 2u);
}

__global__ void dag_mark_kernel(DagLevel a, uint8_t* is_rep) {
    const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= dag_ids(a)) return;
    DagKey k;
    uint64_t post;
    if (!dag_node(a, id, k, post)) return;
    if (a.canon[id] == post) is_rep[post] = 1;
}

// Writes the unique nodes: insertion index = rank among representatives in
// post-order, final index = U-1-insertion index (OctreeBuilder::build).
__global__ void dag_write_kernel(DagLevel a, const unsigned int* ins, uint64_t U, uint32_t* nodes,
                                 unsigned long long* unique_leaves) {
    const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long ul = 0;
    if (id < dag_ids(a)) {
        DagKey k;
        uint64_t post;
        if (dag_node(a, id, k, post) && a.canon[id] == post) {
            uint32_t ch[8];
            const bool leaf = k.leaf_depth & LEAF;
#pragma unroll
            for (int j = 0; j < 8; ++j) ch[j] = leaf ? 0u : (uint32_t)(U - 1 - ins[k.ch[j]]);
            write_node(nodes, U - 1 - ins[post], ch, k.color, k.leaf_depth);
            ul = leaf ? 1 : 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) ul += __shfl_down_sync(0xFFFFFFFFu, ul, o);
    if ((threadIdx.x & 31) == 0 && ul) atomicAdd(unique_leaves, ul);
}

uint64_t ceil_pow2(uint64_t x) {
    --x;
    x |= x >> 1;
    x |= x >> 2;
    x |= x >> 4;
    x |= x >> 8;
    x |= x >> 16;
    x |= x >> 32;
    return ++x;
}

struct Scratch {
    Ctx* c;
    std::vector<std::pair<void*, uint64_t>> bufs;
    explicit Scratch(Ctx* c) : c(c) {}
    ~Scratch() {
        cudaStreamSynchronize(c->stream);
        for (auto& b : bufs) c->device_free(b.first, b.second);
    }
    template <class T>
    int alloc(T** p, uint64_t count, const char* what) {
        void* v = nullptr;
        int r = c->device_alloc(&v, count * sizeof(T) + 16, what);
        if (r) return r;
        bufs.emplace_back(v, count * sizeof(T) + 16);
        *p = static_cast<T*>(v);
        return XN_OK;
    }
};

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Exclusive prefix sum of n small counts into u32 (recursive over block sums).
template <class In>
int exclusive_scan(Scratch& sc, const In* in, uint64_t n, unsigned* out, cudaStream_t s) {
    const uint64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (nb <= 1) {
        scan_apply_kernel<In><<<1, SCAN_T, 0, s>>>(in, n, nullptr, out);
        return XN_OK;
    }
    unsigned* sums = nullptr;
    unsigned* offs = nullptr;
    int r;
    if ((r = sc.alloc(&sums, nb, "xn_build_svo: scan")) || (r = sc.alloc(&offs, nb, "xn_build_svo: scan"))) return r;
    scan_reduce_kernel<In><<<(unsigned)nb, SCAN_T, 0, s>>>(in, n, sums);
    if ((r = exclusive_scan<unsigned>(sc, sums, nb, offs, s))) return r;
    scan_apply_kernel<In><<<(unsigned)nb, SCAN_T, 0, s>>>(in, n, offs, out);
    return XN_OK;
}

}  // namespace

// Builds the reference node array of an RGBA8 grid that is already on the
// device (packed RGBA, x fastest).  On success *d_nodes is a device buffer of
// n_nodes*10 words owned by the caller through ctx->device_free.
int build_svo_device(Ctx* c, const uint32_t* d_vox, uint32_t dx, uint32_t dy, uint32_t dz, int type, int heuristic,
                     double threshold, uint32_t** d_nodes, uint64_t* d_nodes_bytes, xn_build_stats* stats,
                     Volume* lean, SubBuild* sub) {
    cudaStream_t s = c->stream;
    const uint64_t fit = std::max(ceil_pow2(dx), std::max(ceil_pow2(dy), ceil_pow2(dz)));
    const uint64_t side = sub ? sub->side : fit;
    const int depth_off = sub ? sub->depth_offset : 0;
    int L = 0;
    while ((1ull << L) < side) ++L;
    GridDev g{d_vox, dx, dy, dz};
    std::memset(stats, 0, sizeof *stats);
    stats->side = side;
    *d_nodes = nullptr;
    *d_nodes_bytes = 0;
    if (L >= MAX_LEVELS) return fail(XN_ERR_ARG, "xn_build_svo: grid too large");
    if (sub && (side < fit || (side & (side - 1)) || L == 0 || lean || type != XN_SVO_SPARSE))
        return fail(XN_ERR_ARG, "xn_build_svo: invalid cube build (side %llu for a %ux%ux%u grid)",
                    (unsigned long long)side, dx, dy, dz);
    if (lean && L == 0) return LEAN_LEAF_ROOT;

    if (L == 0) {  // a single voxel: the root is a depth-0 leaf
        uint32_t* nodes = nullptr;
        int r = c->device_alloc(reinterpret_cast<void**>(&nodes), 40, "xn_build_svo: nodes");
        if (r) return r;
        uint32_t v = 0;
        cudaError_t e = cudaMemcpyAsync(&v, d_vox, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        uint32_t host[10] = {0, 0, 0, 0, 0, 0, 0, 0, v, LEAF};
        if (e == cudaSuccess) e = cudaMemcpyAsync(nodes, host, 40, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            c->device_free(nodes, 40);
            return cuda_fail(e, "xn_build_svo");
        }
        *d_nodes = nodes;
        *d_nodes_bytes = 40;
        stats->total_leaves = stats->unique_leaves = stats->total_nodes = stats->n_nodes = 1;
        return XN_OK;
    }

    std::vector<LevelGeom> geo(L);
    for (int d = 0; d < L; ++d) {
        const uint64_t e = side >> d;
        auto box = [&](uint64_t dim) -> uint32_t {
            if (d == 0) return 1;
            uint64_t pe = e * 2;  // parent extent
            uint64_t m = (dim + pe - 1) / pe;
            return (uint32_t)std::min<uint64_t>(1ull << d, 2 * m);
        };
        geo[d].bx = box(dx);
        geo[d].by = box(dy);
        geo[d].bz = box(dz);
        geo[d].n = (uint64_t)geo[d].bx * geo[d].by * geo[d].bz;
        geo[d].e = e;
    }

    Scratch sc(c);
    std::vector<unsigned long long*> size(L), start(L);
    std::vector<uint32_t*> color(L);
    std::vector<uint8_t*> flags(L);
    int r;
    for (int d = 0; d < L; ++d) {
        if ((r = sc.alloc(&size[d], geo[d].n, "xn_build_svo: sizes")) ||
            (r = sc.alloc(&start[d], geo[d].n, "xn_build_svo: starts")) ||
            (r = sc.alloc(&color[d], geo[d].n, "xn_build_svo: colours")) ||
            (r = sc.alloc(&flags[d], geo[d].n, "xn_build_svo: flags")))
            return r;
    }
    const uint64_t stat_bytes = heuristic == XN_HEUR_STD_DEV ? sizeof(SDStats) : sizeof(CDStats);
    void* stats_buf[2] = {nullptr, nullptr};
    {
        // level d writes buffer d & 1 and reads d + 1's: size each for its own levels
        uint64_t big[2] = {1, 1};
        for (int d = 0; d < L; ++d) big[d & 1] = std::max(big[d & 1], geo[d].n);
        uint8_t* p0 = nullptr;
        uint8_t* p1 = nullptr;
        if ((r = sc.alloc(&p0, big[0] * stat_bytes, "xn_build_svo: scan statistics")) ||
            (r = sc.alloc(&p1, big[1] * stat_bytes, "xn_build_svo: scan statistics")))
            return r;
        stats_buf[0] = p0;
        stats_buf[1] = p1;
    }
    unsigned int* counters = nullptr;  // [0] ambiguous count, [1] max depth
    unsigned long long* leaf_count = nullptr;
    unsigned long long* ambig_list = nullptr;
    if ((r = sc.alloc(&counters, 4, "xn_build_svo: counters")) ||
        (r = sc.alloc(&leaf_count, 1, "xn_build_svo: counters")))
        return r;
    if (heuristic == XN_HEUR_STD_DEV) {
        uint64_t big = 0;
        for (int d = 0; d < L; ++d) big = std::max(big, geo[d].n);
        if ((r = sc.alloc(&ambig_list, big, "xn_build_svo: stddev list"))) return r;
    }

    cudaError_t e = cudaSuccess;
    const unsigned T = 256;
    // ---- bottom-up
    for (int d = L - 1; d >= 0; --d) {
        UpArgs a{};
        a.g = g;
        a.cur = geo[d];
        a.child_is_voxel = d == L - 1;
        if (d < L - 1) a.child = geo[d + 1];
        a.child_stats = stats_buf[(d + 1) & 1];
        a.stats = stats_buf[d & 1];
        a.child_size = d < L - 1 ? size[d + 1] : nullptr;
        a.size = size[d];
        a.color = color[d];
        a.flags = flags[d];
        a.chan_diff = (uint32_t)(uint8_t)threshold;
        a.stddev = threshold;
        a.ambig_count = counters;
        a.ambig_list = ambig_list;
        a.lean = lean ? 1 : 0;
        if (heuristic == XN_HEUR_STD_DEV) {
            if ((e = cudaMemsetAsync(counters, 0, 4, s)) != cudaSuccess) break;
            up_level_kernel<XN_HEUR_STD_DEV><<<blocks_for(geo[d].n, T), T, 0, s>>>(a);
            unsigned int amb = 0;
            if ((e = cudaMemcpyAsync(&amb, counters, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
            if (getenv("XN_BUILD_STDDEV_SEQUENTIAL")) {
                // check mode: every in-grid decision through the reference loop
                amb = 0;
                std::vector<uint8_t> hf(geo[d].n);
                cudaMemcpy(hf.data(), flags[d], geo[d].n, cudaMemcpyDeviceToHost);
                std::vector<unsigned long long> lst;
                for (uint64_t i = 0; i < geo[d].n; ++i)
                    if (hf[i] & F_INSIDE) lst.push_back(i);
                amb = (unsigned)lst.size();
                cudaMemcpy(ambig_list, lst.data(), lst.size() * 8, cudaMemcpyHostToDevice);
            }
            if (amb) {
                stddev_fixup_kernel<<<blocks_for(amb, 64), 64, 0, s>>>(a, amb);
                resize_level_kernel<<<blocks_for(geo[d].n, T), T, 0, s>>>(a);
            }
        } else {
            up_level_kernel<XN_HEUR_CHANNEL_DIFF><<<blocks_for(geo[d].n, T), T, 0, s>>>(a);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo: bottom-up pass");
    if (sub && (e = cudaMemcpyAsync(sub->root_stats, stats_buf[0], stat_bytes, cudaMemcpyDeviceToHost, s)) !=
                   cudaSuccess)
        return cuda_fail(e, "xn_build_svo: root statistics");

    unsigned long long n_total = 0;
    if ((e = cudaMemcpyAsync(&n_total, size[0], 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "xn_build_svo");
    if (lean) {
        if (n_total == 0) return LEAN_LEAF_ROOT;
        if (n_total >= LEAF) return fail(XN_ERR_FORMAT, "xn_build_svo: more than 2^31 internal nodes");
        // ---- top-down, lean: the device layout's inner nodes only
        lean->n_inner = n_total;
        lean->n_leaves = 0;
        if ((r = c->device_alloc(reinterpret_cast<void**>(&lean->inner), n_total * 32, "xn_build_svo: inner nodes")) ||
            (r = c->device_alloc(reinterpret_cast<void**>(&lean->inner_depth), n_total * 4,
                                 "xn_build_svo: inner depths"))) {
            lean->release_layout();
            return r;
        }
        for (int d = 0; d < L && e == cudaSuccess; ++d) e = cudaMemsetAsync(start[d], 0xFF, geo[d].n * 8, s);
        const unsigned long long zero = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(start[0], &zero, 8, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 16, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(leaf_count, 0, 8, s);
        unsigned long long* counts = nullptr;  // [1]: internal nodes written
        if ((r = sc.alloc(&counts, 2, "xn_build_svo: counters"))) {
            lean->release_layout();
            return r;
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, 16, s);
        for (int d = 0; d < L && e == cudaSuccess; ++d) {
            DownArgs a{};
            a.g = g;
            a.cur = geo[d];
            a.child_is_voxel = d == L - 1;
            if (d < L - 1) a.child = geo[d + 1];
            a.depth = d;
            a.n_total = n_total;
            a.size = size[d];
            a.child_size = d < L - 1 ? size[d + 1] : nullptr;
            a.flags = flags[d];
            a.child_color = d < L - 1 ? color[d + 1] : nullptr;
            a.child_flags = d < L - 1 ? flags[d + 1] : nullptr;
            a.start = start[d];
            a.child_start = d < L - 1 ? start[d + 1] : nullptr;
            a.leaves = leaf_count;
            a.max_depth = counters + 1;
            a.existing = counts;
            lean_down_kernel<<<blocks_for(geo[d].n, T), T, 0, s>>>(a, lean->inner, lean->inner_depth);
            e = cudaGetLastError();
        }
        unsigned long long leaves = 0, hcounts[2] = {0, 0};
        unsigned int hc[2] = {0, 0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(&leaves, leaf_count, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hc, counters, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hcounts, counts, 16, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess && hcounts[1] != n_total) {
            lean->release_layout();
            return fail(XN_ERR_STATE, "xn_build_svo: %llu of %llu internal nodes written",
                        (unsigned long long)hcounts[1], (unsigned long long)n_total);
        }
        if (e != cudaSuccess) {
            lean->release_layout();
            return cuda_fail(e, "xn_build_svo: top-down pass");
        }
        stats->total_leaves = stats->unique_leaves = leaves;
        stats->total_nodes = stats->n_nodes = n_total + leaves;
        stats->depth = hc[1];
        return XN_OK;
    }
    if (n_total > 0xFFFFFFFFull)
        return fail(XN_ERR_FORMAT, "xn_build_svo: %llu nodes exceed the 32-bit node indices of the SVO format",
                    (unsigned long long)n_total);

    const bool dag = type == XN_SVO_DAG;
    unsigned long long* existing = nullptr;  // per level: existing cells, internal cells
    if ((r = sc.alloc(&existing, 2 * (uint64_t)L, "xn_build_svo: counters"))) return r;
    uint32_t* nodes = nullptr;
    uint64_t node_bytes = n_total * 40;
    if (!dag && (r = c->device_alloc(reinterpret_cast<void**>(&nodes), node_bytes, "xn_build_svo: node array")))
        return r;
    auto drop_nodes = [&]() {
        if (nodes) c->device_free(nodes, node_bytes);
        nodes = nullptr;
    };

    // ---- top-down: post-order starts (and, without DAG, the node array)
    for (int d = 0; d < L && e == cudaSuccess; ++d) e = cudaMemsetAsync(start[d], 0xFF, geo[d].n * 8, s);
    const unsigned long long zero = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(start[0], &zero, 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(leaf_count, 0, 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(existing, 0, 16 * (uint64_t)L, s);
    for (int d = 0; d < L && e == cudaSuccess; ++d) {
        DownArgs a{};
        a.g = g;
        a.cur = geo[d];
        a.child_is_voxel = d == L - 1;
        if (d < L - 1) a.child = geo[d + 1];
        a.depth = d + depth_off;
        a.n_total = n_total;
        a.size = size[d];
        a.child_size = d < L - 1 ? size[d + 1] : nullptr;
        a.color = color[d];
        a.flags = flags[d];
        a.start = start[d];
        a.child_start = d < L - 1 ? start[d + 1] : nullptr;
        a.nodes = nodes;
        a.leaves = leaf_count;
        a.max_depth = counters + 1;
        a.existing = existing + 2 * d;
        down_level_kernel<<<blocks_for(geo[d].n, T), T, 0, s>>>(a);
        e = cudaGetLastError();
    }
    // ---- ropes
    if (e == cudaSuccess && type == XN_SVO_ROPE_TREE) {
        RopeArgs ra{};
        ra.L = L;
        ra.n_total = n_total;
        ra.nodes = nodes;
        for (int d = 0; d < L; ++d) ra.lv[d] = LevelDev{geo[d], size[d], start[d], flags[d]};
        for (int d = 0; d < L && e == cudaSuccess; ++d) {
            rope_level_kernel<<<blocks_for(geo[d].n, 128), 128, 0, s>>>(ra, d);
            e = cudaGetLastError();
        }
    }
    unsigned long long leaves = 0;
    unsigned int hc[2] = {0, 0};
    std::vector<unsigned long long> hexist(2 * (size_t)L);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&leaves, leaf_count, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, counters, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hexist.data(), existing, 16 * (uint64_t)L, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        drop_nodes();
        return cuda_fail(e, "xn_build_svo: top-down pass");
    }
    stats->total_leaves = leaves;
    stats->unique_leaves = leaves;
    stats->total_nodes = n_total;
    stats->n_nodes = n_total;
    stats->depth = hc[1];

    if (dag) {
        // ---- DAG: classes depth by depth, deepest first
        std::vector<unsigned long long*> canon(L + 1);
        for (int d = 0; d <= L; ++d) {
            uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
            if ((r = sc.alloc(&canon[d], ids, "xn_build_svo: DAG classes"))) return r;
        }
        auto level_of = [&](int d) {
            DagLevel a{};
            a.depth = d;
            a.L = L;
            a.g = g;
            const int cd = d < L ? d : L - 1;
            a.geom = geo[cd];
            a.start = start[cd];
            a.size = size[cd];
            a.color = color[cd];
            a.flags = flags[cd];
            a.canon = canon[d];
            if (d < L) {
                a.child_is_voxel = d == L - 1;
                a.child_canon = canon[d + 1];
                if (d < L - 1) a.child_geom = geo[d + 1];
            }
            return a;
        };
        for (int d = L; d >= 0 && e == cudaSuccess; --d) {
            const uint64_t count = d < L ? hexist[2 * d] : 8 * hexist[2 * (L - 1) + 1];
            if (count == 0) continue;
            uint64_t tsize = 1;
            while (tsize < 2 * count) tsize <<= 1;
            Slot* table = nullptr;
            if ((r = c->device_alloc(reinterpret_cast<void**>(&table), tsize * sizeof(Slot), "xn_build_svo: DAG table")))
                return r;
            DagLevel a = level_of(d);
            const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
            e = cudaMemsetAsync(table, 0xFF, tsize * sizeof(Slot), s);
            if (e == cudaSuccess) {
                dag_insert_kernel<<<blocks_for(ids, T), T, 0, s>>>(a, table, tsize - 1, counters);
                dag_lookup_kernel<<<blocks_for(ids, T), T, 0, s>>>(a, table, tsize - 1, counters);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            c->device_free(table, tsize * sizeof(Slot));
        }
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo: DAG classes");
        uint8_t* is_rep = nullptr;
        unsigned* ins = nullptr;
        if ((r = sc.alloc(&is_rep, n_total, "xn_build_svo: DAG ranks")) ||
            (r = sc.alloc(&ins, n_total, "xn_build_svo: DAG ranks")))
            return r;
        e = cudaMemsetAsync(is_rep, 0, n_total, s);
        for (int d = L; d >= 0 && e == cudaSuccess; --d) {
            const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
            dag_mark_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), is_rep);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo: DAG ranks");
        if ((r = exclusive_scan<uint8_t>(sc, is_rep, n_total, ins, s))) return r;
        unsigned last_ins = 0;
        uint8_t last_rep = 0;
        unsigned int ovf = 0;
        e = cudaMemcpyAsync(&last_ins, ins + (n_total - 1), 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&last_rep, is_rep + (n_total - 1), 1, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&ovf, counters, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo: DAG ranks");
        if (ovf) return fail(XN_ERR_STATE, "xn_build_svo: DAG hash table overflow (0x%x)", ovf);
        const uint64_t U = (uint64_t)last_ins + last_rep;
        node_bytes = U * 40;
        if ((r = c->device_alloc(reinterpret_cast<void**>(&nodes), node_bytes, "xn_build_svo: node array"))) return r;
        if ((e = cudaMemsetAsync(leaf_count, 0, 8, s)) == cudaSuccess) {
            for (int d = L; d >= 0 && e == cudaSuccess; --d) {
                const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
                dag_write_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), ins, U, nodes, leaf_count);
                e = cudaGetLastError();
            }
        }
        unsigned long long ul = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&ul, leaf_count, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            drop_nodes();
            return cuda_fail(e, "xn_build_svo: DAG write");
        }
        stats->unique_leaves = ul;
        stats->n_nodes = U;
    }
    *d_nodes = nodes;
    *d_nodes_bytes = node_bytes;
    return XN_OK;
}

}  // namespace xn

using namespace xn;

XN_API int xn_build_svo(xn_ctx* h, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                        int heuristic, double threshold, uint32_t** nodes_out, xn_build_stats* stats) {
    if (!h || !rgba || !nodes_out || !stats) return fail(XN_ERR_ARG, "xn_build_svo: NULL argument");
    *nodes_out = nullptr;
    if (!dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_build_svo: empty grid %ux%ux%u", dx, dy, dz);
    if (type < XN_SVO_SPARSE || type > XN_SVO_ROPE_TREE) return fail(XN_ERR_ARG, "xn_build_svo: invalid type %d", type);
    if (heuristic == XN_HEUR_CHANNEL_DIFF) {
        if (!(threshold >= 0.0 && threshold <= 255.0) || threshold != (double)(int)threshold)
            return fail(XN_ERR_ARG, "xn_build_svo: --chan-diff must be an integer in 0..255");
    } else if (heuristic == XN_HEUR_STD_DEV) {
        if (!(threshold >= 0.0)) return fail(XN_ERR_ARG, "xn_build_svo: --std-dev must be >= 0");
    } else {
        return fail(XN_ERR_ARG, "xn_build_svo: invalid heuristic %d", heuristic);
    }
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    const uint64_t vbytes = (uint64_t)dx * dy * dz * 4;
    uint32_t* vox = nullptr;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&vox), vbytes, "xn_build_svo: grid"))) return r;
    cudaError_t e = cudaMemcpyAsync(vox, rgba, vbytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        c->device_free(vox, vbytes);
        return cuda_fail(e, "xn_build_svo: upload");
    }
    uint32_t* d_nodes = nullptr;
    uint64_t nbytes = 0;
    r = build_svo_device(c, vox, dx, dy, dz, type, heuristic, threshold, &d_nodes, &nbytes, stats);
    c->device_free(vox, vbytes);
    if (r) return r;
    uint32_t* host = static_cast<uint32_t*>(std::malloc(nbytes));
    if (!host) {
        c->device_free(d_nodes, nbytes);
        return fail(XN_ERR_NOMEM, "xn_build_svo: out of host memory for %llu bytes", (unsigned long long)nbytes);
    }
    e = cudaMemcpyAsync(host, d_nodes, nbytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    c->device_free(d_nodes, nbytes);
    if (e != cudaSuccess) {
        std::free(host);
        return cuda_fail(e, "xn_build_svo: download");
    }
    *nodes_out = host;
    return XN_OK;
}

XN_API int xn_build_svo_volume(xn_ctx* h, const void* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                               int heuristic, double threshold, xn_volume** out, xn_build_stats* stats) {
    if (!h || !d_rgba || !out || !stats) return fail(XN_ERR_ARG, "xn_build_svo_volume: NULL argument");
    *out = nullptr;
    if (!dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_build_svo_volume: empty grid %ux%ux%u", dx, dy, dz);
    const bool lean = (type & XN_BUILD_LEAN) != 0;
    type &= ~XN_BUILD_LEAN;
    if (type < XN_SVO_SPARSE || type > XN_SVO_ROPE_TREE)
        return fail(XN_ERR_ARG, "xn_build_svo_volume: invalid type %d", type);
    if (lean && type != XN_SVO_SPARSE)
        return fail(XN_ERR_ARG, "xn_build_svo_volume: XN_BUILD_LEAN builds sparse trees only");
    if (heuristic == XN_HEUR_CHANNEL_DIFF) {
        if (!(threshold >= 0.0 && threshold <= 255.0) || threshold != (double)(int)threshold)
            return fail(XN_ERR_ARG, "xn_build_svo_volume: --chan-diff must be an integer in 0..255");
    } else if (heuristic == XN_HEUR_STD_DEV) {
        if (!(threshold >= 0.0)) return fail(XN_ERR_ARG, "xn_build_svo_volume: --std-dev must be >= 0");
    } else {
        return fail(XN_ERR_ARG, "xn_build_svo_volume: invalid heuristic %d", heuristic);
    }
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    // a grid in host memory is copied to the device for the build
    cudaPointerAttributes pa{};
    const uint32_t* d_vox = static_cast<const uint32_t*>(d_rgba);
    void* staged = nullptr;
    const uint64_t grid_bytes = (uint64_t)dx * dy * dz * 4;
    if (cudaPointerGetAttributes(&pa, d_rgba) != cudaSuccess) cudaGetLastError();
    if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) {
        if ((r = c->device_alloc(&staged, grid_bytes, "xn_build_svo_volume: grid"))) return r;
        cudaError_t e = cudaMemcpyAsync(staged, d_rgba, grid_bytes, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) {
            c->device_free(staged, grid_bytes);
            return cuda_fail(e, "xn_build_svo_volume: grid upload");
        }
        d_vox = static_cast<const uint32_t*>(staged);
    }
    struct Staged {
        Ctx* c;
        void* p;
        uint64_t bytes;
        ~Staged() {
            if (p) {
                cudaStreamSynchronize(c->stream);
                c->device_free(p, bytes);
            }
        }
    } staged_guard{c, staged, grid_bytes};
    uint32_t* d_nodes = nullptr;
    uint64_t nbytes = 0;
    if (lean) {
        // straight into the device layout: no reference nodes, no rope records
        Volume* v = new (std::nothrow) Volume();
        if (!v) return fail(XN_ERR_NOMEM, "xn_build_svo_volume: out of host memory");
        v->ctx = c;
        r = build_svo_device(c, d_vox, dx, dy, dz, type, heuristic, threshold, &d_nodes, &nbytes, stats, v);
        if (r == XN_OK) {
            v->kind = XN_VOLUME_SVO;
            v->side = stats->side;
            v->n_nodes = stats->n_nodes;
            const uint64_t sd = stats->side > 0xFFFFFFFFull ? 0xFFFFFFFFull : stats->side;
            v->dim[0] = v->dim[1] = v->dim[2] = (uint32_t)sd;
            v->layout = XN_LAYOUT_COMPACT;
            v->depth_consistent = 1;  // written from the tree itself
            if ((r = measure_inner_depth(c, v))) {
                v->release_layout();
                delete v;
                return r;
            }
            *out = reinterpret_cast<xn_volume*>(v);
            return XN_OK;
        }
        delete v;
        if (r != LEAN_LEAF_ROOT) return r;
        // the root is a leaf: the one-node tree keeps the reference layout
    }
    r = build_svo_device(c, d_vox, dx, dy, dz, type, heuristic, threshold, &d_nodes, &nbytes, stats);
    if (r) return r;
    Volume* v = new (std::nothrow) Volume();
    if (!v) {
        c->device_free(d_nodes, nbytes);
        return fail(XN_ERR_NOMEM, "xn_build_svo_volume: out of host memory");
    }
    v->ctx = c;
    v->kind = XN_VOLUME_SVO;
    v->side = stats->side;
    v->n_nodes = stats->n_nodes;
    const uint64_t sd = stats->side > 0xFFFFFFFFull ? 0xFFFFFFFFull : stats->side;
    v->dim[0] = v->dim[1] = v->dim[2] = (uint32_t)sd;
    v->data = d_nodes;
    v->bytes = nbytes;
    v->has_ropes = type == XN_SVO_ROPE_TREE;
    if ((r = build_svo_layout(c, v))) {
        c->device_free(v->data, v->bytes);
        delete v;
        return r;
    }
    *out = reinterpret_cast<xn_volume*>(v);
    return XN_OK;
}

// ----------------------------------------------------------- streamed build ---
//
// xn_build_svo_streamed: the sparse octree of a grid that is never resident on
// the device as a whole.  The reference's node order is the reverse of a
// post-order build (OctreeConstruction.h:92-112): the root, then the subtree
// of child 7, then child 6's, ..., child 0's, each laid out the same way, with
// child indices absolute.  So the tree is the root followed by the eight
// top-level cubes' own trees (cube k at origin (k>>2 & 1, k>>1 & 1, k & 1) *
// side/2), each built alone -- the same kernels over the cube's part of the
// grid, with the cube's side and its root one level down -- and rebased by the
// number of nodes before it: one running sum over the cubes' sizes.  A cube
// outside the grid is a black leaf (OctreeConstruction.h:146-154).  The root's
// decision and colour (OctreeConstruction.h:141-181) come from the cubes' root
// statistics: sums, byte minima and maxima, or exact moments.  Ropes and DAG
// deduplication relate nodes of different cubes and are not part of it.

namespace xn {
namespace {

static_assert(sizeof(CDStats) <= sizeof(SubBuild::root_stats) && sizeof(SDStats) <= sizeof(SubBuild::root_stats),
              "root statistics fit the cube build's buffer");

__global__ void rebase_kernel(uint32_t* nodes, uint64_t n, uint32_t base) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t* p = nodes + i * 10;
        if (p[9] < LEAF)
            for (int k = 0; k < 8; ++k) p[k] += base;
    }
}

struct Out {
    std::FILE* f = nullptr;
    ~Out() {
        if (f) std::fclose(f);
    }
};

bool write_node_le(std::FILE* f, const uint32_t w[10]) {
    unsigned char b[40];
    for (int i = 0; i < 10; ++i)
        for (int k = 0; k < 4; ++k) b[4 * i + k] = (unsigned char)(w[i] >> (8 * k));
    return std::fwrite(b, 1, 40, f) == 40;
}

// Grid::stddev_scan's sequential double loop (Grid.cpp:193-203) over the whole
// grid, z-slab by z-slab through the reader: the root's decision when the
// exact moments leave it inside the rounding band.
int stddev_root_sequential(xn_region_reader read, void* user, uint32_t dx, uint32_t dy, uint32_t dz,
                           const SDStats& st, double threshold, bool* split) {
    const uint64_t n = (uint64_t)dx * dy * dz;
    const double nd = (double)n;
    double avg[4];
    for (int c = 0; c < 4; ++c) avg[c] = (double)st.s1[c] / nd;
    const uint32_t slab = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(dz, (64ull << 20) / ((uint64_t)dx * dy * 4)));
    std::vector<uint8_t> buf;
    double s = 0.0;
    for (uint32_t z0 = 0; z0 < dz; z0 += slab) {
        const uint32_t nz = std::min(slab, dz - z0);
        buf.resize((uint64_t)dx * dy * nz * 4);
        if (read(user, 0, 0, z0, dx, dy, nz, buf.data()) != 0)
            return fail(XN_ERR_IO, "xn_build_svo_streamed: the reader failed at z %u", z0);
        for (uint64_t i = 0; i < (uint64_t)dx * dy * nz; ++i) {
            const uint8_t* v = &buf[4 * i];
            const double d0 = (double)v[0] - avg[0], d1 = (double)v[1] - avg[1];
            const double d2 = (double)v[2] - avg[2], d3 = (double)v[3] - avg[3];
            s += ((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3;
        }
    }
    *split = std::sqrt(s / nd) > threshold;
    return XN_OK;
}

}  // namespace
}  // namespace xn

XN_API int xn_build_svo_streamed(xn_ctx* h, uint32_t dx, uint32_t dy, uint32_t dz, int heuristic, double threshold,
                                 xn_region_reader read, void* user, const char* out_path, xn_build_stats* stats) {
    if (!h || !read || !out_path || !stats) return fail(XN_ERR_ARG, "xn_build_svo_streamed: NULL argument");
    if (!dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_build_svo_streamed: empty grid %ux%ux%u", dx, dy, dz);
    if (heuristic == XN_HEUR_CHANNEL_DIFF) {
        if (!(threshold >= 0.0 && threshold <= 255.0) || threshold != (double)(int)threshold)
            return fail(XN_ERR_ARG, "xn_build_svo_streamed: --chan-diff must be an integer in 0..255");
    } else if (heuristic == XN_HEUR_STD_DEV) {
        if (!(threshold >= 0.0)) return fail(XN_ERR_ARG, "xn_build_svo_streamed: --std-dev must be >= 0");
    } else {
        return fail(XN_ERR_ARG, "xn_build_svo_streamed: invalid heuristic %d", heuristic);
    }
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    std::memset(stats, 0, sizeof *stats);
    const uint64_t side = std::max(ceil_pow2(dx), std::max(ceil_pow2(dy), ceil_pow2(dz)));
    stats->side = side;
    Out out;
    out.f = std::fopen(out_path, "wb");
    if (!out.f) return fail(XN_ERR_IO, "Failed to open '%s'", out_path);
    unsigned char head[24] = {'X', 'N', 'D', 'N', '-', 'S', 'V', 'O'};
    auto put_header = [&](uint64_t n) {
        for (int k = 0; k < 8; ++k) {
            head[8 + k] = (unsigned char)(side >> (8 * k));
            head[16 + k] = (unsigned char)(n >> (8 * k));
        }
        return std::fseek(out.f, 0, SEEK_SET) == 0 && std::fwrite(head, 1, 24, out.f) == 24;
    };
    if (side == 1) {  // one voxel: the root is that voxel's leaf
        uint8_t v[4];
        if (read(user, 0, 0, 0, 1, 1, 1, v) != 0) return fail(XN_ERR_IO, "xn_build_svo_streamed: the reader failed");
        const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, (uint32_t)v[0] | v[1] << 8 | v[2] << 16 | (uint32_t)v[3] << 24,
                                   LEAF};
        if (!put_header(1) || !write_node_le(out.f, node)) return fail(XN_ERR_IO, "'%s': write failed", out_path);
        stats->total_leaves = stats->unique_leaves = stats->total_nodes = stats->n_nodes = 1;
        return XN_OK;
    }
    const uint64_t S = side / 2;
    const uint32_t zero10[10] = {};
    if (!put_header(0) || !write_node_le(out.f, zero10)) return fail(XN_ERR_IO, "'%s': write failed", out_path);

    uint32_t root_ch[8] = {};
    uint64_t next = 1, leaves = 0, depth = 0, count = 0;
    unsigned long long sum[4] = {0, 0, 0, 0}, sq[4] = {0, 0, 0, 0};
    uint32_t mn = 0xFFFFFFFFu, mx = 0;
    std::vector<uint8_t> host;
    std::vector<uint32_t> chunk;
    cudaStream_t s = c->stream;
    for (int k = 7; k >= 0; --k) {
        const uint64_t ox = ((k >> 2) & 1) * S, oy = ((k >> 1) & 1) * S, oz = (k & 1) * S;
        if (next > 0xFFFFFFFFull)
            return fail(XN_ERR_FORMAT, "xn_build_svo_streamed: more than 2^32 nodes exceed the SVO format");
        root_ch[k] = (uint32_t)next;
        if (ox >= dx || oy >= dy || oz >= dz) {  // outside the grid: a black leaf one level down
            const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, LEAF | 1u};
            if (!write_node_le(out.f, node)) return fail(XN_ERR_IO, "'%s': write failed", out_path);
            next += 1;
            leaves += 1;
            depth = std::max<uint64_t>(depth, 1);
            continue;
        }
        const uint32_t sx = (uint32_t)std::min<uint64_t>(S, dx - ox), sy = (uint32_t)std::min<uint64_t>(S, dy - oy),
                       sz = (uint32_t)std::min<uint64_t>(S, dz - oz);
        const uint64_t nvox = (uint64_t)sx * sy * sz;
        try {
            host.resize(nvox * 4);
        } catch (const std::bad_alloc&) {
            return fail(XN_ERR_NOMEM, "xn_build_svo_streamed: out of host memory");
        }
        if (read(user, (uint32_t)ox, (uint32_t)oy, (uint32_t)oz, sx, sy, sz, host.data()) != 0)
            return fail(XN_ERR_IO, "xn_build_svo_streamed: the reader failed for the cube at (%llu, %llu, %llu)",
                        (unsigned long long)ox, (unsigned long long)oy, (unsigned long long)oz);
        count += nvox;
        if (S == 1) {  // the cube is one voxel: a leaf one level down
            const uint8_t* v = host.data();
            const uint32_t w = (uint32_t)v[0] | v[1] << 8 | v[2] << 16 | (uint32_t)v[3] << 24;
            const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, w, LEAF | 1u};
            if (!write_node_le(out.f, node)) return fail(XN_ERR_IO, "'%s': write failed", out_path);
            for (int ch = 0; ch < 4; ++ch) {
                sum[ch] += v[ch];
                sq[ch] += (unsigned long long)v[ch] * v[ch];
            }
            for (int b = 0; b < 4; ++b) {
                const uint32_t sh = 8 * b;
                const uint32_t lo = std::min((mn >> sh) & 0xFFu, (w >> sh) & 0xFFu);
                const uint32_t hi = std::max((mx >> sh) & 0xFFu, (w >> sh) & 0xFFu);
                mn = (mn & ~(0xFFu << sh)) | (lo << sh);
                mx = (mx & ~(0xFFu << sh)) | (hi << sh);
            }
            next += 1;
            leaves += 1;
            depth = std::max<uint64_t>(depth, 1);
            continue;
        }
        uint32_t* d_vox = nullptr;
        if ((r = c->device_alloc(reinterpret_cast<void**>(&d_vox), nvox * 4, "xn_build_svo_streamed: cube grid")))
            return r;
        cudaError_t e = cudaMemcpyAsync(d_vox, host.data(), nvox * 4, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            c->device_free(d_vox, nvox * 4);
            return cuda_fail(e, "xn_build_svo_streamed: cube upload");
        }
        SubBuild sub;
        sub.side = S;
        sub.depth_offset = 1;
        xn_build_stats st{};
        uint32_t* d_nodes = nullptr;
        uint64_t nbytes = 0;
        r = build_svo_device(c, d_vox, sx, sy, sz, XN_SVO_SPARSE, heuristic, threshold, &d_nodes, &nbytes, &st, nullptr,
                             &sub);
        c->device_free(d_vox, nvox * 4);
        if (r) return r;
        const uint64_t n = st.n_nodes;
        if (next + n > 0x100000000ull) {
            c->device_free(d_nodes, nbytes);
            return fail(XN_ERR_FORMAT, "xn_build_svo_streamed: more than 2^32 nodes exceed the SVO format");
        }
        rebase_kernel<<<1024, 256, 0, s>>>(d_nodes, n, (uint32_t)next);
        e = cudaGetLastError();
        // the cube's nodes to the file, in chunks
        const uint64_t CH = 1ull << 22;  // nodes per chunk
        for (uint64_t off = 0; off < n && e == cudaSuccess; off += CH) {
            const uint64_t take = std::min(CH, n - off);
            chunk.resize(take * 10);
            e = cudaMemcpyAsync(chunk.data(), d_nodes + off * 10, take * 40, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e == cudaSuccess) {
                for (uint64_t i = 0; i < take; ++i)
                    if (!write_node_le(out.f, &chunk[i * 10])) {
                        c->device_free(d_nodes, nbytes);
                        return fail(XN_ERR_IO, "'%s': write failed", out_path);
                    }
            }
        }
        c->device_free(d_nodes, nbytes);
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_streamed: cube nodes");
        next += n;
        leaves += st.total_leaves;
        depth = std::max<uint64_t>(depth, st.depth);
        if (heuristic == XN_HEUR_CHANNEL_DIFF) {
            CDStats cs;
            std::memcpy(&cs, sub.root_stats, sizeof cs);
            for (int ch = 0; ch < 4; ++ch) sum[ch] += cs.sum[ch];
            for (int b = 0; b < 4; ++b) {
                const uint32_t sh = 8 * b;
                const uint32_t lo = std::min((mn >> sh) & 0xFFu, (cs.mn >> sh) & 0xFFu);
                const uint32_t hi = std::max((mx >> sh) & 0xFFu, (cs.mx >> sh) & 0xFFu);
                mn = (mn & ~(0xFFu << sh)) | (lo << sh);
                mx = (mx & ~(0xFFu << sh)) | (hi << sh);
            }
        } else {
            SDStats ss;
            std::memcpy(&ss, sub.root_stats, sizeof ss);
            for (int ch = 0; ch < 4; ++ch) {
                sum[ch] += ss.s1[ch];
                sq[ch] += ss.s2[ch];
            }
        }
    }
    // the root (OctreeConstruction.h:141-181): partly outside -> split;
    // fully inside -> the heuristic on the whole grid
    const bool fully = dx == side && dy == side && dz == side;
    uint32_t avg = 0;
    bool split = true;
    if (heuristic == XN_HEUR_CHANNEL_DIFF) {
        for (int ch = 0; ch < 4; ++ch) avg |= (uint32_t)(uint8_t)(sum[ch] / count) << (8 * ch);
        uint32_t maxdiff = 0;
        for (int b = 0; b < 4; ++b) {
            const uint32_t hi = (mx >> (8 * b)) & 0xFFu, lo = (mn >> (8 * b)) & 0xFFu;
            maxdiff = std::max(maxdiff, hi > lo ? hi - lo : 0u);
        }
        split = maxdiff > (uint32_t)threshold;
    } else {
        const double nd = (double)count;
        unsigned __int128 E = 0;
        for (int ch = 0; ch < 4; ++ch) {
            avg |= (uint32_t)(uint8_t)((double)sum[ch] / nd) << (8 * ch);
            E += (unsigned __int128)count * sq[ch] - (unsigned __int128)sum[ch] * sum[ch];
        }
        if (E == 0) {
            split = 0.0 > threshold;
        } else {
            const double sd = std::sqrt((double)E / (nd * nd));
            const double band = (nd + 16.0) * 2.220446049250313e-16 * sd + 1e-300;
            split = sd > threshold;
            if (fully && std::fabs(sd - threshold) <= band) {
                SDStats all{};
                for (int ch = 0; ch < 4; ++ch) {
                    all.s1[ch] = sum[ch];
                    all.s2[ch] = sq[ch];
                }
                if ((r = stddev_root_sequential(read, user, dx, dy, dz, all, threshold, &split))) return r;
            }
        }
    }
    if (fully && !split) {  // the whole grid is one leaf
        const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, avg, LEAF};
        if (!put_header(1) || !write_node_le(out.f, node) || std::fflush(out.f) != 0 ||
            ftruncate(fileno(out.f), 64) != 0)
            return fail(XN_ERR_IO, "'%s': write failed", out_path);
        stats->total_leaves = stats->unique_leaves = stats->total_nodes = stats->n_nodes = 1;
        return XN_OK;
    }
    uint32_t root[10];
    for (int k = 0; k < 8; ++k) root[k] = root_ch[k];
    root[8] = avg;
    root[9] = 0;
    if (!put_header(next) || !write_node_le(out.f, root) || std::fflush(out.f) != 0)
        return fail(XN_ERR_IO, "'%s': write failed", out_path);
    stats->total_leaves = stats->unique_leaves = leaves;
    stats->total_nodes = stats->n_nodes = next;
    stats->depth = depth;
    return XN_OK;
}

// --------------------------------------------------- allocation-free build ---
//
// xn_build_svo_static: the octree build for callers that cannot call
// cudaMalloc -- code running inside another framework's memory pool or HBM
// budget, or host loops that must not take the device-wide synchronisation a
// cudaMalloc/cudaFree can imply.  The caller passes the grid (device memory)
// and the node buffer (device memory); all scratch comes from one fixed
// file-scope device array of XN_STATIC_SCRATCH_BYTES that every GPU loading
// this library holds until the process exits.  Calls share that array and
// leave their contents in it: whatever must start at zero is cleared by each
// call, and calls that overlap on the GPU (two streams, two threads) race.
// The same kernels as xn_build_svo run in the same order; only the source of
// scratch differs.

#define XN_STATIC_SCRATCH_BYTES (32ull << 20)

static __device__ __align__(256) unsigned char xn_static_build_scratch[XN_STATIC_SCRATCH_BYTES];

namespace xn {
namespace {

constexpr int STATIC_MAX_DEVICES = 64;
std::mutex g_static_mu;
struct StaticScratch {
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;  // the context the address belongs to (0: none yet)
};
StaticScratch g_static_scratch[STATIC_MAX_DEVICES];

// The driver's context identity, looked up through the runtime so that the
// library needs no link against the driver library.  A context that is
// destroyed and created again (cudaDeviceReset by this process, whichever
// runtime makes the call) gets a new id, so an address looked up in the old
// context is never reused.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static int looked_up = 0;  // guarded by g_static_mu
    if (!looked_up) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: driver entry points");
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return fail(XN_ERR_CUDA, "xn_build_svo_static: the driver has no cuCtxGetCurrent/cuCtxGetId");
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
        looked_up = 1;
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS) return fail(XN_ERR_CUDA, "xn_build_svo_static: cuCtxGetCurrent failed");
    *id = 0;
    if (c && get_id(c, id) != CUDA_SUCCESS) return fail(XN_ERR_CUDA, "xn_build_svo_static: cuCtxGetId failed");
    return XN_OK;
}

// Device address of the scratch array in the current device's context.  Host
// code must not use the array's name as an address: the set-up looks it up
// with cudaGetSymbolAddress, once per device and context (the first call on a
// device, and the first after that device's context was reset).
int static_scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: cudaGetDevice");
    if (dev < 0 || dev >= STATIC_MAX_DEVICES)
        return fail(XN_ERR_ARG, "xn_build_svo_static: device %d is beyond the %d supported", dev, STATIC_MAX_DEVICES);
    std::lock_guard<std::mutex> lk(g_static_mu);
    unsigned long long id = 0;
    int r = current_context_id(&id);
    if (r) return r;
    StaticScratch& s = g_static_scratch[dev];
    if (!s.ptr || id == 0 || s.ctx_id != id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, xn_static_build_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: cudaGetSymbolAddress");
        // the lookup makes the device's primary context current if none was
        if (id == 0 && (r = current_context_id(&id))) return r;
        s.ptr = p;
        s.ctx_id = id;
    }
    *out = s.ptr;
    return XN_OK;
}

// The kernels run on the caller's stream and use the scratch array of the
// current device, so the stream must belong to that device.
int check_stream_device(cudaStream_t s) {
    int dev = 0, sdev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaStreamGetDevice(s, &sdev);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: stream device");
    if (sdev != dev)
        return fail(XN_ERR_ARG, "xn_build_svo_static: the stream belongs to device %d, the current device is %d", sdev,
                    dev);
    return XN_OK;
}

// Bump allocation inside the scratch array; with base == nullptr it only
// measures.
struct Arena {
    unsigned char* base;
    uint64_t cap;
    uint64_t used = 0;
    bool overflow = false;
    template <class T>
    T* take(uint64_t count) {
        const uint64_t off = (used + 255) & ~255ull;
        const uint64_t bytes = count * sizeof(T) + 16;
        if (off > cap || bytes > cap - off) {
            overflow = true;
            used = off + bytes;
            return nullptr;
        }
        used = off + bytes;
        return base ? reinterpret_cast<T*>(base + off) : reinterpret_cast<T*>(16);
    }
};

__global__ void single_voxel_kernel(const uint32_t* vox, uint32_t* nodes) {
    for (int k = 0; k < 8; ++k) nodes[k] = 0;
    nodes[8] = vox[0];
    nodes[9] = LEAF;
}

template <class In>
int exclusive_scan_static(Arena& a, const In* in, uint64_t n, unsigned* out, cudaStream_t s) {
    const uint64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (nb <= 1) {
        scan_apply_kernel<In><<<1, SCAN_T, 0, s>>>(in, n, nullptr, out);
        return XN_OK;
    }
    unsigned* sums = a.take<unsigned>(nb);
    unsigned* offs = a.take<unsigned>(nb);
    if (a.overflow)
        return fail(XN_ERR_BUDGET, "xn_build_svo_static: the DAG ranks need more than the %llu-byte static scratch",
                    (unsigned long long)XN_STATIC_SCRATCH_BYTES);
    scan_reduce_kernel<In><<<(unsigned)nb, SCAN_T, 0, s>>>(in, n, sums);
    int r = exclusive_scan_static<unsigned>(a, sums, nb, offs, s);
    if (r) return r;
    scan_apply_kernel<In><<<(unsigned)nb, SCAN_T, 0, s>>>(in, n, offs, out);
    return XN_OK;
}

struct StaticLevels {
    unsigned long long* size[MAX_LEVELS];
    unsigned long long* start[MAX_LEVELS];
    uint32_t* color[MAX_LEVELS];
    uint8_t* flags[MAX_LEVELS];
    void* stats_buf[2];
    unsigned int* counters;
    unsigned long long* leaf_count;
    unsigned long long* existing;
    unsigned long long* ambig_list;
};

// The scratch every build needs before the node count is known.
void plan_levels(Arena& a, StaticLevels& p, const LevelGeom* geo, int L, int heuristic) {
    uint64_t big = 0;
    for (int d = 0; d < L; ++d) {
        p.size[d] = a.take<unsigned long long>(geo[d].n);
        p.start[d] = a.take<unsigned long long>(geo[d].n);
        p.color[d] = a.take<uint32_t>(geo[d].n);
        p.flags[d] = a.take<uint8_t>(geo[d].n);
        big = std::max(big, geo[d].n);
    }
    const uint64_t stat_bytes = heuristic == XN_HEUR_STD_DEV ? sizeof(SDStats) : sizeof(CDStats);
    p.stats_buf[0] = a.take<uint8_t>(big * stat_bytes);
    p.stats_buf[1] = a.take<uint8_t>(big * stat_bytes);
    p.counters = a.take<unsigned int>(4);
    p.leaf_count = a.take<unsigned long long>(1);
    p.existing = a.take<unsigned long long>(2 * (uint64_t)L);
    p.ambig_list = heuristic == XN_HEUR_STD_DEV ? a.take<unsigned long long>(big) : nullptr;
}

int build_static(const uint32_t* d_vox, uint32_t dx, uint32_t dy, uint32_t dz, int type, int heuristic,
                 double threshold, uint32_t* d_nodes, uint64_t capacity, xn_build_stats* stats, cudaStream_t s) {
    const uint64_t side = std::max(ceil_pow2(dx), std::max(ceil_pow2(dy), ceil_pow2(dz)));
    int L = 0;
    while ((1ull << L) < side) ++L;
    std::memset(stats, 0, sizeof *stats);
    stats->side = side;
    if (L >= MAX_LEVELS) return fail(XN_ERR_ARG, "xn_build_svo_static: grid too large");
    if (int rs = check_stream_device(s)) return rs;
    GridDev g{d_vox, dx, dy, dz};
    if (L == 0) {
        stats->total_leaves = stats->unique_leaves = stats->total_nodes = stats->n_nodes = 1;
        if (capacity < 1) return fail(XN_ERR_ARG, "xn_build_svo_static: the node buffer must hold 1 node");
        single_voxel_kernel<<<1, 1, 0, s>>>(d_vox, d_nodes);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e == cudaSuccess ? XN_OK : cuda_fail(e, "xn_build_svo_static");
    }
    LevelGeom geo[MAX_LEVELS];
    for (int d = 0; d < L; ++d) {
        const uint64_t e = side >> d;
        auto box = [&](uint64_t dim) -> uint32_t {
            if (d == 0) return 1;
            const uint64_t pe = e * 2;
            return (uint32_t)std::min<uint64_t>(1ull << d, 2 * ((dim + pe - 1) / pe));
        };
        geo[d].bx = box(dx);
        geo[d].by = box(dy);
        geo[d].bz = box(dz);
        geo[d].n = (uint64_t)geo[d].bx * geo[d].by * geo[d].bz;
        geo[d].e = e;
    }
    // size check before anything touches the device
    StaticLevels p{};
    Arena measure{nullptr, ~0ull};
    plan_levels(measure, p, geo, L, heuristic);
    if (measure.used > XN_STATIC_SCRATCH_BYTES)
        return fail(XN_ERR_BUDGET,
                    "xn_build_svo_static: a %ux%ux%u grid needs %llu bytes of build scratch; the static scratch "
                    "holds %llu (use xn_build_svo)",
                    dx, dy, dz, (unsigned long long)measure.used, (unsigned long long)XN_STATIC_SCRATCH_BYTES);
    void* base = nullptr;
    int r = static_scratch_address(&base);
    if (r) return r;
    Arena a{static_cast<unsigned char*>(base), XN_STATIC_SCRATCH_BYTES};
    plan_levels(a, p, geo, L, heuristic);

    cudaError_t e = cudaSuccess;
    const unsigned T = 256;
    for (int d = L - 1; d >= 0 && e == cudaSuccess; --d) {
        UpArgs u{};
        u.g = g;
        u.cur = geo[d];
        u.child_is_voxel = d == L - 1;
        if (d < L - 1) u.child = geo[d + 1];
        u.child_stats = p.stats_buf[(d + 1) & 1];
        u.stats = p.stats_buf[d & 1];
        u.child_size = d < L - 1 ? p.size[d + 1] : nullptr;
        u.size = p.size[d];
        u.color = p.color[d];
        u.flags = p.flags[d];
        u.chan_diff = (uint32_t)(uint8_t)threshold;
        u.stddev = threshold;
        u.ambig_count = p.counters;
        u.ambig_list = p.ambig_list;
        if (heuristic == XN_HEUR_STD_DEV) {
            unsigned int amb = 0;
            e = cudaMemsetAsync(p.counters, 0, 4, s);
            if (e != cudaSuccess) break;
            up_level_kernel<XN_HEUR_STD_DEV><<<blocks_for(geo[d].n, T), T, 0, s>>>(u);
            if ((e = cudaMemcpyAsync(&amb, p.counters, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
            if (amb) {
                stddev_fixup_kernel<<<blocks_for(amb, 64), 64, 0, s>>>(u, amb);
                resize_level_kernel<<<blocks_for(geo[d].n, T), T, 0, s>>>(u);
            }
        } else {
            up_level_kernel<XN_HEUR_CHANNEL_DIFF><<<blocks_for(geo[d].n, T), T, 0, s>>>(u);
        }
        e = cudaGetLastError();
    }
    unsigned long long n_total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n_total, p.size[0], 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: bottom-up pass");
    if (n_total > 0xFFFFFFFFull) return fail(XN_ERR_FORMAT, "xn_build_svo_static: more than 2^32 nodes");
    const bool dag = type == XN_SVO_DAG;
    stats->n_nodes = n_total;
    if (!dag && n_total > capacity)
        return fail(XN_ERR_ARG, "xn_build_svo_static: the octree has %llu nodes; the node buffer holds %llu",
                    (unsigned long long)n_total, (unsigned long long)capacity);

    for (int d = 0; d < L && e == cudaSuccess; ++d) e = cudaMemsetAsync(p.start[d], 0xFF, geo[d].n * 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.start[0], 0, 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.counters, 0, 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.leaf_count, 0, 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.existing, 0, 16 * (uint64_t)L, s);
    for (int d = 0; d < L && e == cudaSuccess; ++d) {
        DownArgs w{};
        w.g = g;
        w.cur = geo[d];
        w.child_is_voxel = d == L - 1;
        if (d < L - 1) w.child = geo[d + 1];
        w.depth = d;
        w.n_total = n_total;
        w.size = p.size[d];
        w.child_size = d < L - 1 ? p.size[d + 1] : nullptr;
        w.color = p.color[d];
        w.flags = p.flags[d];
        w.start = p.start[d];
        w.child_start = d < L - 1 ? p.start[d + 1] : nullptr;
        w.nodes = dag ? nullptr : d_nodes;
        w.leaves = p.leaf_count;
        w.max_depth = p.counters + 1;
        w.existing = p.existing + 2 * d;
        down_level_kernel<<<blocks_for(geo[d].n, T), T, 0, s>>>(w);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && type == XN_SVO_ROPE_TREE) {
        RopeArgs ra{};
        ra.L = L;
        ra.n_total = n_total;
        ra.nodes = d_nodes;
        for (int d = 0; d < L; ++d) ra.lv[d] = LevelDev{geo[d], p.size[d], p.start[d], p.flags[d]};
        for (int d = 0; d < L && e == cudaSuccess; ++d) {
            rope_level_kernel<<<blocks_for(geo[d].n, 128), 128, 0, s>>>(ra, d);
            e = cudaGetLastError();
        }
    }
    unsigned long long leaves = 0;
    unsigned int hc[2] = {0, 0};
    unsigned long long hexist[2 * MAX_LEVELS];
    if (e == cudaSuccess) e = cudaMemcpyAsync(&leaves, p.leaf_count, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, p.counters, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hexist, p.existing, 16 * (uint64_t)L, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: top-down pass");
    stats->total_leaves = leaves;
    stats->unique_leaves = leaves;
    stats->total_nodes = n_total;
    stats->depth = hc[1];
    if (!dag) return XN_OK;

    // DAG classes, ranks and nodes, with the same kernels as xn_build_svo
    unsigned long long* canon[MAX_LEVELS + 1];
    uint64_t tsize_max = 1;
    for (int d = 0; d <= L; ++d) {
        const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
        canon[d] = a.take<unsigned long long>(ids);
        const uint64_t count = d < L ? hexist[2 * d] : 8 * hexist[2 * (L - 1) + 1];
        uint64_t ts = 1;
        while (ts < 2 * count) ts <<= 1;
        tsize_max = std::max(tsize_max, ts);
    }
    Slot* table = a.take<Slot>(tsize_max);
    uint8_t* is_rep = a.take<uint8_t>(n_total);
    unsigned* ins = a.take<unsigned>(n_total);
    if (a.overflow)
        return fail(XN_ERR_BUDGET,
                    "xn_build_svo_static: the DAG of this %ux%ux%u grid needs more than the %llu-byte static scratch "
                    "(use xn_build_svo)",
                    dx, dy, dz, (unsigned long long)XN_STATIC_SCRATCH_BYTES);
    auto level_of = [&](int d) {
        DagLevel q{};
        q.depth = d;
        q.L = L;
        q.g = g;
        const int cd = d < L ? d : L - 1;
        q.geom = geo[cd];
        q.start = p.start[cd];
        q.size = p.size[cd];
        q.color = p.color[cd];
        q.flags = p.flags[cd];
        q.canon = canon[d];
        if (d < L) {
            q.child_is_voxel = d == L - 1;
            q.child_canon = canon[d + 1];
            if (d < L - 1) q.child_geom = geo[d + 1];
        }
        return q;
    };
    for (int d = L; d >= 0 && e == cudaSuccess; --d) {
        const uint64_t count = d < L ? hexist[2 * d] : 8 * hexist[2 * (L - 1) + 1];
        if (count == 0) continue;
        uint64_t ts = 1;
        while (ts < 2 * count) ts <<= 1;
        const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
        e = cudaMemsetAsync(table, 0xFF, ts * sizeof(Slot), s);
        if (e != cudaSuccess) break;
        dag_insert_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), table, ts - 1, p.counters);
        dag_lookup_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), table, ts - 1, p.counters);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(is_rep, 0, n_total, s);
    for (int d = L; d >= 0 && e == cudaSuccess; --d) {
        const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
        dag_mark_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), is_rep);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: DAG classes");
    if ((r = exclusive_scan_static<uint8_t>(a, is_rep, n_total, ins, s))) return r;
    unsigned last_ins = 0;
    uint8_t last_rep = 0;
    unsigned int ovf = 0;
    e = cudaMemcpyAsync(&last_ins, ins + (n_total - 1), 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last_rep, is_rep + (n_total - 1), 1, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ovf, p.counters, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: DAG ranks");
    if (ovf) return fail(XN_ERR_STATE, "xn_build_svo_static: DAG hash table overflow (0x%x)", ovf);
    const uint64_t U = (uint64_t)last_ins + last_rep;
    stats->n_nodes = U;
    if (U > capacity)
        return fail(XN_ERR_ARG, "xn_build_svo_static: the DAG has %llu nodes; the node buffer holds %llu",
                    (unsigned long long)U, (unsigned long long)capacity);
    e = cudaMemsetAsync(p.leaf_count, 0, 8, s);
    for (int d = L; d >= 0 && e == cudaSuccess; --d) {
        const uint64_t ids = d < L ? geo[d].n : 8 * geo[L - 1].n;
        dag_write_kernel<<<blocks_for(ids, T), T, 0, s>>>(level_of(d), ins, U, d_nodes, p.leaf_count);
        e = cudaGetLastError();
    }
    unsigned long long ul = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ul, p.leaf_count, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "xn_build_svo_static: DAG write");
    stats->unique_leaves = ul;
    return XN_OK;
}

}  // namespace
}  // namespace xn

XN_API int xn_build_svo_static(const uint32_t* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                               int heuristic, double threshold, uint32_t* d_nodes, uint64_t node_capacity,
                               xn_build_stats* stats, void* stream) {
    if (!d_rgba || !d_nodes || !stats) return fail(XN_ERR_ARG, "xn_build_svo_static: NULL argument");
    if (!dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_build_svo_static: empty grid %ux%ux%u", dx, dy, dz);
    if (type < XN_SVO_SPARSE || type > XN_SVO_ROPE_TREE)
        return fail(XN_ERR_ARG, "xn_build_svo_static: invalid type %d", type);
    if (heuristic == XN_HEUR_CHANNEL_DIFF) {
        if (!(threshold >= 0.0 && threshold <= 255.0) || threshold != (double)(int)threshold)
            return fail(XN_ERR_ARG, "xn_build_svo_static: --chan-diff must be an integer in 0..255");
    } else if (heuristic == XN_HEUR_STD_DEV) {
        if (!(threshold >= 0.0)) return fail(XN_ERR_ARG, "xn_build_svo_static: --std-dev must be >= 0");
    } else {
        return fail(XN_ERR_ARG, "xn_build_svo_static: invalid heuristic %d", heuristic);
    }
    if ((reinterpret_cast<uintptr_t>(d_rgba) & 3) || (reinterpret_cast<uintptr_t>(d_nodes) & 7))
        return fail(XN_ERR_ARG, "xn_build_svo_static: the grid must be 4-byte and the node buffer 8-byte aligned");
    return xn::build_static(d_rgba, dx, dy, dz, type, heuristic, threshold, d_nodes, node_capacity, stats,
                            static_cast<cudaStream_t>(stream));
}
