// Traversal kernels: the five reference shaders as sm_103a CUDA.
//
//   DDA        resources/dda.comp:13-73
//   svo-naive  resources/svo_naive.comp:8-89
//   svo-df     resources/svo_df.comp:6-85
//   esvo       resources/esvo.comp:10-157
//   svo-rope   resources/svo_rope.comp:8-153
//
// One thread traces one primary ray.  A warp owns an 8x4 pixel tile so that
// neighbouring rays stay coherent; a block is 16x8 pixels (4 warps).  Every
// loop the shaders leave unbounded carries an iteration cap; a ray that hits
// it (where the shader would not terminate) raises a bit in the context's
// error word instead of hanging the GPU.
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

#include "xn_device.cuh"
#include "xn_internal.h"

namespace xn {

constexpr uint32_t LEAF_MASK = 0x80000000u;
constexpr uint32_t DEPTH_MASK = 0x7FFFFFFFu;
constexpr uint32_t SVO_MAX_ITER = 1u << 22;
constexpr int FIND_MAX_DEPTH = 64;
constexpr int STACK_DEPTH = 23;  // FLOAT_MANTISSA_BITS, resources/common.glsl:37

struct Outputs {
    uint32_t* rgba;      // packed RGBA8, row pitch out_w
    float* emission;     // 3 floats per pixel, or null
    uint32_t* loads;     // reference word reads per ray, or null
    uint32_t* err_word;  // error bits (atomicOr)
};

// ----------------------------------------------------------------- grid ---

struct GridVol {
    const uchar4* texels;  // x fastest
    uint32_t dx, dy, dz;
    uint64_t sy, sz;       // element strides of y and z
};

__device__ __forceinline__ V3 fetch_texel(const GridVol& g, int x, int y, int z) {
    if ((uint32_t)x >= g.dx || (uint32_t)y >= g.dy || (uint32_t)z >= g.dz) return vs(0.0f);
    uchar4 t = __ldg(g.texels + (uint64_t)(uint32_t)x + (uint64_t)(uint32_t)y * g.sy + (uint64_t)(uint32_t)z * g.sz);
    return V3{unorm8(t.x), unorm8(t.y), unorm8(t.z)};
}

// resources/dda.comp:13-53
template <bool COUNT>
__device__ V3 trace_dda(const GridVol& g, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    V3 box_min = -bias;
    V3 md = v3((float)g.dx, (float)g.dy, (float)g.dz);
    V3 box_max = md * rrd - bias;
    float t_min = max_elem(vmin(box_min, box_max));
    float t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs(0.0f);
    t_min = fmaxf(t_min, 0.0f);
    ro = ro + rd * t_min;
    int px = f2i(ro.x), py = f2i(ro.y), pz = f2i(ro.z);
    V3 t_delta = v3(fabsf(rrd.x), fabsf(rrd.y), fabsf(rrd.z));
    V3 sgn = v3(gl_sign(rd.x), gl_sign(rd.y), gl_sign(rd.z));
    int sx = (int)sgn.x, sy = (int)sgn.y, sz = (int)sgn.z;
    V3 fr = (v3(floorf(ro.x), floorf(ro.y), floorf(ro.z)) - ro) + vs(0.5f);
    V3 side = (sgn * fr + vs(0.5f)) * t_delta;
    float t = 0.0f;
    V3 total = vs(0.0f);
    const float lim = t_max - t_min;
    const uint32_t cap = 2u * (g.dx + g.dy + g.dz) + 64u;
    uint32_t iter = 0;
    while (t < lim) {
        if (++iter > cap) { err |= 1u; break; }
        // lessThanEqual(side, min(side.yzx, side.zxy)) is side.k == min of
        // all three (the sides are finite and positive)
        float t0 = min_elem(side);
        bool mx = side.x == t0;
        bool my = side.y == t0;
        bool mz = side.z == t0;
        V3 tx = fetch_texel(g, px, py, pz);
        if (COUNT) ++loads;
        float dt = t0 - t;
        total = total + tx * dt;
        t = t0;
        if (mx) { side.x = side.x + t_delta.x; px += sx; }
        if (my) { side.y = side.y + t_delta.y; py += sy; }
        if (mz) { side.z = side.z + t_delta.z; pz += sz; }
    }
    return total;
}

// Texture form of the grid: a 3D cudaArray (block-linear, so texels that
// are near in 3D share cache lines) sampled with point filtering and a zero
// border, which makes out-of-range reads 0 without a bounds check and leaves
// the address arithmetic to the texture unit.  NORM: the unit returns
// byte/255 (used when that conversion is exact, see xn_volume_upload_grid);
// otherwise the raw bytes are converted with unorm8.
// UNORM8 -> float of leaf colours from a 256-entry table in shared memory,
// filled with unorm8 itself (the same bits) by every octree kernel before its
// first leaf: two instructions per channel instead of five.
__shared__ float s_unorm_lut[256];

__device__ __forceinline__ void fill_unorm_lut() {
    for (uint32_t i = threadIdx.x; i < 256u; i += blockDim.x) s_unorm_lut[i] = unorm8(i);
    __syncthreads();
}

__device__ __forceinline__ V3 leaf_rgb(uint32_t col) {
    return V3{s_unorm_lut[col & 0xFFu], s_unorm_lut[(col >> 8) & 0xFFu], s_unorm_lut[(col >> 16) & 0xFFu]};
}

// Texel reads of the three texture forms (TEX_*): the texture unit returns
// byte/255 as four floats; or four bytes, converted through the shared
// table (the kernel fills it); or one 32-bit word of four bytes (a
// one-channel texture over the same bytes: one register returned per lane
// instead of four), converted in registers.
constexpr int TEX_RAW = 0, TEX_NORM = 1, TEX_PACKED = 2;
template <int MODE>
__device__ __forceinline__ V3 tex_texel(cudaTextureObject_t t, float x, float y, float z) {
    if (MODE == TEX_NORM) {
        float4 v = tex3D<float4>(t, x, y, z);
        return V3{v.x, v.y, v.z};
    }
    if (MODE == TEX_PACKED) return unpack_rgb_bits(tex3D<unsigned int>(t, x, y, z));
    uchar4 v = tex3D<uchar4>(t, x, y, z);
    return V3{s_unorm_lut[v.x], s_unorm_lut[v.y], s_unorm_lut[v.z]};
}

// resources/dda.comp:13-53 over the texture form; coordinates are kept as
// texel centres (integers + 0.5, exact in float).
template <bool COUNT, int NORM>
__device__ V3 trace_dda_tex(cudaTextureObject_t tex, uint32_t dx, uint32_t dy, uint32_t dz, V3 ro, V3 rd,
                            uint32_t& loads, uint32_t& err) {
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    V3 box_min = -bias;
    V3 md = v3((float)dx, (float)dy, (float)dz);
    V3 box_max = md * rrd - bias;
    float t_min = max_elem(vmin(box_min, box_max));
    float t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs(0.0f);
    t_min = fmaxf(t_min, 0.0f);
    ro = ro + rd * t_min;
    float px = (float)f2i(ro.x) + 0.5f, py = (float)f2i(ro.y) + 0.5f, pz = (float)f2i(ro.z) + 0.5f;
    V3 t_delta = v3(fabsf(rrd.x), fabsf(rrd.y), fabsf(rrd.z));
    V3 sgn = v3(gl_sign(rd.x), gl_sign(rd.y), gl_sign(rd.z));
    V3 fr = (v3(floorf(ro.x), floorf(ro.y), floorf(ro.z)) - ro) + vs(0.5f);
    V3 side = (sgn * fr + vs(0.5f)) * t_delta;
    float t = 0.0f;
    V3 total = vs(0.0f);
    const float lim = t_max - t_min;
    const uint32_t cap = 2u * (dx + dy + dz) + 64u;
    uint32_t iter = 0;
    // The texel of the next step does not depend on this one's value: fetch
    // it before accumulating the current one so the texture latency overlaps
    // the step arithmetic.  The fetch after the last step reads a texel the
    // sum never uses (in range or the zero border).
    V3 tx = tex_texel<NORM>(tex, px, py, pz);
    while (t < lim) {
        if (++iter > cap) { err |= 1u; break; }
        if (COUNT) ++loads;
        // lessThanEqual(side, min(side.yzx, side.zxy)) is side.k == min of
        // all three (the sides are finite and positive)
        const float t0 = min3f(side.x, side.y, side.z);
        if (side.x == t0) { side.x = side.x + t_delta.x; px += sgn.x; }
        if (side.y == t0) { side.y = side.y + t_delta.y; py += sgn.y; }
        if (side.z == t0) { side.z = side.z + t_delta.z; pz += sgn.z; }
        const V3 next = tex_texel<NORM>(tex, px, py, pz);
        total = total + tx * (t0 - t);
        t = t0;
        tx = next;
    }
    return total;
}

// Bricked form of the grid: 8x8x8-texel bricks (2 KB), x-fastest over a brick
// grid with one brick of zeros on every side; within a brick, 16-byte groups
// of 2x2x1 texels ordered (x, y, z pair bits, then the rest) so that a 32-byte
// sector holds 2x2x2 texels and a 128-byte line 4x4x2.  A ray keeps the group
// it is in (four texels, one 16-byte load) while its steps stay inside it.
// The padding makes every read the loop can make -- one cell past the box on
// a tie, and the fetch one step ahead -- land on zeros, like the texture's
// border, without a bounds check.
struct BrickGrid {
    const uint4* groups;
    uint32_t dx, dy, dz;
    uint32_t nbx, nby;  // bricks per row and per column of the padded brick grid
};

constexpr int BRICK_PAD = 8;  // texels of zeros before the grid on each axis

__host__ __device__ __forceinline__ uint32_t bricks_along(uint32_t d) { return (d + 7) / 8 + 2; }

uint64_t brick_grid_bytes(uint32_t dx, uint32_t dy, uint32_t dz) {
    return (uint64_t)bricks_along(dx) * bricks_along(dy) * bricks_along(dz) * 2048ull;
}

// 16-byte group holding padded texel (qx, qy, qz)
__device__ __forceinline__ uint64_t brick_group(uint32_t nbx, uint32_t nby, uint32_t qx, uint32_t qy, uint32_t qz) {
    const uint64_t brick = ((uint64_t)(qz >> 3) * nby + (qy >> 3)) * nbx + (qx >> 3);
    const uint32_t in = ((qx >> 1) & 1) | (((qy >> 1) & 1) << 1) | ((qz & 1) << 2) | (((qx >> 2) & 1) << 3) |
                        (((qy >> 2) & 1) << 4) | (((qz >> 1) & 3) << 5);
    return (brick << 7) | in;
}

__global__ void brick_grid_kernel(const uint32_t* src, uint32_t dx, uint32_t dy, uint32_t dz, uint32_t* dst,
                                  uint32_t nbx, uint32_t nby) {
    const uint64_t n = (uint64_t)dx * dy * dz;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t x = (uint32_t)(i % dx);
        const uint64_t r = i / dx;
        const uint32_t y = (uint32_t)(r % dy), z = (uint32_t)(r / dy);
        const uint32_t qx = x + BRICK_PAD, qy = y + BRICK_PAD, qz = z + BRICK_PAD;
        dst[brick_group(nbx, nby, qx, qy, qz) * 4 + (qx & 1) + 2 * (qy & 1)] = src[i];
    }
}

cudaError_t brick_grid(const uint32_t* src, uint32_t dx, uint32_t dy, uint32_t dz, void* bricks, cudaStream_t s) {
    brick_grid_kernel<<<2048, 256, 0, s>>>(src, dx, dy, dz, static_cast<uint32_t*>(bricks), bricks_along(dx),
                                           bricks_along(dy));
    return cudaGetLastError();
}

// resources/dda.comp:13-53 over the bricked grid; the arithmetic of
// trace_dda_tex, with the texel taken from the ray's current 16-byte group
// (loaded again only when a step leaves it) and converted through the
// shared UNORM8 table.
template <bool COUNT>
__device__ V3 trace_dda_brick(const BrickGrid& g, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    V3 box_min = -bias;
    V3 md = v3((float)g.dx, (float)g.dy, (float)g.dz);
    V3 box_max = md * rrd - bias;
    float t_min = max_elem(vmin(box_min, box_max));
    float t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs(0.0f);
    t_min = fmaxf(t_min, 0.0f);
    ro = ro + rd * t_min;
    int px = f2i(ro.x), py = f2i(ro.y), pz = f2i(ro.z);
    V3 t_delta = v3(fabsf(rrd.x), fabsf(rrd.y), fabsf(rrd.z));
    V3 sgn = v3(gl_sign(rd.x), gl_sign(rd.y), gl_sign(rd.z));
    const int sx = (int)sgn.x, sy = (int)sgn.y, sz = (int)sgn.z;
    V3 fr = (v3(floorf(ro.x), floorf(ro.y), floorf(ro.z)) - ro) + vs(0.5f);
    V3 side = (sgn * fr + vs(0.5f)) * t_delta;
    float t = 0.0f;
    V3 total = vs(0.0f);
    const float lim = t_max - t_min;
    const uint32_t cap = 2u * (g.dx + g.dy + g.dz) + 64u;
    uint32_t iter = 0;
    uint64_t key = ~0ull;
    uint4 grp = make_uint4(0, 0, 0, 0);
    auto texel = [&](int x, int y, int z) -> V3 {
        // the padding covers every cell the loop reaches; the clamp only
        // guards rays that ran into the iteration cap
        const uint32_t qx = (uint32_t)min(max(x + BRICK_PAD, 0), (int)g.dx + 2 * BRICK_PAD - 1);
        const uint32_t qy = (uint32_t)min(max(y + BRICK_PAD, 0), (int)g.dy + 2 * BRICK_PAD - 1);
        const uint32_t qz = (uint32_t)min(max(z + BRICK_PAD, 0), (int)g.dz + 2 * BRICK_PAD - 1);
        const uint64_t k = brick_group(g.nbx, g.nby, qx, qy, qz);
        if (k != key) {
            grp = __ldg(g.groups + k);
            key = k;
        }
        const uint32_t lo = (qx & 1) ? grp.y : grp.x, hi = (qx & 1) ? grp.w : grp.z;
        const uint32_t w = (qy & 1) ? hi : lo;
        return V3{s_unorm_lut[w & 0xFFu], s_unorm_lut[(w >> 8) & 0xFFu], s_unorm_lut[(w >> 16) & 0xFFu]};
    };
    V3 tx = texel(px, py, pz);
    while (t < lim) {
        if (++iter > cap) { err |= 1u; break; }
        if (COUNT) ++loads;
        const float t0 = min3f(side.x, side.y, side.z);
        if (side.x == t0) { side.x = side.x + t_delta.x; px += sx; }
        if (side.y == t0) { side.y = side.y + t_delta.y; py += sy; }
        if (side.z == t0) { side.z = side.z + t_delta.z; pz += sz; }
        const V3 next = texel(px, py, pz);
        total = total + tx * (t0 - t);
        t = t0;
        tx = next;
    }
    return total;
}

// --------------------------------------------------------------- octree ---

// Reference node layout on the device: 10 u32 words per node
// (resources/octree.glsl:6-10).  Node handles are node indices.
struct RefNodes {
    const uint32_t* w;
    __device__ __forceinline__ uint32_t root() const { return 0; }
    __device__ __forceinline__ bool is_leaf(uint32_t n) const { return __ldg(w + (uint64_t)n * 10 + 9) >= LEAF_MASK; }
    __device__ __forceinline__ uint32_t child(uint32_t n, uint32_t k) const { return __ldg(w + (uint64_t)n * 10 + k); }
    __device__ __forceinline__ uint32_t color(uint32_t n) const { return __ldg(w + (uint64_t)n * 10 + 8); }
    __device__ __forceinline__ uint32_t depth(uint32_t n) const { return __ldg(w + (uint64_t)n * 10 + 9) & DEPTH_MASK; }
    __device__ __forceinline__ uint32_t exit_word() const { return 0; }
};

// Compact layout (svo_layout.cu) for svo-naive, svo-df and esvo: handles are
// child words; a leaf word carries the leaf's RGB.
struct CompactNodes {
    const uint32_t* inner;
    const uint32_t* depth_of;
    __device__ __forceinline__ uint32_t root() const { return 0; }
    __device__ __forceinline__ bool is_leaf(uint32_t r) const { return r >= LEAF_MASK; }
    __device__ __forceinline__ uint32_t child(uint32_t r, uint32_t k) const { return __ldg(inner + (uint64_t)r * 8 + k); }
    __device__ __forceinline__ uint32_t color(uint32_t r) const { return r & 0xFFFFFFu; }
    __device__ __forceinline__ uint32_t depth(uint32_t r) const { return __ldg(depth_of + r) & DEPTH_MASK; }
    __device__ __forceinline__ uint32_t exit_word() const { return 0; }
};

// Compact layout for svo-rope: a leaf word carries the index of the leaf's
// record (colour, six ropes, is_leaf_depth); the children of a leaf are its ropes.
struct RopeNodes {
    const uint32_t* inner;
    const uint32_t* depth_of;
    const uint32_t* leaves;
    __device__ __forceinline__ uint32_t root() const { return 0; }
    __device__ __forceinline__ bool is_leaf(uint32_t r) const { return r >= LEAF_MASK; }
    __device__ __forceinline__ uint32_t child(uint32_t r, uint32_t k) const {
        return r >= LEAF_MASK ? __ldg(leaves + (uint64_t)(r & DEPTH_MASK) * 8 + 1 + k) : __ldg(inner + (uint64_t)r * 8 + k);
    }
    __device__ __forceinline__ uint32_t color(uint32_t r) const { return __ldg(leaves + (uint64_t)(r & DEPTH_MASK) * 8); }
    __device__ __forceinline__ uint32_t depth(uint32_t r) const {
        return (r >= LEAF_MASK ? __ldg(leaves + (uint64_t)(r & DEPTH_MASK) * 8 + 7) : __ldg(depth_of + r)) & DEPTH_MASK;
    }
    __device__ __forceinline__ uint32_t exit_word() const { return ROPE_EXIT; }
};

// resources/svo_naive.comp:8-27 (identical to svo_rope.comp:8-27); reads per
// level: is_leaf_depth + children[child]; then is_leaf_depth of the leaf.
template <bool COUNT, class Acc>
__device__ __forceinline__ uint32_t find(const Acc& a, V3 pos, V3& base, float& side, uint32_t& loads,
                                         uint32_t& err) {
    float extent = 1.0f;
    uint32_t index = a.root();
    V3 offset = vs(0.0f);
    for (int level = 0;; ++level) {
        if (COUNT) ++loads;
        if (a.is_leaf(index)) {
            base = offset;
            side = extent;
            return index;
        }
        if (level >= FIND_MAX_DEPTH) { err |= 1u; base = offset; side = extent; return index; }
        extent *= 0.5f;
        V3 oe = offset + vs(extent);
        bool mx = pos.x >= oe.x, my = pos.y >= oe.y, mz = pos.z >= oe.z;
        uint32_t child = (mx ? 4u : 0u) | (my ? 2u : 0u) | (mz ? 1u : 0u);
        offset = offset + v3(mx ? 1.0f : 0.0f, my ? 1.0f : 0.0f, mz ? 1.0f : 0.0f) * vs(extent);
        index = a.child(index, child);
        if (COUNT) ++loads;
    }
}

// find() resumed from the previous step's path.  find(p) depends only on p:
// the descent from the root reaches node A at depth j exactly when p lies in
// A's capture region, per axis [O_A, O_A + 2^-j) with a bound replaced by
// -inf/+inf where it is the root's (O_A == 0 / O_A + 2^-j == 1), O_A being
// A's origin, which the root descent computes exactly (dyadic sums).  So the
// descent can restart at the deepest node of the last path whose region holds
// p, with the same offsets and extents, and reach the same leaf with the same
// base and side.  The reference's word reads are still 2 per level + 1.
// The descent path of the last find: its nodes below the root (levels 1 ..
// FIX_DEPTH, in local memory or a column of shared memory) and the scalars,
// kept apart so that the scalars can stay in registers.
constexpr int FIX_BITS = 30;
constexpr int FIX_DEPTH = 24;

struct LocalPath {
    uint32_t n[FIX_DEPTH];
    __device__ __forceinline__ uint32_t& node(int level) { return n[level - 1]; }
};
struct SharedPath {
    uint32_t* base;  // this thread's column
    uint32_t stride;
    __device__ __forceinline__ uint32_t& node(int level) { return base[(level - 1) * stride]; }
};
struct FindPath {
    int depth = -1;          // depth of the last leaf found, -1: none (or too deep to cache)
    uint32_t cx, cy, cz;     // the last leaf's origin in units of 2^-FIX_BITS
};

// Positions in fixed point: a coordinate p becomes clamp(floor(p * 2^30), 0,
// 2^30 - 1).  For a node at depth j <= 24 with origin O (a multiple of 2^-j),
// "p >= O + 2^-(j+1)" (the reference's descent test) is bit 29-j of that
// integer, and the capture region of the node (its box, with a bound at
// -inf/+inf where it is the root's) holds p exactly when the top j bits of
// the integer equal O's: the clamp supplies the open bounds.  Origins and
// extents of depth <= 24 are exact floats either way.

__device__ __forceinline__ uint32_t fix_coord(float p) {
    // floor(p * 2^30) (the scaling is exact); the unsigned conversion
    // saturates (negative values to 0) and the clamp then gives the open
    // bounds of the border cells
    const uint32_t v = __float2uint_rd(p * 1073741824.0f);
    return min(v, (1u << FIX_BITS) - 1u);
}

__device__ __forceinline__ float fix_to_float(uint32_t v) { return (float)v * (1.0f / 1073741824.0f); }

template <bool COUNT, class Acc, class Path>
__device__ __forceinline__ uint32_t find_cached(const Acc& a, FindPath& path, Path& pn, V3 pos, V3& base,
                                                float& side, uint32_t& loads, uint32_t& err) {
    const uint32_t px = fix_coord(pos.x), py = fix_coord(pos.y), pz = fix_coord(pos.z);
    int level = 0;
    uint32_t index = a.root();
    if (path.depth > 0) {
        // the deepest level of the last path whose capture region holds p:
        // the number of leading bits p shares with the last leaf's origin
        const uint32_t diff = (px ^ path.cx) | (py ^ path.cy) | (pz ^ path.cz);
        int j = diff ? __clz(diff) - (32 - FIX_BITS) : FIX_BITS;
        if (j > path.depth) j = path.depth;
        if (j >= 1) {
            level = j;
            index = pn.node(j);
        }
    }
    // the path's levels up to the resumed one are already in place
    for (;; ++level) {
        if (a.is_leaf(index) || level == FIX_DEPTH) break;
        const int b = FIX_BITS - 1 - level;
        const uint32_t k = (((px >> b) & 1u) << 2) | (((py >> b) & 1u) << 1) | ((pz >> b) & 1u);
        index = a.child(index, k);
        pn.node(level + 1) = index;
    }
    const uint32_t keep = ~((1u << (FIX_BITS - level)) - 1u);
    V3 offset = v3(fix_to_float(px & keep), fix_to_float(py & keep), fix_to_float(pz & keep));
    float extent = __uint_as_float((uint32_t)(127 - level) << 23);  // 2^-level
    if (!a.is_leaf(index)) {
        // below depth 24 (deeper than any grid of 2^24 voxels per axis): the
        // reference's float descent
        for (;; ++level) {
            if (a.is_leaf(index)) break;
            if (level >= FIND_MAX_DEPTH) {
                err |= 1u;
                base = offset;
                side = extent;
                path.depth = -1;
                return index;
            }
            extent *= 0.5f;
            const V3 oe = offset + vs(extent);
            const bool mx = pos.x >= oe.x, my = pos.y >= oe.y, mz = pos.z >= oe.z;
            offset = offset + v3(mx ? 1.0f : 0.0f, my ? 1.0f : 0.0f, mz ? 1.0f : 0.0f) * vs(extent);
            index = a.child(index, (mx ? 4u : 0u) | (my ? 2u : 0u) | (mz ? 1u : 0u));
        }
    }
    base = offset;
    side = extent;
    if (COUNT) loads += 2u * (uint32_t)level + 1u;
    if (level <= FIX_DEPTH) {
        path.depth = level;
        path.cx = px & keep;
        path.cy = py & keep;
        path.cz = pz & keep;
    } else {
        path.depth = -1;
    }
    return index;
}

// resources/svo_naive.comp:29-71.  RESUME: each step's find resumes from the
// previous path (find_cached); else it descends from the root (find), as the
// reference does.  Both find the same node with the same base and side.
template <bool COUNT, class Acc, bool RESUME = true, class Path = LocalPath>
__device__ V3 trace_naive(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err, Path* shared_path = nullptr) {
    const float MIN_STEP = 0.00001f;
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    V3 box_min = -bias;
    V3 box_max = rrd - bias;
    float t_min = max_elem(vmin(box_min, box_max));
    float t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs(0.0f);
    t_min = fmaxf(t_min, 0.0f);
    V3 total = vs(0.0f);
    float t = t_min + MIN_STEP;
    uint32_t iter = 0;
    FindPath path;
    Path local;
    Path& pn = shared_path ? *shared_path : local;
    while (t < t_max) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        V3 p = rd * t + ro;
        V3 offset;
        float side;
        uint32_t node = RESUME ? find_cached<COUNT>(a, path, pn, p, offset, side, loads, err)
                               : find<COUNT>(a, p, offset, side, loads, err);
        V3 node_min = offset * rrd - bias;
        V3 node_max = (offset + vs(side)) * rrd - bias;
        float u_min = max_elem(vmin(node_min, node_max));
        float u_max = min_elem(vmax(node_min, node_max));
        u_min = fmaxf(u_min, 0.0f);
        float step = fmaxf(u_max - u_min, MIN_STEP);
        t += step;
        V3 color = leaf_rgb(a.color(node));
        if (COUNT) ++loads;
        total = total + color * step;
    }
    return total;
}

// resources/svo_df.comp:6-67
template <bool COUNT, class Acc>
__device__ V3 trace_df(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    int sp = 0;
    uint32_t node_stack[STACK_DEPTH];
    uint32_t child_index_stack[STACK_DEPTH];
    uint32_t node = a.root();
    uint32_t child_idx = 0;
    V3 pos = vs(0.0f);
    float side = 0.5f;
    float s2_cached = -1.0f, s2_inv = 0.0f;
    bool s2_exact = false;
    V3 total = vs(0.0f);
    uint32_t iter = 0;
    for (;;) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        uint32_t child = a.child(node, child_idx);
        if (COUNT) ++loads;
        V3 box_min = pos * rrd - bias;
        V3 box_max = (pos + vs(side)) * rrd - bias;
        float t_min = max_elem(vmin(box_min, box_max));
        float t_max = min_elem(vmax(box_min, box_max));
        if (t_min < t_max && t_max > 0.0f) {
            if (COUNT) ++loads;
            if (a.is_leaf(child)) {
                V3 color = leaf_rgb(a.color(child));
                if (COUNT) ++loads;
                total = total + color * (t_max - fmaxf(t_min, 0.0f));
            } else {
                if (child_idx != 7) {
                    if (sp >= STACK_DEPTH) { err |= 2u; break; }
                    node_stack[sp] = node;
                    child_index_stack[sp] = child_idx;
                    ++sp;
                }
                side *= 0.5f;
                node = child;
                child_idx = 0;
                continue;
            }
        }
        if (child_idx == 7) {
            --sp;
            if (sp < 0) break;
            node = node_stack[sp];
            child_idx = child_index_stack[sp];
            uint32_t d = a.depth(node);
            if (COUNT) ++loads;
            side = ldexpf(1.0f, -(int)(d > 1000u ? 1000u : d)) * 0.5f;
        }
        const float s2 = side * 2.0f;
        if (s2 != s2_cached) {  // side changes only on a push or a pop
            s2_cached = s2;
            s2_exact = pow2_with_normal_reciprocal(s2);
            s2_inv = __frcp_rn(s2);
        }
        pos = pos - v3(gl_mod_pow2(pos.x, s2, s2_inv, s2_exact), gl_mod_pow2(pos.y, s2, s2_inv, s2_exact),
                       gl_mod_pow2(pos.z, s2, s2_inv, s2_exact));
        ++child_idx;
        if (child_idx & 4u) pos.x = pos.x + side;
        if (child_idx & 2u) pos.y = pos.y + side;
        if (child_idx & 1u) pos.z = pos.z + side;
    }
    return total;
}

// Two 32-bit stacks of STACK_DEPTH entries per thread (svo-df: node and
// remaining mask | depth; esvo: parent and t_max bits), in local memory or in
// shared memory with one column per thread (entry i of a thread at i * stride
// from its column start, so a warp touching one entry hits 32 banks).
struct LocalStacks {
    uint32_t a[STACK_DEPTH];
    uint32_t b[STACK_DEPTH];
    __device__ __forceinline__ uint32_t& first(uint32_t i) { return a[i]; }
    __device__ __forceinline__ uint32_t& second(uint32_t i) { return b[i]; }
};

struct SharedStacks {
    uint32_t* a;  // this thread's column in each array
    uint32_t* b;
    uint32_t stride;
    __device__ __forceinline__ uint32_t& first(uint32_t i) { return a[i * stride]; }
    __device__ __forceinline__ uint32_t& second(uint32_t i) { return b[i * stride]; }
};

// resources/svo_df.comp:6-67 for octrees whose depth fields match the tree
// (checked on upload; every octree the reference's builder writes does).
// The reference tests the 8 child boxes of a node one loop iteration at a
// time.  Here the 8 boxes of a node are tested together: with node origin O
// and child size s, the reference's box_min/box_max floats of child k are, per
// axis, two of the three plane distances O*rrd-bias, (O+s)*rrd-bias and
// ((O+s)+s)*rrd-bias (positions are dyadic, so these sums are exactly the
// reference's `pos` values), giving a hit mask; then the hit children are
// visited in index order.  Accumulation order and every accumulated value are
// the reference's, so the result is bit-identical; so is the word-read count.
// Plane distances of the 8 child boxes of one node: per axis the lower and
// upper bound of the low child (l0, h0) and of the high child (l1, h1).
struct ChildSlabs {
    float xl0, xl1, xh0, xh1, yl0, yl1, yh0, yh1, zl0, zl1, zh0, zh1;
};

__device__ __forceinline__ ChildSlabs child_slabs(V3 origin, float s, V3 rrd, V3 bias) {
    const float px1 = origin.x + s, py1 = origin.y + s, pz1 = origin.z + s;
    const float x0 = origin.x * rrd.x - bias.x, x1 = px1 * rrd.x - bias.x, x2 = (px1 + s) * rrd.x - bias.x;
    const float y0 = origin.y * rrd.y - bias.y, y1 = py1 * rrd.y - bias.y, y2 = (py1 + s) * rrd.y - bias.y;
    const float z0 = origin.z * rrd.z - bias.z, z1 = pz1 * rrd.z - bias.z, z2 = (pz1 + s) * rrd.z - bias.z;
    // the x entry slabs are clamped at 0: every use of a child's t_min is
    // max(t_min, 0) (the leaf's step, and the hit test t_min < t_max &&
    // t_max > 0, which is max(t_min, 0) < t_max), and fmaxf is exact and
    // associative on these finite values
    return ChildSlabs{fmaxf(fminf(x0, x1), 0.0f), fmaxf(fminf(x1, x2), 0.0f), fmaxf(x0, x1), fmaxf(x1, x2),
                      fminf(y0, y1), fminf(y1, y2), fmaxf(y0, y1), fmaxf(y1, y2),
                      fminf(z0, z1), fminf(z1, z2), fmaxf(z0, z1), fmaxf(z1, z2)};
}

// max(t_min, 0) / t_max of child k, as the reference computes them for that box
__device__ __forceinline__ void child_span(const ChildSlabs& c, uint32_t k, float& t0, float& t1) {
    const bool bx = k & 4u, by = k & 2u, bz = k & 1u;
    t0 = max3f(bx ? c.xl1 : c.xl0, by ? c.yl1 : c.yl0, bz ? c.zl1 : c.zl0);
    t1 = min3f(bx ? c.xh1 : c.xh0, by ? c.yh1 : c.yh0, bz ? c.zh1 : c.zh0);
}

// fmaxf/fminf are exact and the slab values are finite (every ray direction
// component is at least 2^-23 in magnitude), so each child's max/min of
// three is one three-input operation.
__device__ __forceinline__ uint32_t hit_mask(const ChildSlabs& c) {
    uint32_t m = 0;
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k) {
        const bool bx = k & 4u, by = k & 2u, bz = k & 1u;
        const float t0 = max3f(bx ? c.xl1 : c.xl0, by ? c.yl1 : c.yl0, bz ? c.zl1 : c.zl0);
        const float t1 = min3f(bx ? c.xh1 : c.xh0, by ? c.yh1 : c.yh0, bz ? c.zh1 : c.zh0);
        if (t0 < t1) m |= 1u << k;  // t0 >= 0: t_max > 0 follows
    }
    return m;
}

// resources/svo_df.comp:6-67 for octrees whose depth fields match the tree
// (checked on upload; every octree the reference's builder writes does).
// The reference tests the 8 child boxes of a node one loop iteration at a
// time.  Here they are tested together: with node origin O and child size s,
// child k's box_min/box_max floats are, per axis, two of the plane distances
// O*rrd-bias, (O+s)*rrd-bias and ((O+s)+s)*rrd-bias (positions are dyadic, so
// these sums are exactly the reference's `pos` values), which gives a hit
// mask; the hit children are then visited in index order.  Pushes and pops
// happen exactly where the reference's do, the accumulation order and every
// accumulated value are the reference's, so the result is bit-identical, and
// so is the count of words the reference reads.
template <bool COUNT, class Acc, class Stacks = LocalStacks>
__device__ V3 trace_df_masked(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err,
                              Stacks* shared_stacks = nullptr) {
    const V3 rrd = vs(1.0f) / rd;
    const V3 bias = rrd * ro;
    Stacks local;
    Stacks& stk = shared_stacks ? *shared_stacks : local;  // first: node, second: remaining mask | depth << 8
    int sp = 0;
    uint32_t node = a.root();
    uint32_t depth = 0;
    V3 origin = vs(0.0f);
    float side = 0.5f;  // child box size of `node`
    V3 total = vs(0.0f);
    ChildSlabs slabs = child_slabs(origin, side, rrd, bias);
    uint32_t mask = hit_mask(slabs);
    if (COUNT) loads += 8;  // the reference reads children[0..7] of every node it visits
    uint32_t iter = 0;
    for (;;) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        if (mask == 0) {
            // node finished: the reference pops, reading the parent's depth
            --sp;
            if (sp < 0) break;
            node = stk.first(sp);
            const uint32_t st = stk.second(sp);
            mask = st & 0xFFu;
            depth = st >> 8;
            if (COUNT) ++loads;
            float s2, inv;
            bool ex;
            if (depth <= 124u) {
                // 2^-depth and 2^depth built from their exponents: the values
                // ldexpf and the correctly rounded reciprocal give
                s2 = __uint_as_float((127u - depth) << 23);
                inv = __uint_as_float((127u + depth) << 23);
                side = s2 * 0.5f;
                ex = true;
            } else {
                side = ldexpf(1.0f, -(int)(depth > 1000u ? 1000u : depth)) * 0.5f;
                s2 = side * 2.0f;
                inv = __frcp_rn(s2);
                ex = pow2_with_normal_reciprocal(s2);
            }
            origin = v3(snap_down_pow2(origin.x, s2, inv, ex), snap_down_pow2(origin.y, s2, inv, ex),
                        snap_down_pow2(origin.z, s2, inv, ex));
            slabs = child_slabs(origin, side, rrd, bias);
            continue;
        }
        const uint32_t k = __ffs(mask) - 1;
        mask &= mask - 1;
        const uint32_t child = a.child(node, k);
        if (COUNT) ++loads;  // is_leaf_depth of the hit child
        float t0, t1;
        child_span(slabs, k, t0, t1);
        if (a.is_leaf(child)) {
            const V3 color = leaf_rgb(a.color(child));
            if (COUNT) ++loads;
            total = total + color * (t1 - t0);
            continue;
        }
        // descend into child k; the reference pushes unless k == 7
        if (k != 7) {
            if (sp >= STACK_DEPTH) { err |= 2u; break; }
            stk.first(sp) = node;
            stk.second(sp) = mask | (depth << 8);
            ++sp;
        }
        origin = v3(origin.x + ((k & 4u) ? side : 0.0f), origin.y + ((k & 2u) ? side : 0.0f),
                    origin.z + ((k & 1u) ? side : 0.0f));
        node = child;
        ++depth;
        side *= 0.5f;
        slabs = child_slabs(origin, side, rrd, bias);
        mask = hit_mask(slabs);
        if (COUNT) loads += 8;
    }
    return total;
}

__device__ __forceinline__ uint32_t cxor(uint32_t x, bool ax, bool ay, bool az) {
    return x ^ (ax ? 4u : 0u) ^ (ay ? 2u : 0u) ^ (az ? 1u : 0u);
}

// resources/esvo.comp:30-136
// ESVO's (parent, t_max) stack, indexed by scale: LocalStacks / SharedStacks
// (t_max kept as its bits).
template <bool COUNT, class Acc, class Stacks = LocalStacks>
__device__ V3 trace_esvo(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err, Stacks* shared_stacks = nullptr) {
    const uint32_t depth = STACK_DEPTH;
    Stacks local;
    Stacks& stk = shared_stacks ? *shared_stacks : local;  // first: parent, second: t_max bits
#pragma unroll
    for (int i = 0; i < STACK_DEPTH; ++i) { stk.first(i) = 0; stk.second(i) = 0u; }

    V3 t_coeff = v3(1.0f / -fabsf(rd.x), 1.0f / -fabsf(rd.y), 1.0f / -fabsf(rd.z));
    V3 t_bias = t_coeff * ro;
    bool gx = rd.x > 0.0f, gy = rd.y > 0.0f, gz = rd.z > 0.0f;
    {
        V3 alt = t_coeff * 3.0f - t_bias;
        if (gx) t_bias.x = alt.x;
        if (gy) t_bias.y = alt.y;
        if (gz) t_bias.z = alt.z;
    }
    const uint32_t octant_mask = cxor(0u, gx, gy, gz);
    float t_min = max_elem(t_coeff * 2.0f - t_bias);
    float t_max = min_elem(t_coeff - t_bias);
    float h = t_max;
    t_min = fmaxf(t_min, 0.0f);
    t_max = fminf(t_max, 1.73205078f);  // float(sqrt(3))

    uint32_t parent = a.root();
    uint32_t idx = 0;
    V3 pos = vs(1.0f);
    uint32_t scale = depth - 1;
    float scale_exp2 = 0.5f;
    {
        V3 tc = t_coeff * 1.5f - t_bias;
        bool ax = tc.x > t_min, ay = tc.y > t_min, az = tc.z > t_min;
        if (ax) pos.x = 1.5f;
        if (ay) pos.y = 1.5f;
        if (az) pos.z = 1.5f;
        idx = cxor(idx, ax, ay, az);
    }
    V3 total = vs(0.0f);
    // Between two pops the loop descends at most `depth` times (the scale
    // runs out) and advances at most 3 times per level, so a cap on the pops
    // bounds it.
    uint32_t pops = 0;
    while (scale < depth) {
        V3 t_corner = pos * t_coeff - t_bias;
        float tc_max = min_elem(t_corner);
        // the reference tests t_min <= t_max and then t_min <= tv_max; as
        // tv_max <= t_max, the second test alone decides
        float tv_max = fminf(t_max, tc_max);
        if (t_min <= tv_max) {
            uint32_t child = a.child(parent, idx ^ octant_mask);
            if (COUNT) loads += 2;
            if (a.is_leaf(child)) {
                V3 color = leaf_rgb(a.color(child));
                if (COUNT) ++loads;
                total = total + color * (tv_max - t_min);
            } else {
                if (tc_max < h) {
                    stk.first(scale) = parent;
                    stk.second(scale) = __float_as_uint(t_max);
                }
                h = tc_max;
                parent = child;
                --scale;
                scale_exp2 *= 0.5f;
                // t_coeff * scale_exp2 is exact (a power of two, 2^-23..2^-1,
                // times |t_coeff| in [1, 2^23]), so the fused form rounds
                // once, like the reference's product-then-sum
                V3 t_center = v3(__fmaf_rn(t_coeff.x, scale_exp2, t_corner.x), __fmaf_rn(t_coeff.y, scale_exp2, t_corner.y),
                                 __fmaf_rn(t_coeff.z, scale_exp2, t_corner.z));
                bool ax = t_center.x > t_min, ay = t_center.y > t_min, az = t_center.z > t_min;
                idx = cxor(0u, ax, ay, az);
                if (ax) pos.x = pos.x + scale_exp2;
                if (ay) pos.y = pos.y + scale_exp2;
                if (az) pos.z = pos.z + scale_exp2;
                t_max = tv_max;
                continue;
            }
        }
        // ADVANCE
        bool ax = t_corner.x <= tc_max, ay = t_corner.y <= tc_max, az = t_corner.z <= tc_max;
        uint32_t step_mask = cxor(0u, ax, ay, az);
        if (ax) pos.x = pos.x - scale_exp2;
        if (ay) pos.y = pos.y - scale_exp2;
        if (az) pos.z = pos.z - scale_exp2;
        t_min = tc_max;
        idx ^= step_mask;
        if ((idx & step_mask) != 0) {
            // POP
            if (++pops > SVO_MAX_ITER) { err |= 1u; break; }
            uint32_t xx = __float_as_uint(pos.x) ^ __float_as_uint(pos.x + scale_exp2);
            uint32_t xy = __float_as_uint(pos.y) ^ __float_as_uint(pos.y + scale_exp2);
            uint32_t xz = __float_as_uint(pos.z) ^ __float_as_uint(pos.z + scale_exp2);
            uint32_t dbits = (ax ? xx : 0u) | (ay ? xy : 0u) | (az ? xz : 0u);
            scale = (__float_as_uint(__uint2float_rn(dbits)) >> 23) - 127u;
            if (scale >= depth) break;  // the loop condition ends the ray
            scale_exp2 = __uint_as_float((scale - depth + 127u) << 23);
            parent = stk.first(scale);
            t_max = __uint_as_float(stk.second(scale));
            uint32_t shx = __float_as_uint(pos.x) >> scale;
            uint32_t shy = __float_as_uint(pos.y) >> scale;
            uint32_t shz = __float_as_uint(pos.z) >> scale;
            pos = v3(__uint_as_float(shx << scale), __uint_as_float(shy << scale), __uint_as_float(shz << scale));
            idx = (shx & 1u) * 4u + (shy & 1u) * 2u + (shz & 1u);
            h = 0.0f;
        }
    }
    return total;
}

// resources/svo_rope.comp:29-48
template <bool COUNT, class Acc>
__device__ __forceinline__ uint32_t find_relative(const Acc& a, uint32_t parent, V3 offset, V3 pos, V3& base,
                                                  float& side, uint32_t& loads, uint32_t& err) {
    uint32_t d = a.depth(parent);
    if (COUNT) ++loads;
    // mod by extent = 2^-d: for d <= 124 the division is the exact multiply
    // by 2^d (both built from their exponents), as in gl_mod_pow2
    float extent, inv = 0.0f;
    bool ex = false;
    if (d <= 124u) {
        extent = __uint_as_float((127u - d) << 23);
        inv = __uint_as_float((127u + d) << 23);
        ex = true;
    } else {
        extent = ldexpf(1.0f, -(int)(d > 1000u ? 1000u : d));
    }
    offset = v3(snap_down_pow2(offset.x, extent, inv, ex), snap_down_pow2(offset.y, extent, inv, ex),
                snap_down_pow2(offset.z, extent, inv, ex));
    for (int level = 0;; ++level) {
        if (COUNT) ++loads;
        if (a.is_leaf(parent)) {
            base = offset;
            side = extent;
            return parent;
        }
        if (level >= FIND_MAX_DEPTH) { err |= 1u; base = offset; side = extent; return parent; }
        extent *= 0.5f;
        V3 oe = offset + vs(extent);
        bool mx = pos.x >= oe.x, my = pos.y >= oe.y, mz = pos.z >= oe.z;
        uint32_t child = (mx ? 4u : 0u) | (my ? 2u : 0u) | (mz ? 1u : 0u);
        offset = offset + v3(mx ? 1.0f : 0.0f, my ? 1.0f : 0.0f, mz ? 1.0f : 0.0f) * vs(extent);
        parent = a.child(parent, child);
        if (COUNT) ++loads;
    }
}

// resources/svo_rope.comp:50-63.  The reference returns a one-hot mask and
// moves the offset by (mask * sgn) * side: the chosen axis by sgn * side,
// the others by +-0, which leaves them unchanged (offsets are never -0).  So
// only the chosen axis is moved here.
__device__ __forceinline__ uint32_t neighbor_index(uint32_t nx, uint32_t ny, uint32_t nz, V3 far, V3 sgn, float side,
                                                   V3& offset) {
    if (far.x < fminf(far.y, far.z)) {
        offset.x = offset.x + sgn.x * side;
        return nx;
    }
    if (far.y < far.z) {
        offset.y = offset.y + sgn.y * side;
        return ny;
    }
    offset.z = offset.z + sgn.z * side;
    return nz;
}

// resources/svo_rope.comp:65-135
template <bool COUNT, class Acc>
__device__ V3 trace_rope(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
    V3 sgn = v3(gl_sign(rd.x), gl_sign(rd.y), gl_sign(rd.z));
    const uint32_t nbx = 1u - (uint32_t)fmaxf(sgn.x, 0.0f);
    const uint32_t nby = 3u - (uint32_t)fmaxf(sgn.y, 0.0f);
    const uint32_t nbz = 5u - (uint32_t)fmaxf(sgn.z, 0.0f);
    sgn = sgn + vs(0.1f);
    V3 rrd = vs(1.0f) / rd;
    V3 bias = rrd * ro;
    V3 box_min = -bias;
    V3 box_max = rrd - bias;
    float t_min = max_elem(vmin(box_min, box_max));
    float t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs(0.0f);
    t_min = fmaxf(t_min, 0.0f);
    V3 pos = ro + rd * t_min;
    V3 offset;
    float side;
    uint32_t node = find<COUNT>(a, pos, offset, side, loads, err);
    V3 node_min = offset * rrd - bias;
    V3 node_max = (offset + vs(side)) * rrd - bias;
    V3 far = vmax(node_min, node_max);
    float u_min = max_elem(vmin(node_min, node_max));
    float u_max = min_elem(far);
    float step = u_max - fmaxf(u_min, 0.0f);
    V3 color = leaf_rgb(a.color(node));
    V3 total = color * step;
    uint32_t n = neighbor_index(nbx, nby, nbz, far, sgn, side, offset);
    node = a.child(node, n);
    if (COUNT) loads += 2;
    uint32_t iter = 0;
    while (node != a.exit_word()) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        pos = ro + rd * u_max;
        node = find_relative<COUNT>(a, node, offset, pos, offset, side, loads, err);
        node_min = offset * rrd - bias;
        node_max = (offset + vs(side)) * rrd - bias;
        far = vmax(node_min, node_max);
        u_min = max_elem(vmin(node_min, node_max));
        u_max = min_elem(far);
        step = u_max - fmaxf(u_min, 0.0f);
        color = leaf_rgb(a.color(node));
        total = total + color * step;
        n = neighbor_index(nbx, nby, nbz, far, sgn, side, offset);
        node = a.child(node, n);
        if (COUNT) loads += 2;
    }
    return total;
}

// esvo.comp:10-21
__device__ __forceinline__ float aabb_entry(V3 bmin, V3 bmax, V3 ro, V3 rd) {
    V3 rrd = vs(1.0f) / (rd + vs(0.00000001f));
    V3 tbot = (bmin - ro) * rrd;
    V3 ttop = (bmax - ro) * rrd;
    V3 tmin = vmin(ttop, tbot);
    return max3f(tmin.x, tmin.y, tmin.z);  // the same value as the reference's max(max(x, y), max(x, z))
}

// ---------------------------------------------------------------- kernels ---

constexpr int TILE_W = 16;  // block covers 16x8 pixels: 2x2 warps of 8x4
constexpr int TILE_H = 8;
constexpr int BLOCK_THREADS = TILE_W * TILE_H;


// Blocks of BT threads cover 16 x (BT/16) pixels: warps of 8x4 pixels, two
// per row of warps.
template <int BT>
__device__ __forceinline__ bool pixel_of_thread_bt(const Frame& f, uint32_t& ix, uint32_t& iy) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    ix = blockIdx.x * 16u + (warp & 1u) * 8u + (lane & 7u);
    iy = blockIdx.y * (uint32_t)(BT / 16) + (warp >> 1) * 4u + (lane >> 3);
    return ix < f.out_w && iy < f.out_h;
}

__device__ __forceinline__ bool pixel_of_thread(const Frame& f, uint32_t& ix, uint32_t& iy) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    ix = blockIdx.x * TILE_W + (warp & 1u) * 8u + (lane & 7u);
    iy = blockIdx.y * TILE_H + (warp >> 1) * 4u + (lane >> 3);
    return ix < f.out_w && iy < f.out_h;
}

__device__ __forceinline__ void write_outputs(const Frame& f, const Outputs& o, uint32_t ix, uint32_t iy, V3 color,
                                              uint32_t loads, uint32_t err) {
    const uint64_t p = (uint64_t)iy * f.out_w + ix;
    o.rgba[p] = pack_rgba(color);
    if (o.emission) {
        o.emission[3 * p + 0] = color.x;
        o.emission[3 * p + 1] = color.y;
        o.emission[3 * p + 2] = color.z;
    }
    if (o.loads) o.loads[p] = loads;
    if (err) atomicOr(o.err_word, err);
}

// resources/dda.comp:55-73
template <bool COUNT>
__global__ void __launch_bounds__(BLOCK_THREADS) dda_kernel(Frame f, GridVol g, Outputs o) {
    uint32_t ix, iy;
    if (!pixel_of_thread(f, ix, iy)) return;
    uint32_t m = max(g.dx, max(g.dy, g.dz));
    float side = (float)m;
    V3 ro = f.translation * side;
    V3 rd = primary_ray(f, ix, iy);
    float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
    uint32_t loads = 0, err = 0;
    V3 color = trace_dda<COUNT>(g, ro, rd, loads, err) * ec;
    write_outputs(f, o, ix, iy, color, loads, err);
}

// Warps of WW x 32/WW pixels, 2 x 2 warps a block (WW = 8: the 8x4 tiles of
// every other kernel).
template <uint32_t WW>
__device__ __forceinline__ bool pixel_of_thread_ww(const Frame& f, uint32_t& ix, uint32_t& iy) {
    constexpr uint32_t WH = 32 / WW;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    ix = blockIdx.x * (2 * WW) + (warp & 1u) * WW + lane % WW;
    iy = blockIdx.y * (2 * WH) + (warp >> 1) * WH + lane / WW;
    return ix < f.out_w && iy < f.out_h;
}

template <bool COUNT, int NORM, uint32_t WW = 8>
__global__ void __launch_bounds__(BLOCK_THREADS) dda_tex_kernel(Frame f, cudaTextureObject_t tex, uint32_t dx,
                                                               uint32_t dy, uint32_t dz, Outputs o) {
    if (NORM == TEX_RAW) fill_unorm_lut();
    uint32_t ix, iy;
    if (!pixel_of_thread_ww<WW>(f, ix, iy)) return;
    uint32_t m = max(dx, max(dy, dz));
    float side = (float)m;
    V3 ro = f.translation * side;
    V3 rd = primary_ray(f, ix, iy);
    float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
    uint32_t loads = 0, err = 0;
    V3 color = trace_dda_tex<COUNT, NORM>(tex, dx, dy, dz, ro, rd, loads, err) * ec;
    write_outputs(f, o, ix, iy, color, loads, err);
}

// The texture unit's data stage limits the texture DDA on large frames (its
// tex wavefronts near their peak while the L1 banks and the LSU path idle).
// Here one warp in `share` (warp index % share == 0) reads the x-fastest copy
// of the grid through the LSU path instead; the arithmetic is the reference's
// either way, so every pixel is the same.
template <bool COUNT>
__global__ void __launch_bounds__(BLOCK_THREADS) dda_hybrid_kernel(Frame f, cudaTextureObject_t tex, GridVol g,
                                                                  uint32_t share, Outputs o) {
    uint32_t ix, iy;
    if (!pixel_of_thread(f, ix, iy)) return;
    uint32_t m = max(g.dx, max(g.dy, g.dz));
    float side = (float)m;
    V3 ro = f.translation * side;
    V3 rd = primary_ray(f, ix, iy);
    float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
    uint32_t loads = 0, err = 0;
    const uint32_t warp = (blockIdx.y * gridDim.x + blockIdx.x) * (BLOCK_THREADS / 32) + (threadIdx.x >> 5);
    V3 total = warp % share == 0 ? trace_dda<COUNT>(g, ro, rd, loads, err)
                                 : trace_dda_tex<COUNT, true>(tex, g.dx, g.dy, g.dz, ro, rd, loads, err);
    write_outputs(f, o, ix, iy, total * ec, loads, err);
}

template <bool COUNT>
__global__ void __launch_bounds__(BLOCK_THREADS) dda_brick_kernel(Frame f, BrickGrid g, Outputs o) {
    fill_unorm_lut();
    uint32_t ix, iy;
    if (!pixel_of_thread(f, ix, iy)) return;
    uint32_t m = max(g.dx, max(g.dy, g.dz));
    float side = (float)m;
    V3 ro = f.translation * side;
    V3 rd = primary_ray(f, ix, iy);
    float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
    uint32_t loads = 0, err = 0;
    V3 color = trace_dda_brick<COUNT>(g, ro, rd, loads, err) * ec;
    write_outputs(f, o, ix, iy, color, loads, err);
}

template <int TRAV, bool COUNT, class Acc>
__device__ __forceinline__ void svo_pixel(const Frame& f, const Acc& a, const Outputs& o) {
    fill_unorm_lut();
    uint32_t ix, iy;
    if (!pixel_of_thread(f, ix, iy)) return;
    V3 rd = primary_ray(f, ix, iy);
    uint32_t loads = 0, err = 0;
    V3 total;
    if (TRAV == XN_TRAV_ESVO) {
        // resources/esvo.comp:148-152
        V3 ro = f.translation + vs(1.0f);
        float t0 = aabb_entry(vs(1.0f), vs(2.0f), ro, rd);
        ro = ro + rd * fmaxf(t0, 0.0f);
        total = trace_esvo<COUNT>(a, ro, rd, loads, err);
    } else if constexpr (TRAV == XN_TRAV_SVO_NAIVE) {
        // the find's path nodes in a column of shared memory (12 KB per block)
        __shared__ uint32_t s_path[FIX_DEPTH * BLOCK_THREADS];
        SharedPath sp{s_path + threadIdx.x, BLOCK_THREADS};
        total = trace_naive<COUNT, Acc, true, SharedPath>(a, f.translation, rd, loads, err, &sp);
    } else if (TRAV == XN_TRAV_SVO_NAIVE_ROOT) {
        total = trace_naive<COUNT, Acc, false>(a, f.translation, rd, loads, err);
    } else if (TRAV == XN_TRAV_SVO_DF) {
        total = trace_df<COUNT>(a, f.translation, rd, loads, err);
    } else if (TRAV == XN_TRAV_SVO_DF_MASKED) {
        total = trace_df_masked<COUNT>(a, f.translation, rd, loads, err);
    } else {
        total = trace_rope<COUNT>(a, f.translation, rd, loads, err);
    }
    V3 color = total * voxel_emission_coeff(f, rd);
    write_outputs(f, o, ix, iy, color, loads, err);
}

template <int TRAV, bool COUNT, class Acc>
__global__ void __launch_bounds__(BLOCK_THREADS) svo_kernel(Frame f, Acc a, Outputs o) {
    svo_pixel<TRAV, COUNT>(f, a, o);
}

// svo-rope's steps are short dependent chains of node reads: held to 40
// registers, twelve blocks an SM keep more of them in flight.
template <bool COUNT, class Acc>
__global__ void __launch_bounds__(BLOCK_THREADS, 12) svo_rope_kernel(Frame f, Acc a, Outputs o) {
    svo_pixel<XN_TRAV_SVO_ROPE, COUNT>(f, a, o);
}

// svo-df, masked form, walked by the whole warp at once.  Each lane has its
// own ray and its own hit masks; the warp visits the union of the lanes' hit
// children in index order, descending depth first as the reference does.  A
// lane that hits a child does exactly what its own masked traversal would do
// there (accumulate a leaf, or descend and take the child's hit mask), a lane
// that does not sits out that child's subtree with empty masks.  Restricted
// to one lane, the union walk visits that lane's hit children in the same
// order with the same arithmetic, so every ray's result (and its word count)
// is the one-ray-per-thread result, while the control flow, the node loads
// (one address per warp) and the pops are shared by the warp.
//   each stack entry: the node, the union of the lanes' remaining masks, the
//   node's origin and child size (all warp-uniform), and each lane's own
//   remaining mask.
// The warp's stacks for trace_df_packet: per-warp arrays (its own kernel; the
// uniform part as one 8-byte and one 16-byte word per entry) or, in the batch
// kernel, carved from the per-thread columns of the shared stacks (the
// uniform words in lanes 0..5's first columns, each lane's masks in its own
// second column), so they never overlap another warp's.
struct PacketStacksWarp {
    uint2* w_ns;     // node, union mask
    float4* w_geo;   // origin x, y, z, child size
    uint8_t* l_mask;
    uint32_t lane;
    __device__ __forceinline__ void push(int i, uint32_t node, uint32_t uni, V3 o, float side) {
        w_ns[i] = make_uint2(node, uni);
        w_geo[i] = make_float4(o.x, o.y, o.z, side);
    }
    __device__ __forceinline__ void pop(int i, uint32_t& node, uint32_t& uni, V3& o, float& side) const {
        const uint2 ns = w_ns[i];
        const float4 g = w_geo[i];
        node = ns.x;
        uni = ns.y;
        o = v3(g.x, g.y, g.z);
        side = g.w;
    }
    __device__ __forceinline__ uint32_t mask(int i) const { return l_mask[i * 32 + lane]; }
    __device__ __forceinline__ void set_mask(int i, uint32_t m) { l_mask[i * 32 + lane] = (uint8_t)m; }
};

struct PacketStacksColumns {
    uint32_t* w0;    // lane 0's first column (lanes 0..5: node, union mask, origin x, y, z, child size)
    uint32_t* mine;  // this lane's second column
    uint32_t stride;
    __device__ __forceinline__ void push(int i, uint32_t node, uint32_t uni, V3 o, float side) {
        uint32_t* e = w0 + (size_t)i * stride;
        e[0] = node;
        e[1] = uni;
        e[2] = __float_as_uint(o.x);
        e[3] = __float_as_uint(o.y);
        e[4] = __float_as_uint(o.z);
        e[5] = __float_as_uint(side);
    }
    __device__ __forceinline__ void pop(int i, uint32_t& node, uint32_t& uni, V3& o, float& side) const {
        const uint32_t* e = w0 + (size_t)i * stride;
        node = e[0];
        uni = e[1];
        o = v3(__uint_as_float(e[2]), __uint_as_float(e[3]), __uint_as_float(e[4]));
        side = __uint_as_float(e[5]);
    }
    __device__ __forceinline__ uint32_t mask(int i) const { return mine[i * stride]; }
    __device__ __forceinline__ void set_mask(int i, uint32_t m) { mine[i * stride] = m; }
};

// The bottom of the octree walked by each lane alone.  In a depth-consistent
// tree whose deepest internal nodes are at depth D, a node at depth D-1 has
// only leaves and internal children whose children are all leaves, and a
// node at depth D-2 only leaves and such D-1 nodes.  Below such a node each
// lane takes its own hit children in index order: a leaf is accumulated, an
// internal child gets its own hit mask and is walked the same way.  That is
// the lane's own traversal, with the same arithmetic and word reads; the warp
// loops over the largest per-lane count instead of the union.

// The hit leaves of node c (origin co, child size cs; all children leaves),
// in index order.  The eight children are tested in an unrolled loop, so
// each child's span is formed from the slabs without a select on a run-time
// index, and a hit leaf is accumulated where it is found: the same spans,
// the same hit test and the same order as the hit mask and its walk.
template <bool COUNT, class Acc>
__device__ __forceinline__ void lane_leaves(const Acc& a, uint32_t c, V3 co, float cs, V3 rrd, V3 bias, V3& total,
                                            uint32_t& loads) {
    const ChildSlabs sl = child_slabs(co, cs, rrd, bias);
#pragma unroll
    for (uint32_t j = 0; j < 8; ++j) {
        float t0, t1;
        child_span(sl, j, t0, t1);
        if (t0 < t1) {  // t0 >= 0: t_max > 0 follows
            if (COUNT) loads += 2;  // the leaf's is_leaf_depth and colour
            total = total + leaf_rgb(a.color(a.child(c, j))) * (t1 - t0);
        }
    }
}

// Origin of child k of a node with origin o and child size s.
__device__ __forceinline__ V3 child_origin(V3 o, float s, uint32_t k) {
    return v3(o.x + ((k & 4u) ? s : 0.0f), o.y + ((k & 2u) ? s : 0.0f), o.z + ((k & 1u) ? s : 0.0f));
}

// Node c at depth D-1 (origin co, child size cs), visited by this lane only.
template <bool COUNT, class Acc>
__device__ __forceinline__ void lane_walk_own(const Acc& a, uint32_t c, V3 co, float cs, V3 rrd, V3 bias, V3& total,
                                              uint32_t& loads) {
    const ChildSlabs sl = child_slabs(co, cs, rrd, bias);
    uint32_t m = hit_mask(sl);
    while (m != 0) {
        const uint32_t k = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t w = a.child(c, k);
        if (a.is_leaf(w)) {
            float t0, t1;
            child_span(sl, k, t0, t1);
            if (COUNT) loads += 2;
            total = total + leaf_rgb(a.color(w)) * (t1 - t0);
        } else {
            // descend (its is_leaf_depth and 8 children; the pop back reads
            // this node's depth unless k == 7)
            if (COUNT) loads += 9u + (k != 7u ? 1u : 0u);
            lane_leaves<COUNT>(a, w, child_origin(co, cs, k), cs * 0.5f, rrd, bias, total, loads);
        }
    }
}

// A node the whole warp holds, LEVELS above the deepest internal nodes:
// `words` its child words (lane j: word j & 7), `own` this lane's hit mask.
template <bool COUNT, int LEVELS, class Acc>
__device__ __forceinline__ void lane_walk(const Acc& a, uint32_t words, uint32_t own, V3 origin, float side,
                                          const ChildSlabs& slabs, V3 rrd, V3 bias, V3& total, uint32_t& loads) {
    while (__any_sync(0xFFFFFFFFu, own != 0)) {
        const bool has = own != 0;
        const uint32_t k = has ? __ffs(own) - 1 : 0u;
        own &= own - 1;
        const uint32_t c = __shfl_sync(0xFFFFFFFFu, words, k);
        if (a.is_leaf(c)) {
            float t0, t1;
            child_span(slabs, k, t0, t1);
            const V3 color = leaf_rgb(a.color(c));
            if (COUNT && has) loads += 2;
            // a lane without a child here adds color * 0 = +0
            total = total + color * (has ? t1 - t0 : 0.0f);
        } else if (has) {
            if (COUNT) loads += 9u + (k != 7u ? 1u : 0u);
            const V3 co = child_origin(origin, side, k);
            if constexpr (LEVELS == 2) lane_walk_own<COUNT>(a, c, co, side * 0.5f, rrd, bias, total, loads);
            else lane_leaves<COUNT>(a, c, co, side * 0.5f, rrd, bias, total, loads);
        }
    }
}

// lane_side: the child size of the nodes the lanes walk alone (LEVELS = 1:
// 2^-D, D the deepest internal node's depth; LEVELS = 2: 2^-(D-1)), or 0.
template <bool COUNT, class Acc, class PS, int LEVELS = 1>
__device__ V3 trace_df_packet(const Acc& a, V3 ro, V3 rd, bool active, uint32_t& loads, uint32_t& err, PS& ps,
                              float lane_side = 0.0f) {
    const V3 rrd = vs(1.0f) / rd;
    const V3 bias = rrd * ro;
    int sp = 0;
    uint32_t node = a.root();
    // the node is the same on every lane: lane j holds its child word j & 7,
    // and a child word is a shuffle away
    const uint32_t slot = threadIdx.x & 7u;
    uint32_t words = a.child(node, slot);
    // which of the node's children are leaves: lanes 0..7 hold words 0..7
    uint32_t leaves = __ballot_sync(0xFFFFFFFFu, a.is_leaf(words)) & 0xFFu;
    V3 origin = vs(0.0f);
    float side = 0.5f;
    V3 total = vs(0.0f);
    ChildSlabs slabs = child_slabs(origin, side, rrd, bias);
    uint32_t own = active ? hit_mask(slabs) : 0u;
    if (COUNT && active) loads += 8;
    uint32_t uni;
    if (side == lane_side) {
        lane_walk<COUNT, LEVELS>(a, words, own, origin, side, slabs, rrd, bias, total, loads);
        uni = 0;
    } else {
        uni = __reduce_or_sync(0xFFFFFFFFu, own);
    }
    // Between two pops the walk only descends, and after about 150 descents
    // the child size is 0 and no child is hit; so a cap on the pops bounds
    // the loop.
    uint32_t pops = 0;
    for (;;) {
        if (uni == 0) {
            // every lane is done with this node: pop (the reference reads the
            // parent's depth; masked svo-df takes it from the stack)
            --sp;
            if (sp < 0) break;
            if (++pops > SVO_MAX_ITER) {
                if (active) err |= 1u;
                break;
            }
            // the reference recomputes the node's child size from its depth
            // field and its origin as pos - mod(pos, 2 side); with consistent
            // depth fields those are the values stored when the node was
            // pushed, bit for bit
            ps.pop(sp, node, uni, origin, side);
            own = ps.mask(sp);
            words = a.child(node, slot);
            leaves = __ballot_sync(0xFFFFFFFFu, a.is_leaf(words)) & 0xFFu;
            slabs = child_slabs(origin, side, rrd, bias);
            continue;
        }
        // The run of leaf children before the next internal child of the
        // union: each lane accumulates its own hit leaves of the run in index
        // order (the warp loops over the largest count), which is the order
        // of its own traversal.  A lane's mask bits of passed children are
        // never read again, so they are left set.
        const uint32_t inner_left = uni & ~leaves;
        const uint32_t run = inner_left ? uni & ((inner_left & (0u - inner_left)) - 1u) : uni;
        if (run) {
            uni &= ~run;
            uint32_t mine_run = own & run;
            while (__any_sync(0xFFFFFFFFu, mine_run != 0)) {
                const bool hit = mine_run != 0;
                const uint32_t k = hit ? __ffs(mine_run) - 1 : 0u;
                mine_run &= mine_run - 1;
                const uint32_t child = __shfl_sync(0xFFFFFFFFu, words, k);
                float t0, t1;
                child_span(slabs, k, t0, t1);
                const V3 color = leaf_rgb(a.color(child));
                if (COUNT && hit) loads += 2;  // the child's is_leaf_depth and colour
                // a lane without a leaf here adds color * 0 = +0, which
                // leaves its sum (never -0) unchanged
                total = total + color * (hit ? t1 - t0 : 0.0f);
            }
            if (uni == 0) continue;
        }
        // the lowest child left is internal: descend into it (lanes that
        // miss it sit out its subtree)
        const uint32_t k = __ffs(uni) - 1;
        const uint32_t child = __shfl_sync(0xFFFFFFFFu, words, k);
        uni &= uni - 1;
        const bool mine = (own >> k) & 1u;
        if (COUNT && mine) ++loads;
        if (uni != 0) {
            if (sp >= STACK_DEPTH) {
                if (active) err |= 2u;
                break;
            }
            // every lane holds the same node, masks union, origin and size
            // and writes them itself, so its later reads see its own writes
            ps.push(sp, node, uni, origin, side);
            ps.set_mask(sp, own);
            ++sp;
        }
        if (COUNT && mine && k != 7) ++loads;  // the pop back to this node reads its depth
        origin = v3(origin.x + ((k & 4u) ? side : 0.0f), origin.y + ((k & 2u) ? side : 0.0f),
                    origin.z + ((k & 1u) ? side : 0.0f));
        node = child;
        words = a.child(node, slot);
        side *= 0.5f;
        slabs = child_slabs(origin, side, rrd, bias);
        own = mine ? hit_mask(slabs) : 0u;
        if (COUNT && mine) loads += 8;
        if (side == lane_side) {
            lane_walk<COUNT, LEVELS>(a, words, own, origin, side, slabs, rrd, bias, total, loads);
            uni = 0;
        } else {
            leaves = __ballot_sync(0xFFFFFFFFu, a.is_leaf(words)) & 0xFFu;
            uni = __reduce_or_sync(0xFFFFFFFFu, own);
        }
    }
    return total;
}

template <bool COUNT, class Acc, int LEVELS = 1>
__global__ void __launch_bounds__(BLOCK_THREADS, 5) df_packet_kernel(Frame f, Acc a, Outputs o, float lane_side) {
    __shared__ float4 s_geo[(BLOCK_THREADS / 32) * STACK_DEPTH];
    __shared__ uint2 s_ns[(BLOCK_THREADS / 32) * STACK_DEPTH];
    __shared__ uint8_t s_mask[(BLOCK_THREADS / 32) * STACK_DEPTH * 32];
    fill_unorm_lut();
    const uint32_t warp = threadIdx.x >> 5;
    uint32_t ix, iy;
    const bool active = pixel_of_thread(f, ix, iy);
    const V3 rd = primary_ray(f, active ? ix : 0u, active ? iy : 0u);
    uint32_t loads = 0, err = 0;
    PacketStacksWarp ps{s_ns + warp * STACK_DEPTH, s_geo + warp * STACK_DEPTH, s_mask + warp * STACK_DEPTH * 32,
                        threadIdx.x & 31u};
    const V3 total = trace_df_packet<COUNT, Acc, PacketStacksWarp, LEVELS>(a, f.translation, rd, active, loads, err,
                                                                          ps, lane_side);
    if (active) write_outputs(f, o, ix, iy, total * voxel_emission_coeff(f, rd), loads, err);
}

// esvo and the masked svo-df with their stacks in shared memory (23.5 KB per
// block of 128).
// SHARED_BLOCK threads a block (16x16 pixels): on large octrees larger
// blocks measured faster (esvo on the 2048^3 gas field at 3840x2160: 99 vs 59
// Mrays/s with blocks of 128), with no change on small ones.
constexpr int SHARED_BLOCK = 256;

template <int TRAV, bool COUNT, class Acc>
__global__ void __launch_bounds__(SHARED_BLOCK) shared_stack_kernel(Frame f, Acc a, Outputs o) {
    __shared__ uint32_t s_a[STACK_DEPTH * SHARED_BLOCK];
    __shared__ uint32_t s_b[STACK_DEPTH * SHARED_BLOCK];
    fill_unorm_lut();
    uint32_t ix, iy;
    if (!pixel_of_thread_bt<SHARED_BLOCK>(f, ix, iy)) return;
    SharedStacks stk{s_a + threadIdx.x, s_b + threadIdx.x, SHARED_BLOCK};
    const V3 rd = primary_ray(f, ix, iy);
    uint32_t loads = 0, err = 0;
    V3 total;
    if constexpr (TRAV == XN_TRAV_ESVO) {
        // resources/esvo.comp:148-152
        V3 ro = f.translation + vs(1.0f);
        const float t0 = aabb_entry(vs(1.0f), vs(2.0f), ro, rd);
        ro = ro + rd * fmaxf(t0, 0.0f);
        total = trace_esvo<COUNT, Acc, SharedStacks>(a, ro, rd, loads, err, &stk);
    } else {
        total = trace_df_masked<COUNT, Acc, SharedStacks>(a, f.translation, rd, loads, err, &stk);
    }
    write_outputs(f, o, ix, iy, total * voxel_emission_coeff(f, rd), loads, err);
}

template <int TRAV, class Acc>
static void launch_svo_any(bool count, const Frame& f, const Acc& a, const Outputs& o, dim3 grid, cudaStream_t s) {
    if constexpr (TRAV == XN_TRAV_SVO_ROPE) {
        if (count) svo_rope_kernel<true, Acc><<<grid, BLOCK_THREADS, 0, s>>>(f, a, o);
        else svo_rope_kernel<false, Acc><<<grid, BLOCK_THREADS, 0, s>>>(f, a, o);
    } else {
        if (count) svo_kernel<TRAV, true, Acc><<<grid, BLOCK_THREADS, 0, s>>>(f, a, o);
        else svo_kernel<TRAV, false, Acc><<<grid, BLOCK_THREADS, 0, s>>>(f, a, o);
    }
}

template <class Acc>
static void launch_traversal(int traversal, bool count, const Frame& f, const Acc& a, const Outputs& o, dim3 grid,
                             cudaStream_t s) {
    switch (traversal) {
    case XN_TRAV_SVO_NAIVE: launch_svo_any<XN_TRAV_SVO_NAIVE>(count, f, a, o, grid, s); break;
    case XN_TRAV_SVO_NAIVE_ROOT: launch_svo_any<XN_TRAV_SVO_NAIVE_ROOT>(count, f, a, o, grid, s); break;
    case XN_TRAV_ESVO: launch_svo_any<XN_TRAV_ESVO>(count, f, a, o, grid, s); break;
    case XN_TRAV_SVO_DF: launch_svo_any<XN_TRAV_SVO_DF>(count, f, a, o, grid, s); break;
    case XN_TRAV_SVO_DF_MASKED: launch_svo_any<XN_TRAV_SVO_DF_MASKED>(count, f, a, o, grid, s); break;
    default: launch_svo_any<XN_TRAV_SVO_ROPE>(count, f, a, o, grid, s); break;
    }
}

cudaError_t launch_render(const RenderLaunch& L, cudaStream_t stream) {
    Frame f;
    f.forward = v3(L.forward[0], L.forward[1], L.forward[2]);
    f.up = v3(L.up[0], L.up[1], L.up[2]);
    f.translation = v3(L.translation[0], L.translation[1], L.translation[2]);
    f.voxel_ratio = v3(L.voxel_ratio[0], L.voxel_ratio[1], L.voxel_ratio[2]);
    f.aspect = L.aspect;
    f.emission_coeff = L.emission_coeff;
    f.out_x = L.out_x;
    f.out_y = L.out_y;
    f.out_w = L.out_w;
    f.out_h = L.out_h;
    f.disp_x = L.disp_x;
    f.disp_y = L.disp_y;
    f.disp_w = L.disp_w;
    f.disp_h = L.disp_h;
    Outputs o{static_cast<uint32_t*>(L.d_rgba), L.d_emission, L.d_loads, L.d_err_word};
    dim3 grid((L.out_w + TILE_W - 1) / TILE_W, (L.out_h + TILE_H - 1) / TILE_H);
    const bool count = L.d_loads != nullptr;
    if (L.traversal == XN_TRAV_DDA && L.tex) {
        const cudaTextureObject_t t = L.tex;
        const uint32_t x = L.dim[0], y = L.dim[1], z = L.dim[2];
        // XN_DDA_WARP_TILE = 4 / 16 / 32: warps of 4x8, 16x2 or 32x1 pixels
        // instead of 8x4 (which texels the lanes of a fetch share depends on it)
        const char* wt = std::getenv("XN_DDA_WARP_TILE");
        const uint32_t ww = wt ? (uint32_t)std::atoi(wt) : 8u;
        if (L.tex_normalized == TEX_NORM && L.grid_hybrid) {
            // XN_DDA_LSU_SHARE: one warp in this many reads the x-fastest copy
            const char* sh = std::getenv("XN_DDA_LSU_SHARE");
            const uint32_t share = sh && std::atoi(sh) > 0 ? (uint32_t)std::atoi(sh) : 4u;
            GridVol g{static_cast<const uchar4*>(L.grid), x, y, z, (uint64_t)x, (uint64_t)x * y};
            if (count) dda_hybrid_kernel<true><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, g, share, o);
            else dda_hybrid_kernel<false><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, g, share, o);
        } else if (L.tex_normalized == TEX_NORM && (ww == 4 || ww == 16 || ww == 32)) {
            const dim3 g2((L.out_w + 2 * ww - 1) / (2 * ww), (L.out_h + 2 * (32 / ww) - 1) / (2 * (32 / ww)));
            if (ww == 4) {
                if (count) dda_tex_kernel<true, true, 4><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
                else dda_tex_kernel<false, true, 4><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            } else if (ww == 16) {
                if (count) dda_tex_kernel<true, true, 16><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
                else dda_tex_kernel<false, true, 16><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            } else {
                if (count) dda_tex_kernel<true, true, 32><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
                else dda_tex_kernel<false, true, 32><<<g2, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            }
        } else if (L.tex_normalized == TEX_NORM) {
            if (count) dda_tex_kernel<true, TEX_NORM><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            else dda_tex_kernel<false, TEX_NORM><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
        } else if (L.tex_normalized == TEX_PACKED) {
            if (count) dda_tex_kernel<true, TEX_PACKED><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            else dda_tex_kernel<false, TEX_PACKED><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
        } else {
            if (count) dda_tex_kernel<true, false><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
            else dda_tex_kernel<false, false><<<grid, BLOCK_THREADS, 0, stream>>>(f, t, x, y, z, o);
        }
    } else if (L.traversal == XN_TRAV_DDA && L.grid_bricked) {
        const BrickGrid g{static_cast<const uint4*>(L.grid), L.dim[0], L.dim[1], L.dim[2], bricks_along(L.dim[0]),
                          bricks_along(L.dim[1])};
        if (count) dda_brick_kernel<true><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
        else dda_brick_kernel<false><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
    } else if (L.traversal == XN_TRAV_DDA) {
        GridVol g{static_cast<const uchar4*>(L.grid), L.dim[0], L.dim[1], L.dim[2], (uint64_t)L.dim[0],
                  (uint64_t)L.dim[0] * L.dim[1]};
        if (count) dda_kernel<true><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
        else dda_kernel<false><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
    } else if (L.traversal == XN_TRAV_ESVO && L.shared_stacks) {
        const dim3 grid16((L.out_w + 15) / 16, (L.out_h + SHARED_BLOCK / 16 - 1) / (SHARED_BLOCK / 16));
        if (L.layout == XN_LAYOUT_REFERENCE) {
            const RefNodes acc{static_cast<const uint32_t*>(L.nodes)};
            if (count) shared_stack_kernel<XN_TRAV_ESVO, true><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
            else shared_stack_kernel<XN_TRAV_ESVO, false><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
        } else {
            const CompactNodes acc{L.inner, L.inner_depth};
            if (count) shared_stack_kernel<XN_TRAV_ESVO, true><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
            else shared_stack_kernel<XN_TRAV_ESVO, false><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
        }
    } else if (L.traversal == XN_TRAV_SVO_DF && L.df_packet && L.layout == XN_LAYOUT_COMPACT && L.depth_consistent) {
        const CompactNodes acc{L.inner, L.inner_depth};
        if (L.df_lane_levels == 2) {
            if (count) df_packet_kernel<true, CompactNodes, 2><<<grid, BLOCK_THREADS, 0, stream>>>(f, acc, o, L.df_lane_side);
            else df_packet_kernel<false, CompactNodes, 2><<<grid, BLOCK_THREADS, 0, stream>>>(f, acc, o, L.df_lane_side);
        } else {
            if (count) df_packet_kernel<true><<<grid, BLOCK_THREADS, 0, stream>>>(f, acc, o, L.df_lane_side);
            else df_packet_kernel<false><<<grid, BLOCK_THREADS, 0, stream>>>(f, acc, o, L.df_lane_side);
        }
    } else if (L.traversal == XN_TRAV_SVO_DF && L.shared_stacks && L.layout == XN_LAYOUT_COMPACT &&
               L.depth_consistent) {
        const CompactNodes acc{L.inner, L.inner_depth};
        const dim3 grid16((L.out_w + 15) / 16, (L.out_h + SHARED_BLOCK / 16 - 1) / (SHARED_BLOCK / 16));
        if (count) shared_stack_kernel<XN_TRAV_SVO_DF_MASKED, true><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
        else shared_stack_kernel<XN_TRAV_SVO_DF_MASKED, false><<<grid16, SHARED_BLOCK, 0, stream>>>(f, acc, o);
    } else if (L.layout == XN_LAYOUT_REFERENCE) {
        launch_traversal(L.traversal, count, f, RefNodes{static_cast<const uint32_t*>(L.nodes)}, o, grid, stream);
    } else if (L.traversal == XN_TRAV_SVO_ROPE) {
        launch_traversal(L.traversal, count, f, RopeNodes{L.rinner, L.inner_depth, L.leaves}, o, grid, stream);
    } else {
        int trav = L.traversal == XN_TRAV_SVO_DF && L.depth_consistent ? XN_TRAV_SVO_DF_MASKED : L.traversal;
        if (trav == XN_TRAV_SVO_NAIVE && !L.naive_resume) trav = XN_TRAV_SVO_NAIVE_ROOT;
        launch_traversal(trav, count, f, CompactNodes{L.inner, L.inner_depth}, o, grid, stream);
    }
    return cudaGetLastError();
}

}  // namespace xn

// ------------------------------------------------------- persistent batch ---
//
// One launch renders many jobs (cameras x volumes x traversals x
// resolutions).  The jobs' warp tiles (tile_w x 32/tile_w pixels) form one
// sequence; resident warps take `chunk` tiles at a time from a global counter
// (one atomic per warp per chunk) until the sequence is exhausted, so uneven
// jobs balance across the SMs and small frames fill the GPU together.

namespace xn {

BatchJob make_batch_job(const RenderLaunch& L) {
    BatchJob j{};
    for (int i = 0; i < 3; ++i) {
        j.forward[i] = L.forward[i];
        j.up[i] = L.up[i];
        j.translation[i] = L.translation[i];
        j.voxel_ratio[i] = L.voxel_ratio[i];
        j.dim[i] = L.dim[i];
    }
    j.aspect = L.aspect;
    j.emission_coeff = L.emission_coeff;
    j.out_x = L.out_x;
    j.out_y = L.out_y;
    j.out_w = L.out_w;
    j.out_h = L.out_h;
    j.disp_x = L.disp_x;
    j.disp_y = L.disp_y;
    j.disp_w = L.disp_w;
    j.disp_h = L.disp_h;
    j.traversal = L.traversal;
    j.tex = L.tex;
    j.tex_normalized = L.tex_normalized;
    j.layout = L.traversal == XN_TRAV_DDA ? (L.tex ? 1 : L.grid_bricked ? 2 : 0) : L.layout;
    j.grid = L.grid;
    j.nodes = L.nodes;
    j.inner = L.inner;
    j.rinner = L.rinner;
    j.inner_depth = L.inner_depth;
    j.leaves = L.leaves;
    j.rgba = L.d_rgba;
    j.depth_consistent = L.depth_consistent;
    // the batch's svo-df form walks one level per lane (its blocks of up to
    // 1024 threads leave 64 registers a thread): child size 2^-D
    j.df_lane_side = L.df_lane_levels == 2 ? L.df_lane_side * 0.5f : L.df_lane_side;
    return j;
}

int batch_spec(const BatchJob& j) {
    if (j.traversal == XN_TRAV_DDA)
        return j.layout == 1 ? (j.tex_normalized == TEX_NORM ? XN_BATCH_DDA_TEX_NORM : XN_BATCH_DDA_TEX_RAW)
                             : XN_BATCH_ANY;
    if (j.layout != XN_LAYOUT_COMPACT) return XN_BATCH_ANY;
    switch (j.traversal) {
    case XN_TRAV_ESVO: return XN_BATCH_ESVO;
    case XN_TRAV_SVO_NAIVE: return XN_BATCH_NAIVE;
    case XN_TRAV_SVO_DF: return j.depth_consistent ? XN_BATCH_DF : XN_BATCH_ANY;
    case XN_TRAV_SVO_ROPE: return XN_BATCH_ROPE;
    default: return XN_BATCH_ANY;
    }
}

__device__ __forceinline__ Frame frame_of(const BatchJob& J) {
    Frame f;
    f.forward = v3(J.forward[0], J.forward[1], J.forward[2]);
    f.up = v3(J.up[0], J.up[1], J.up[2]);
    f.translation = v3(J.translation[0], J.translation[1], J.translation[2]);
    f.voxel_ratio = v3(J.voxel_ratio[0], J.voxel_ratio[1], J.voxel_ratio[2]);
    f.aspect = J.aspect;
    f.emission_coeff = J.emission_coeff;
    f.out_x = J.out_x;
    f.out_y = J.out_y;
    f.out_w = J.out_w;
    f.out_h = J.out_h;
    f.disp_x = J.disp_x;
    f.disp_y = J.disp_y;
    f.disp_w = J.disp_w;
    f.disp_h = J.disp_h;
    return f;
}

template <int TRAV, class Acc>
__device__ __forceinline__ V3 trace_svo_job(const Acc& a, const Frame& f, V3 rd, uint32_t& loads, uint32_t& err,
                                            SharedStacks* stk) {
    if (TRAV == XN_TRAV_ESVO) {
        V3 ro = f.translation + vs(1.0f);
        float t0 = aabb_entry(vs(1.0f), vs(2.0f), ro, rd);
        ro = ro + rd * fmaxf(t0, 0.0f);
        return trace_esvo<false, Acc, SharedStacks>(a, ro, rd, loads, err, stk);
    } else if (TRAV == XN_TRAV_SVO_NAIVE) {
        return trace_naive<false>(a, f.translation, rd, loads, err);
    } else if (TRAV == XN_TRAV_SVO_DF) {
        return trace_df<false>(a, f.translation, rd, loads, err);
    } else if (TRAV == XN_TRAV_SVO_DF_MASKED) {
        return trace_df_masked<false, Acc, SharedStacks>(a, f.translation, rd, loads, err, stk);
    }
    return trace_rope<false>(a, f.translation, rd, loads, err);
}

// One pixel of one job: the same arithmetic as the single-frame kernels.
__device__ __noinline__ uint32_t render_job_pixel(const BatchJob& J, uint32_t ix, uint32_t iy, uint32_t& err,
                                                  SharedStacks* stk) {
    const Frame f = frame_of(J);
    const V3 rd = primary_ray(f, ix, iy);
    uint32_t loads = 0;
    V3 color;
    if (J.traversal == XN_TRAV_DDA) {
        const uint32_t m = max(J.dim[0], max(J.dim[1], J.dim[2]));
        const float side = (float)m;
        const V3 ro = f.translation * side;
        const float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
        V3 total;
        if (J.layout == 1) {
            total = J.tex_normalized == TEX_NORM
                        ? trace_dda_tex<false, TEX_NORM>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err)
                    : J.tex_normalized == TEX_PACKED
                        ? trace_dda_tex<false, TEX_PACKED>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err)
                        : trace_dda_tex<false, TEX_RAW>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err);
        } else if (J.layout == 2) {
            const BrickGrid g{static_cast<const uint4*>(J.grid), J.dim[0], J.dim[1], J.dim[2], bricks_along(J.dim[0]),
                              bricks_along(J.dim[1])};
            total = trace_dda_brick<false>(g, ro, rd, loads, err);
        } else {
            GridVol g{static_cast<const uchar4*>(J.grid), J.dim[0], J.dim[1], J.dim[2], (uint64_t)J.dim[0],
                      (uint64_t)J.dim[0] * J.dim[1]};
            total = trace_dda<false>(g, ro, rd, loads, err);
        }
        color = total * ec;
    } else {
        V3 total;
        if (J.layout == XN_LAYOUT_REFERENCE) {
            RefNodes a{static_cast<const uint32_t*>(J.nodes)};
            switch (J.traversal) {
            case XN_TRAV_SVO_NAIVE: total = trace_svo_job<XN_TRAV_SVO_NAIVE>(a, f, rd, loads, err, stk); break;
            case XN_TRAV_ESVO: total = trace_svo_job<XN_TRAV_ESVO>(a, f, rd, loads, err, stk); break;
            case XN_TRAV_SVO_DF: total = trace_svo_job<XN_TRAV_SVO_DF>(a, f, rd, loads, err, stk); break;
            default: total = trace_svo_job<XN_TRAV_SVO_ROPE>(a, f, rd, loads, err, stk); break;
            }
        } else if (J.traversal == XN_TRAV_SVO_ROPE) {
            total = trace_svo_job<XN_TRAV_SVO_ROPE>(RopeNodes{J.rinner, J.inner_depth, J.leaves}, f, rd, loads, err,
                                                    stk);
        } else {
            CompactNodes a{J.inner, J.inner_depth};
            switch (J.traversal) {
            case XN_TRAV_SVO_NAIVE: total = trace_svo_job<XN_TRAV_SVO_NAIVE>(a, f, rd, loads, err, stk); break;
            case XN_TRAV_ESVO: total = trace_svo_job<XN_TRAV_ESVO>(a, f, rd, loads, err, stk); break;
            default:
                total = J.depth_consistent ? trace_svo_job<XN_TRAV_SVO_DF_MASKED>(a, f, rd, loads, err, stk)
                                           : trace_svo_job<XN_TRAV_SVO_DF>(a, f, rd, loads, err, stk);
                break;
            }
        }
        color = total * voxel_emission_coeff(f, rd);
    }
    return pack_rgba(color);
}

// One pixel of a job whose traversal and layout the whole batch shares
// (BatchSpec): that traversal inlined, the arithmetic of render_job_pixel.
// Called by every lane of a warp tile (active: the pixel is in the job's
// output); the svo-df form walks the tree with the whole warp.
template <int SPEC>
__device__ __forceinline__ uint32_t render_job_pixel_spec(const BatchJob& J, uint32_t ix, uint32_t iy, bool active,
                                                          uint32_t& err, SharedStacks* stk) {
    if constexpr (SPEC == XN_BATCH_DF) {
        const Frame f = frame_of(J);
        const V3 rd = primary_ray(f, active ? ix : 0u, active ? iy : 0u);
        const uint32_t lane = threadIdx.x & 31u;
        PacketStacksColumns ps{stk->a - lane, stk->b, stk->stride};
        uint32_t loads = 0;
        const V3 total = trace_df_packet<false>(CompactNodes{J.inner, J.inner_depth}, f.translation, rd, active,
                                                loads, err, ps, J.df_lane_side);
        return pack_rgba(total * voxel_emission_coeff(f, rd));
    }
    if constexpr (SPEC == XN_BATCH_ANY) {
        if (J.form == XN_BATCH_DF) return render_job_pixel_spec<XN_BATCH_DF>(J, ix, iy, active, err, stk);
    }
    if (!active) return 0u;
    if constexpr (SPEC == XN_BATCH_ANY) {
        // a mixed batch: the job's own inlined form, chosen per tile (every
        // lane of a warp tile has the same job); linear grids, reference
        // layouts and the literal svo-df go through the generic function
        switch (J.form) {
        case XN_BATCH_DDA_TEX_NORM: return render_job_pixel_spec<XN_BATCH_DDA_TEX_NORM>(J, ix, iy, true, err, stk);
        case XN_BATCH_DDA_TEX_RAW: return render_job_pixel_spec<XN_BATCH_DDA_TEX_RAW>(J, ix, iy, true, err, stk);
        case XN_BATCH_ESVO: return render_job_pixel_spec<XN_BATCH_ESVO>(J, ix, iy, true, err, stk);
        case XN_BATCH_NAIVE: return render_job_pixel_spec<XN_BATCH_NAIVE>(J, ix, iy, true, err, stk);
        case XN_BATCH_ROPE: return render_job_pixel_spec<XN_BATCH_ROPE>(J, ix, iy, true, err, stk);
        default: return render_job_pixel(J, ix, iy, err, stk);
        }
    } else {
        const Frame f = frame_of(J);
        const V3 rd = primary_ray(f, ix, iy);
        uint32_t loads = 0;
        V3 color;
        if constexpr (SPEC == XN_BATCH_DDA_TEX_NORM || SPEC == XN_BATCH_DDA_TEX_RAW) {
            const uint32_t m = max(J.dim[0], max(J.dim[1], J.dim[2]));
            const float side = (float)m;
            const V3 ro = f.translation * side;
            const float ec = __fdiv_rn(voxel_emission_coeff(f, rd), side);
            if (SPEC == XN_BATCH_DDA_TEX_NORM)
                color = trace_dda_tex<false, TEX_NORM>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err) * ec;
            else if (J.tex_normalized == TEX_PACKED)
                color = trace_dda_tex<false, TEX_PACKED>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err) * ec;
            else
                color = trace_dda_tex<false, TEX_RAW>(J.tex, J.dim[0], J.dim[1], J.dim[2], ro, rd, loads, err) * ec;
        } else if constexpr (SPEC == XN_BATCH_ROPE) {
            color = trace_svo_job<XN_TRAV_SVO_ROPE>(RopeNodes{J.rinner, J.inner_depth, J.leaves}, f, rd, loads, err,
                                                    stk) *
                    voxel_emission_coeff(f, rd);
        } else {
            constexpr int TRAV = SPEC == XN_BATCH_ESVO ? XN_TRAV_ESVO
                                 : SPEC == XN_BATCH_NAIVE ? XN_TRAV_SVO_NAIVE
                                                          : XN_TRAV_SVO_DF_MASKED;
            color = trace_svo_job<TRAV>(CompactNodes{J.inner, J.inner_depth}, f, rd, loads, err, stk) *
                    voxel_emission_coeff(f, rd);
        }
        return pack_rgba(color);
    }
}

// The texture-DDA forms are held to 32 registers (two blocks of 1024 per SM):
// DDA hides texture latency with resident warps.
constexpr int batch_min_blocks(int spec) {
    return spec == XN_BATCH_DDA_TEX_NORM || spec == XN_BATCH_DDA_TEX_RAW ? 2 : 1;
}

template <int TW, int SPEC>
__global__ void __launch_bounds__(1024, batch_min_blocks(SPEC)) batch_kernel(const BatchHeader* hdr, const BatchJob* jobs,
                                                     unsigned long long* queue, uint32_t chunk, uint32_t* err_word) {
    fill_unorm_lut();
    constexpr int TH = 32 / TW;
    // esvo and svo-df stacks: two columns per thread in dynamic shared memory
    // (2 * STACK_DEPTH words a thread, given at launch for the forms that use them)
    extern __shared__ uint32_t batch_stacks[];
    SharedStacks stk{batch_stacks + threadIdx.x, batch_stacks + STACK_DEPTH * blockDim.x + threadIdx.x, blockDim.x};
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long total = hdr->total_tiles;
    const uint32_t n = hdr->n_jobs;
    uint32_t err = 0;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(queue, (unsigned long long)chunk);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total) break;
        const unsigned long long end = base + chunk < total ? base + chunk : total;
        for (unsigned long long t = base; t < end; ++t) {
            uint32_t lo = 0, hi = n;  // last job whose first tile is <= t
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (jobs[mid].tile_begin <= t) lo = mid;
                else hi = mid;
            }
            const BatchJob& J = jobs[lo];
            const unsigned long long local = t - J.tile_begin;
            const uint32_t ty = (uint32_t)(local / J.tiles_x);
            const uint32_t tx = (uint32_t)(local - (unsigned long long)ty * J.tiles_x);
            const uint32_t ix = tx * TW + lane % TW, iy = ty * TH + lane / TW;
            const bool active = ix < J.out_w && iy < J.out_h;
            const uint32_t px = render_job_pixel_spec<SPEC>(J, ix, iy, active, err, &stk);
            if (active) static_cast<uint32_t*>(J.rgba)[(uint64_t)iy * J.out_w + ix] = px;
        }
    }
    if (err) atomicOr(err_word, err);
}

// The queue-less form of the batch kernel (chunk 0): a grid with one warp
// per tile of every job, in tile order; the hardware block scheduler
// balances the load.  Same per-pixel arithmetic as batch_kernel.
template <int TW, int SPEC>
__global__ void __launch_bounds__(1024, batch_min_blocks(SPEC)) batch_grid_kernel(const BatchHeader* hdr, const BatchJob* jobs,
                                                          uint32_t* err_word) {
    fill_unorm_lut();
    constexpr int TH = 32 / TW;
    extern __shared__ uint32_t batch_stacks[];
    SharedStacks stk{batch_stacks + threadIdx.x, batch_stacks + STACK_DEPTH * blockDim.x + threadIdx.x, blockDim.x};
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long t =
        (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= hdr->total_tiles) return;
    uint32_t lo = 0, hi = hdr->n_jobs;  // last job whose first tile is <= t
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].tile_begin <= t) lo = mid;
        else hi = mid;
    }
    const BatchJob& J = jobs[lo];
    const unsigned long long local = t - J.tile_begin;
    const uint32_t ty = (uint32_t)(local / J.tiles_x);
    const uint32_t tx = (uint32_t)(local - (unsigned long long)ty * J.tiles_x);
    const uint32_t ix = tx * TW + lane % TW, iy = ty * TH + lane / TW;
    const bool active = ix < J.out_w && iy < J.out_h;
    uint32_t err = 0;
    const uint32_t px = render_job_pixel_spec<SPEC>(J, ix, iy, active, err, &stk);
    if (active) static_cast<uint32_t*>(J.rgba)[(uint64_t)iy * J.out_w + ix] = px;
    if (err) atomicOr(err_word, err);
}

constexpr bool batch_needs_stacks(int spec) {
    return spec == XN_BATCH_ANY || spec == XN_BATCH_ESVO || spec == XN_BATCH_DF;
}

template <int TW, int SPEC>
static cudaError_t launch_batch_tws(const void* table, unsigned long long* q, uint32_t* err, uint32_t threads,
                                    uint32_t blocks, uint32_t chunk, cudaStream_t s) {
    const BatchHeader* hdr = static_cast<const BatchHeader*>(table);
    const BatchJob* jobs = reinterpret_cast<const BatchJob*>(hdr + 1);
    const size_t smem = batch_needs_stacks(SPEC) ? (size_t)2 * STACK_DEPTH * 4 * threads : 0;
    if (chunk == 0) {
        // queue-less form: one warp per tile; `blocks` is the grid for all tiles
        if (smem > 48 * 1024) {
            const cudaError_t e =
                cudaFuncSetAttribute(batch_grid_kernel<TW, SPEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        batch_grid_kernel<TW, SPEC><<<blocks, threads, smem, s>>>(hdr, jobs, err);
        return cudaGetLastError();
    }
    if (smem > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(batch_kernel<TW, SPEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    batch_kernel<TW, SPEC><<<blocks, threads, smem, s>>>(hdr, jobs, q, chunk, err);
    return cudaGetLastError();
}

template <int TW>
static cudaError_t launch_batch_tw(const void* table, unsigned long long* q, uint32_t* err, uint32_t threads,
                                   uint32_t blocks, uint32_t chunk, int spec, cudaStream_t s) {
    switch (spec) {
    case XN_BATCH_DDA_TEX_NORM: return launch_batch_tws<TW, XN_BATCH_DDA_TEX_NORM>(table, q, err, threads, blocks, chunk, s);
    case XN_BATCH_DDA_TEX_RAW: return launch_batch_tws<TW, XN_BATCH_DDA_TEX_RAW>(table, q, err, threads, blocks, chunk, s);
    case XN_BATCH_ESVO: return launch_batch_tws<TW, XN_BATCH_ESVO>(table, q, err, threads, blocks, chunk, s);
    case XN_BATCH_NAIVE: return launch_batch_tws<TW, XN_BATCH_NAIVE>(table, q, err, threads, blocks, chunk, s);
    case XN_BATCH_DF: return launch_batch_tws<TW, XN_BATCH_DF>(table, q, err, threads, blocks, chunk, s);
    case XN_BATCH_ROPE: return launch_batch_tws<TW, XN_BATCH_ROPE>(table, q, err, threads, blocks, chunk, s);
    default: return launch_batch_tws<TW, XN_BATCH_ANY>(table, q, err, threads, blocks, chunk, s);
    }
}

cudaError_t launch_batch(const void* table, unsigned long long* q, uint32_t* err, uint32_t tile_w,
                         uint32_t threads, uint32_t blocks, uint32_t chunk, int spec, cudaStream_t s) {
    switch (tile_w) {
    case 4: return launch_batch_tw<4>(table, q, err, threads, blocks, chunk, spec, s);
    case 16: return launch_batch_tw<16>(table, q, err, threads, blocks, chunk, spec, s);
    case 32: return launch_batch_tw<32>(table, q, err, threads, blocks, chunk, spec, s);
    default: return launch_batch_tw<8>(table, q, err, threads, blocks, chunk, spec, s);
    }
}

// ------------------------------------------------------------ folding ring ---
//
// The persistent kernel of the render server: jobs arrive while it runs.  The
// host appends a job to a ring in device memory and then raises the published
// tile count (two copies in one stream, so a count is never visible before the
// jobs it covers); ring slots not yet written hold tile_begin = ~0, so the
// binary search over the whole ring finds only published jobs.  A warp claims
// the next published tile with a compare-and-swap (never past the count),
// renders it with the batch kernel's per-pixel code, and counts it done; the
// warp that completes a job raises the job's flag in mapped host memory.
// Every wait is bounded: a warp that finds nothing to claim sleeps (1 us,
// doubling to 32 us while nothing comes) and looks again.  A warp that has
// found nothing for idle_ns raises the exit flag (status bit 0); from then on
// no warp claims a tile, so the kernel leaves as soon as the tiles in hand are
// done (were claims still taken, the warps that momentarily found nothing
// would leave one by one while the rest kept taking newly published jobs, and
// a kernel down to a few warps would hold the ring).  The decision is also
// written to the flag after the ring's done flags in mapped host memory, so
// the host publishes new jobs to the other ring at once.  A closed ring is
// drained: every published tile is taken before the warps leave.  Jobs left
// unfinished are found so by the host when the kernel has ended and are
// published again to the next launch; re-rendering a tile writes the same
// pixels.
//
// The polls are relaxed loads and the ring slots are read around L1 (.cg):
// an acquire load would invalidate the SM's L1 on every poll, which the
// single-frame kernels running beside this one depend on.  The slot reads
// depend on the claimed tile number, which depends on the count read, so they
// are issued after it; the copy of a slot completed before the copy of the
// count that covers it began.

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// A ring slot copied by the warp into its shared-memory job, read around L1:
// an L1 line can hold part of a neighbouring slot from before that slot was
// published.
__device__ __forceinline__ void load_job_cg(const BatchJob* src, BatchJob* dst, uint32_t lane) {
    static_assert(sizeof(BatchJob) % 16 == 0 && sizeof(BatchJob) / 16 <= 32, "ring slots are read in 16-byte pieces");
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    if (lane < sizeof(BatchJob) / 16) d[lane] = __ldcg(s + lane);
    __syncwarp();
}

// Blocks of THREADS (32 or 128) threads: a one-warp block needs a quarter of
// the registers and shared memory of a four-warp one, so it also fits where
// a large frame's retiring block freed little.
template <int TW, uint32_t THREADS>
__global__ void __launch_bounds__(THREADS, 512 / THREADS) fold_kernel(FoldCtl* ctl, const BatchJob* ring, uint32_t cap,
                                                            uint32_t* done_tiles, volatile uint32_t* done_flags,
                                                            uint32_t* err_word, unsigned long long idle_ns) {
    fill_unorm_lut();
    __shared__ BatchJob s_job[THREADS / 32];
    constexpr int TH = 32 / TW;
    extern __shared__ uint32_t batch_stacks[];
    SharedStacks stk{batch_stacks + threadIdx.x, batch_stacks + STACK_DEPTH * blockDim.x + threadIdx.x, blockDim.x};
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t err = 0;
    unsigned long long idle_since = global_ns();
    uint32_t backoff = 1000;  // ns
    // every pass claims a tile, sleeps, or exits; the pass count is bounded
    // as well
    for (uint32_t pass = 0; pass < (1u << 30); ++pass) {
        unsigned long long t = ~0ull;
        int quit = 0;
        if (lane == 0) {
            if (ld_relaxed_u32(&ctl->exit_flag)) {
                quit = 1;  // the kernel is leaving: no new claims
            } else {
                const unsigned long long pub = ld_relaxed_u64(&ctl->published);
                unsigned long long cur = ld_relaxed_u64(&ctl->taken);
                while (cur < pub) {
                    const unsigned long long prev = atomicCAS(&ctl->taken, cur, cur + 1);
                    if (prev == cur) {
                        t = cur;
                        break;
                    }
                    cur = prev;
                }
                if (t == ~0ull) {
                    if (ld_relaxed_u32(&ctl->closed)) {
                        quit = 1;
                    } else if (global_ns() - idle_since > idle_ns) {
                        atomicExch(&ctl->exit_flag, 1u);
                        atomicOr(&ctl->status, 1u);
                        done_flags[cap] = 1u;  // the host stops publishing to this ring
                        quit = 1;
                    }
                }
            }
        }
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        quit = __shfl_sync(0xFFFFFFFFu, quit, 0);
        if (quit) break;
        if (t == ~0ull) {
            __nanosleep(backoff);
            backoff = backoff < 32000u ? backoff * 2u : 32000u;
            continue;
        }
        backoff = 1000;
        // the slot of tile t: the last job whose first tile is <= t
        uint32_t lo = 0, hi = cap;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldcg(&ring[mid].tile_begin) <= t) lo = mid;
            else hi = mid;
        }
        BatchJob& J = s_job[threadIdx.x >> 5];
        __syncwarp();  // the previous tile's reads of this warp's job are done
        load_job_cg(ring + lo, &J, lane);
        const unsigned long long local = t - J.tile_begin;
        if (local >= (unsigned long long)J.tiles_x * J.tiles_y || !J.rgba) {
            // cannot happen with the publication order above; the job is left
            // unfinished (the host renders it again) rather than written astray
            err |= 4u;
            idle_since = global_ns();
            continue;
        }
        const uint32_t ty = (uint32_t)(local / J.tiles_x);
        const uint32_t tx = (uint32_t)(local - (unsigned long long)ty * J.tiles_x);
        const uint32_t ix = tx * TW + lane % TW, iy = ty * TH + lane / TW;
        const bool active = ix < J.out_w && iy < J.out_h;
        const uint32_t px = render_job_pixel_spec<XN_BATCH_ANY>(J, ix, iy, active, err, &stk);
        if (active) static_cast<uint32_t*>(J.rgba)[(uint64_t)iy * J.out_w + ix] = px;
        __threadfence();  // this tile's pixels before its count
        __syncwarp();
        if (lane == 0) {
            const uint32_t n = atomicAdd(&done_tiles[lo], 1u) + 1u;
            if ((unsigned long long)n == (unsigned long long)J.tiles_x * J.tiles_y) {
                __threadfence_system();
                done_flags[lo] = 1u;
            }
        }
        idle_since = global_ns();
    }
    if (err) atomicOr(err_word, err);
}

cudaError_t launch_fold(FoldCtl* ctl, const BatchJob* ring, uint32_t cap, uint32_t* done_tiles,
                        uint32_t* done_flags_mapped, uint32_t* err, uint32_t tile_w, uint32_t threads, uint32_t blocks,
                        unsigned long long idle_ns, cudaStream_t s) {
    if (threads != 32 && threads != 128) return cudaErrorInvalidValue;
    const size_t smem = (size_t)2 * STACK_DEPTH * 4 * threads;
    if (tile_w == 4 && threads == 32)
        fold_kernel<4, 32><<<blocks, 32, smem, s>>>(ctl, ring, cap, done_tiles, done_flags_mapped, err, idle_ns);
    else if (tile_w == 4)
        fold_kernel<4, 128><<<blocks, 128, smem, s>>>(ctl, ring, cap, done_tiles, done_flags_mapped, err, idle_ns);
    else if (threads == 32)
        fold_kernel<8, 32><<<blocks, 32, smem, s>>>(ctl, ring, cap, done_tiles, done_flags_mapped, err, idle_ns);
    else
        fold_kernel<8, 128><<<blocks, 128, smem, s>>>(ctl, ring, cap, done_tiles, done_flags_mapped, err, idle_ns);
    return cudaGetLastError();
}

// Resident blocks per SM of the generic kernel with its stacks (the most
// demanding of the forms, so the specialised ones fit the same grid).
int batch_kernel_blocks_per_sm(uint32_t tile_w, uint32_t threads) {
    int n = 0;
    const size_t smem = (size_t)2 * STACK_DEPTH * 4 * threads;
    cudaError_t e;
    switch (tile_w) {
    case 4: e = cudaFuncSetAttribute(batch_kernel<4, XN_BATCH_ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<4, XN_BATCH_ANY>, (int)threads, smem);
        break;
    case 16: e = cudaFuncSetAttribute(batch_kernel<16, XN_BATCH_ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<16, XN_BATCH_ANY>, (int)threads, smem);
        break;
    case 32: e = cudaFuncSetAttribute(batch_kernel<32, XN_BATCH_ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<32, XN_BATCH_ANY>, (int)threads, smem);
        break;
    default: e = cudaFuncSetAttribute(batch_kernel<8, XN_BATCH_ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<8, XN_BATCH_ANY>, (int)threads, smem);
        break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace xn

