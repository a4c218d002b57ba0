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
        bool mx = side.x <= fminf(side.y, side.z);
        bool my = side.y <= fminf(side.z, side.x);
        bool mz = side.z <= fminf(side.x, side.y);
        float t0 = min_elem(side);
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

// resources/svo_naive.comp:29-71
template <bool COUNT, class Acc>
__device__ V3 trace_naive(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
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
    while (t < t_max) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        V3 p = rd * t + ro;
        V3 offset;
        float side;
        uint32_t node = find<COUNT>(a, p, offset, side, loads, err);
        V3 node_min = offset * rrd - bias;
        V3 node_max = (offset + vs(side)) * rrd - bias;
        float u_min = max_elem(vmin(node_min, node_max));
        float u_max = min_elem(vmax(node_min, node_max));
        u_min = fmaxf(u_min, 0.0f);
        float step = fmaxf(u_max - u_min, MIN_STEP);
        t += step;
        V3 color = unpack_rgb(a.color(node));
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
                V3 color = unpack_rgb(a.color(child));
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
        float s2 = side * 2.0f;
        pos = pos - v3(gl_mod(pos.x, s2), gl_mod(pos.y, s2), gl_mod(pos.z, s2));
        ++child_idx;
        if (child_idx & 4u) pos.x = pos.x + side;
        if (child_idx & 2u) pos.y = pos.y + side;
        if (child_idx & 1u) pos.z = pos.z + side;
    }
    return total;
}

__device__ __forceinline__ uint32_t cxor(uint32_t x, bool ax, bool ay, bool az) {
    return x ^ (ax ? 4u : 0u) ^ (ay ? 2u : 0u) ^ (az ? 1u : 0u);
}

// resources/esvo.comp:30-136
template <bool COUNT, class Acc>
__device__ V3 trace_esvo(const Acc& a, V3 ro, V3 rd, uint32_t& loads, uint32_t& err) {
    const uint32_t depth = STACK_DEPTH;
    uint32_t node_stack[STACK_DEPTH];
    float t_max_stack[STACK_DEPTH];
#pragma unroll
    for (int i = 0; i < STACK_DEPTH; ++i) { node_stack[i] = 0; t_max_stack[i] = 0.0f; }

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
    uint32_t iter = 0;
    while (scale < depth) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        V3 t_corner = pos * t_coeff - t_bias;
        float tc_max = min_elem(t_corner);
        if (t_min <= t_max) {
            float tv_max = fminf(t_max, tc_max);
            if (t_min <= tv_max) {
                uint32_t child = a.child(parent, idx ^ octant_mask);
                if (COUNT) loads += 2;
                if (a.is_leaf(child)) {
                    V3 color = unpack_rgb(a.color(child));
                    if (COUNT) ++loads;
                    total = total + color * (tv_max - t_min);
                } else {
                    if (tc_max < h) {
                        node_stack[scale] = parent;
                        t_max_stack[scale] = t_max;
                    }
                    h = tc_max;
                    parent = child;
                    --scale;
                    scale_exp2 *= 0.5f;
                    V3 t_center = t_coeff * scale_exp2 + t_corner;
                    bool ax = t_center.x > t_min, ay = t_center.y > t_min, az = t_center.z > t_min;
                    idx = cxor(0u, ax, ay, az);
                    if (ax) pos.x = pos.x + scale_exp2;
                    if (ay) pos.y = pos.y + scale_exp2;
                    if (az) pos.z = pos.z + scale_exp2;
                    t_max = tv_max;
                    continue;
                }
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
            uint32_t xx = __float_as_uint(pos.x) ^ __float_as_uint(pos.x + scale_exp2);
            uint32_t xy = __float_as_uint(pos.y) ^ __float_as_uint(pos.y + scale_exp2);
            uint32_t xz = __float_as_uint(pos.z) ^ __float_as_uint(pos.z + scale_exp2);
            uint32_t dbits = (ax ? xx : 0u) | (ay ? xy : 0u) | (az ? xz : 0u);
            scale = (__float_as_uint(__uint2float_rn(dbits)) >> 23) - 127u;
            if (scale >= depth) break;  // the loop condition ends the ray
            scale_exp2 = __uint_as_float((scale - depth + 127u) << 23);
            parent = node_stack[scale];
            t_max = t_max_stack[scale];
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
    float extent = ldexpf(1.0f, -(int)(d > 1000u ? 1000u : d));
    offset = v3(offset.x - gl_mod(offset.x, extent), offset.y - gl_mod(offset.y, extent),
                offset.z - gl_mod(offset.z, extent));
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

// resources/svo_rope.comp:50-63
__device__ __forceinline__ uint32_t neighbor_index(uint32_t nx, uint32_t ny, uint32_t nz, V3 far, V3& mask) {
    if (far.x < fminf(far.y, far.z)) { mask = v3(1.f, 0.f, 0.f); return nx; }
    if (far.y < far.z) { mask = v3(0.f, 1.f, 0.f); return ny; }
    mask = v3(0.f, 0.f, 1.f);
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
    V3 color = unpack_rgb(a.color(node));
    V3 total = color * step;
    V3 mask;
    uint32_t n = neighbor_index(nbx, nby, nbz, far, mask);
    node = a.child(node, n);
    if (COUNT) loads += 2;
    offset = offset + (mask * sgn) * side;
    uint32_t iter = 0;
    while (node != 0) {
        if (++iter > SVO_MAX_ITER) { err |= 1u; break; }
        pos = ro + rd * u_max;
        node = find_relative<COUNT>(a, node, offset, pos, offset, side, loads, err);
        node_min = offset * rrd - bias;
        node_max = (offset + vs(side)) * rrd - bias;
        far = vmax(node_min, node_max);
        u_min = max_elem(vmin(node_min, node_max));
        u_max = min_elem(far);
        step = u_max - fmaxf(u_min, 0.0f);
        color = unpack_rgb(a.color(node));
        total = total + color * step;
        n = neighbor_index(nbx, nby, nbz, far, mask);
        node = a.child(node, n);
        if (COUNT) loads += 2;
        offset = offset + (mask * sgn) * side;
    }
    return total;
}

// esvo.comp:10-21
__device__ __forceinline__ float aabb_entry(V3 bmin, V3 bmax, V3 ro, V3 rd) {
    V3 rrd = vs(1.0f) / (rd + vs(0.00000001f));
    V3 tbot = (bmin - ro) * rrd;
    V3 ttop = (bmax - ro) * rrd;
    V3 tmin = vmin(ttop, tbot);
    return fmaxf(fmaxf(tmin.x, tmin.y), fmaxf(tmin.x, tmin.z));
}

// ---------------------------------------------------------------- kernels ---

constexpr int TILE_W = 16;  // block covers 16x8 pixels: 2x2 warps of 8x4
constexpr int TILE_H = 8;
constexpr int BLOCK_THREADS = TILE_W * TILE_H;

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

template <int TRAV, bool COUNT, class Acc>
__global__ void __launch_bounds__(BLOCK_THREADS) svo_kernel(Frame f, Acc a, Outputs o) {
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
    } else if (TRAV == XN_TRAV_SVO_NAIVE) {
        total = trace_naive<COUNT>(a, f.translation, rd, loads, err);
    } else if (TRAV == XN_TRAV_SVO_DF) {
        total = trace_df<COUNT>(a, f.translation, rd, loads, err);
    } else {
        total = trace_rope<COUNT>(a, f.translation, rd, loads, err);
    }
    V3 color = total * voxel_emission_coeff(f, rd);
    write_outputs(f, o, ix, iy, color, loads, err);
}

template <int TRAV, bool COUNT>
static void launch_svo(const Frame& f, const RefNodes& a, const Outputs& o, dim3 grid, cudaStream_t s) {
    svo_kernel<TRAV, COUNT, RefNodes><<<grid, BLOCK_THREADS, 0, s>>>(f, a, o);
}

template <int TRAV>
static void launch_svo_any(bool count, const Frame& f, const RefNodes& a, const Outputs& o, dim3 grid,
                           cudaStream_t s) {
    if (count) launch_svo<TRAV, true>(f, a, o, grid, s);
    else launch_svo<TRAV, false>(f, a, o, grid, s);
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
    if (L.traversal == XN_TRAV_DDA) {
        GridVol g{static_cast<const uchar4*>(L.grid), L.dim[0], L.dim[1], L.dim[2], (uint64_t)L.dim[0],
                  (uint64_t)L.dim[0] * L.dim[1]};
        if (count) dda_kernel<true><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
        else dda_kernel<false><<<grid, BLOCK_THREADS, 0, stream>>>(f, g, o);
    } else {
        RefNodes a{static_cast<const uint32_t*>(L.nodes)};
        switch (L.traversal) {
        case XN_TRAV_SVO_NAIVE: launch_svo_any<XN_TRAV_SVO_NAIVE>(count, f, a, o, grid, stream); break;
        case XN_TRAV_ESVO: launch_svo_any<XN_TRAV_ESVO>(count, f, a, o, grid, stream); break;
        case XN_TRAV_SVO_DF: launch_svo_any<XN_TRAV_SVO_DF>(count, f, a, o, grid, stream); break;
        default: launch_svo_any<XN_TRAV_SVO_ROPE>(count, f, a, o, grid, stream); break;
        }
    }
    return cudaGetLastError();
}

}  // namespace xn
