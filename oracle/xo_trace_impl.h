/*
 * Oracle (test infrastructure only): restatement of the five Xenodon traversal
 * shaders in C with GLSL semantics.  Included by xo_trace_f32.c and
 * xo_trace_f64.c with XO_REAL set to float or double; the FP64 build is the
 * per-ray emission re-trace, the FP32 build is the image oracle and the timed
 * CPU baseline.
 *
 * GLSL semantics made explicit here (and matched by the CUDA kernels):
 *   - no fused multiply-add anywhere (compile with -ffp-contract=off);
 *   - a*b+c is (a*b)+c, dot(a,b) is (a.x*b.x + a.y*b.y) + a.z*b.z;
 *   - normalize(v) = v / sqrt(dot(v, v)), IEEE division and square root;
 *   - mod(x, y) = x - y*floor(x/y);
 *   - unpackUnorm4x8 / UNORM texel reads: byte/255 correctly rounded;
 *   - the RGBA8 UNORM store: floor(clamp(x, 0, 1)*255 + 0.5), alpha 255;
 *   - an out-of-range texelFetch (undefined in Vulkan) reads 0.
 * Loops that the shaders leave unbounded get iteration caps; a ray that hits a
 * cap or overflows a traversal stack sets an error bit (the shader's behaviour
 * there is undefined).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "xo.h"

typedef XO_REAL R;

typedef struct { R x, y, z; } V3;

#define XO_DDA_ITER_EXTRA 64
#define XO_SVO_MAX_ITER (1u << 22)
#define XO_FIND_MAX_DEPTH 64
#define XO_STACK_DEPTH 23 /* FLOAT_MANTISSA_BITS, resources/common.glsl:37 */

static inline V3 v3(R x, R y, R z) { V3 r = {x, y, z}; return r; }
static inline V3 vs(R s) { return v3(s, s, s); }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vmul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 vdiv(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline V3 vscale(V3 a, R s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline R rmin(R a, R b) { return (b < a) ? b : a; } /* GLSL min */
static inline R rmax(R a, R b) { return (a < b) ? b : a; } /* GLSL max */
static inline V3 vmin(V3 a, V3 b) { return v3(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); }
static inline V3 vmax(V3 a, V3 b) { return v3(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }
static inline R min_elem(V3 v) { return rmin(v.x, rmin(v.y, v.z)); } /* common.glsl:58-60 */
static inline R max_elem(V3 v) { return rmax(v.x, rmax(v.y, v.z)); } /* common.glsl:62-64 */
static inline R rdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 vcross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline V3 vnormalize(V3 v) {
    R l = sizeof(R) == 4 ? (R)sqrtf((float)rdot(v, v)) : (R)sqrt((double)rdot(v, v));
    return v3(v.x / l, v.y / l, v.z / l);
}
static inline R rfloor(R x) { return sizeof(R) == 4 ? (R)floorf((float)x) : (R)floor((double)x); }
static inline R rsqrt1(R x) { return sizeof(R) == 4 ? (R)sqrtf((float)x) : (R)sqrt((double)x); }
static inline R rabs(R x) { return x < 0 ? -x : x; }
static inline R rsign(R x) { return x > 0 ? (R)1 : (x < 0 ? (R)-1 : (R)0); }
static inline R rmod(R x, R y) { return x - y * rfloor(x / y); }
/* float -> int truncation; out-of-range values (never used by the shaders)
 * are clamped so the conversion is defined on every host. */
static inline int32_t f2i(R x) {
    if (!(x > (R)-1073741824.0)) return -1073741824;
    if (!(x < (R)1073741824.0)) return 1073741824;
    return (int32_t)x;
}
static inline R unorm8f(uint32_t c) { return sizeof(R) == 4 ? (R)((float)c / 255.0f) : (R)c / (R)255.0; }

/* common.glsl:40-43 */
static inline V3 adjust_ray(V3 rd) {
    const R eps = (R)(1.0f / 8388608.0f); /* exp2(-23) */
    V3 r = rd;
    if (rabs(r.x) < eps) r.x = eps;
    if (rabs(r.y) < eps) r.y = eps;
    if (rabs(r.z) < eps) r.z = eps;
    return r;
}

typedef struct {
    V3 fwd, up, ratio;
    R aspect; /* display extent.y / extent.x */
    R ec;     /* emission coefficient */
} RaySetup;

/* common.glsl:45-56, uv from dda.comp:62-63 */
static inline V3 ray_dir(const RaySetup* s, const xo_view* v, int32_t px, int32_t py) {
    R u = (R)(px - v->display_offset[0]) / (R)v->display_extent[0];
    R w = (R)(py - v->display_offset[1]) / (R)v->display_extent[1];
    u -= (R)0.5f;
    w -= (R)0.5f;
    w *= s->aspect;
    V3 right = vnormalize(vcross(s->up, s->fwd));
    V3 up = vnormalize(vcross(right, s->fwd));
    V3 rd = vnormalize(vadd(vadd(vscale(right, u), vscale(up, w)), s->fwd));
    return adjust_ray(vnormalize(vdiv(rd, s->ratio)));
}

/* common.glsl:68-72 */
static inline R voxel_emission_coeff(const RaySetup* s, V3 rd) {
    V3 rd2 = vmul(rd, rd);
    V3 dim2 = vmul(s->ratio, s->ratio);
    return s->ec * rsqrt1(rdot(rd2, dim2) / rdot(rd2, vs((R)1)));
}

typedef struct {
    const xo_volume* vol;
    uint32_t loads;
    uint8_t err;
} Ctx;

/* ---------------------------------------------------------------- DDA --- */

static inline V3 texel(Ctx* c, int32_t x, int32_t y, int32_t z) {
    const xo_volume* vol = c->vol;
    c->loads++;
    if (x < 0 || y < 0 || z < 0 || (uint32_t)x >= vol->dim[0] || (uint32_t)y >= vol->dim[1] ||
        (uint32_t)z >= vol->dim[2])
        return vs((R)0);
    uint64_t i = (uint64_t)x + (uint64_t)y * vol->dim[0] + (uint64_t)z * vol->dim[0] * vol->dim[1];
    const uint8_t* p = vol->rgba + 4 * i;
    return v3(unorm8f(p[0]), unorm8f(p[1]), unorm8f(p[2]));
}

/* dda.comp:13-53 */
static V3 trace_dda(Ctx* c, V3 ro, V3 rd) {
    const xo_volume* vol = c->vol;
    V3 rrd = vdiv(vs((R)1), rd);
    V3 bias = vmul(rrd, ro);
    V3 box_min = v3(-bias.x, -bias.y, -bias.z);
    V3 md = v3((R)vol->dim[0], (R)vol->dim[1], (R)vol->dim[2]);
    V3 box_max = vsub(vmul(md, rrd), bias);
    R t_min = max_elem(vmin(box_min, box_max));
    R t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs((R)0);
    t_min = rmax(t_min, (R)0);
    ro = vadd(ro, vscale(rd, t_min));
    int32_t pos[3] = {f2i(ro.x), f2i(ro.y), f2i(ro.z)};
    V3 t_delta = v3(rabs(rrd.x), rabs(rrd.y), rabs(rrd.z));
    V3 sgn = v3(rsign(rd.x), rsign(rd.y), rsign(rd.z));
    int32_t step[3] = {(int32_t)sgn.x, (int32_t)sgn.y, (int32_t)sgn.z};
    V3 fr = vadd(vsub(v3(rfloor(ro.x), rfloor(ro.y), rfloor(ro.z)), ro), vs((R)0.5f));
    V3 side = vmul(vadd(vmul(sgn, fr), vs((R)0.5f)), t_delta);
    R t = 0;
    V3 total = vs((R)0);
    const uint64_t cap = 2ull * ((uint64_t)vol->dim[0] + vol->dim[1] + vol->dim[2]) + XO_DDA_ITER_EXTRA;
    uint64_t iter = 0;
    while (t < t_max - t_min) {
        if (++iter > cap) { c->err |= XO_ERR_ITER; break; }
        int mx = side.x <= rmin(side.y, side.z);
        int my = side.y <= rmin(side.z, side.x);
        int mz = side.z <= rmin(side.x, side.y);
        R t0 = min_elem(side);
        V3 tx = texel(c, pos[0], pos[1], pos[2]);
        R dt = t0 - t;
        total = vadd(total, vscale(tx, dt));
        t = t0;
        if (mx) { side.x = side.x + t_delta.x; pos[0] += step[0]; }
        if (my) { side.y = side.y + t_delta.y; pos[1] += step[1]; }
        if (mz) { side.z = side.z + t_delta.z; pos[2] += step[2]; }
    }
    return total;
}

/* ------------------------------------------------------------ octree --- */

#define NODE_WORDS 10
#define LEAF_MASK 0x80000000u
#define DEPTH_MASK 0x7FFFFFFFu

static inline int node_ok(Ctx* c, uint64_t i) {
    if (i >= c->vol->n_nodes) { c->err |= XO_ERR_INDEX; return 0; }
    return 1;
}
static inline uint32_t w_child(Ctx* c, uint64_t i, uint32_t k) {
    c->loads++;
    return c->vol->nodes[i * NODE_WORDS + k];
}
static inline uint32_t w_color(Ctx* c, uint64_t i) {
    c->loads++;
    return c->vol->nodes[i * NODE_WORDS + 8];
}
static inline uint32_t w_leafdepth(Ctx* c, uint64_t i) {
    c->loads++;
    return c->vol->nodes[i * NODE_WORDS + 9];
}
static inline V3 unpack_rgb(uint32_t col) {
    return v3(unorm8f(col & 0xFFu), unorm8f((col >> 8) & 0xFFu), unorm8f((col >> 16) & 0xFFu));
}

/* svo_naive.comp:8-27, identical to svo_rope.comp:8-27 */
static uint32_t find(Ctx* c, V3 pos, V3* base, R* side) {
    R extent = (R)1;
    uint32_t index = 0;
    V3 offset = vs((R)0);
    for (int level = 0;; ++level) {
        if (!node_ok(c, index)) return 0;
        if (w_leafdepth(c, index) >= LEAF_MASK) {
            *base = offset;
            *side = extent;
            return index;
        }
        if (level >= XO_FIND_MAX_DEPTH) { c->err |= XO_ERR_ITER; return 0; }
        extent *= (R)0.5f;
        V3 oe = vadd(offset, vs(extent));
        int mx = pos.x >= oe.x, my = pos.y >= oe.y, mz = pos.z >= oe.z;
        uint32_t child = (uint32_t)(mx * 4 + my * 2 + mz);
        offset = vadd(offset, vmul(v3((R)mx, (R)my, (R)mz), vs(extent)));
        index = w_child(c, index, child);
    }
}

/* svo_naive.comp:29-71 */
static V3 trace_naive(Ctx* c, V3 ro, V3 rd) {
    const R MIN_STEP = (R)0.00001f;
    V3 rrd = vdiv(vs((R)1), rd);
    V3 bias = vmul(rrd, ro);
    V3 box_min = v3(-bias.x, -bias.y, -bias.z);
    V3 box_max = vsub(rrd, bias);
    R t_min = max_elem(vmin(box_min, box_max));
    R t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs((R)0);
    t_min = rmax(t_min, (R)0);
    V3 total = vs((R)0);
    R t = t_min + MIN_STEP;
    uint32_t iter = 0;
    while (t < t_max) {
        if (++iter > XO_SVO_MAX_ITER) { c->err |= XO_ERR_ITER; break; }
        V3 p = vadd(vscale(rd, t), ro);
        V3 offset;
        R side;
        uint32_t node = find(c, p, &offset, &side);
        if (c->err) break;
        V3 node_min = vsub(vmul(offset, rrd), bias);
        V3 node_max = vsub(vmul(vadd(offset, vs(side)), rrd), bias);
        R u_min = max_elem(vmin(node_min, node_max));
        R u_max = min_elem(vmax(node_min, node_max));
        u_min = rmax(u_min, (R)0);
        R step = rmax(u_max - u_min, MIN_STEP);
        t += step;
        V3 color = unpack_rgb(w_color(c, node));
        total = vadd(total, vscale(color, step));
    }
    return total;
}

/* svo_df.comp:6-67 */
static V3 trace_df(Ctx* c, V3 ro, V3 rd) {
    V3 rrd = vdiv(vs((R)1), rd);
    V3 bias = vmul(rrd, ro);
    int sp = 0;
    uint32_t node_stack[XO_STACK_DEPTH];
    uint32_t child_index_stack[XO_STACK_DEPTH];
    uint32_t node = 0, child_idx = 0;
    V3 pos = vs((R)0);
    R side = (R)0.5f;
    V3 total = vs((R)0);
    uint32_t iter = 0;
    for (;;) {
        if (++iter > XO_SVO_MAX_ITER) { c->err |= XO_ERR_ITER; break; }
        if (!node_ok(c, node)) break;
        uint32_t child = w_child(c, node, child_idx);
        V3 box_min = vsub(vmul(pos, rrd), bias);
        V3 box_max = vsub(vmul(vadd(pos, vs(side)), rrd), bias);
        R t_min = max_elem(vmin(box_min, box_max));
        R t_max = min_elem(vmax(box_min, box_max));
        if (t_min < t_max && t_max > 0) {
            if (!node_ok(c, child)) break;
            if (w_leafdepth(c, child) >= LEAF_MASK) {
                V3 color = unpack_rgb(w_color(c, child));
                total = vadd(total, vscale(color, t_max - rmax(t_min, (R)0)));
            } else {
                if (child_idx != 7) {
                    if (sp >= XO_STACK_DEPTH) { c->err |= XO_ERR_STACK; break; }
                    node_stack[sp] = node;
                    child_index_stack[sp] = child_idx;
                    ++sp;
                }
                side *= (R)0.5f;
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
            int32_t d = (int32_t)(w_leafdepth(c, node) & DEPTH_MASK);
            side = (R)ldexp(1.0, -(d > 1000 ? 1000 : d)) * (R)0.5f;
        }
        V3 s2 = vs(side * (R)2.0f);
        pos = vsub(pos, v3(rmod(pos.x, s2.x), rmod(pos.y, s2.y), rmod(pos.z, s2.z)));
        ++child_idx;
        if (child_idx & 4) pos.x = pos.x + side;
        if (child_idx & 2) pos.y = pos.y + side;
        if (child_idx & 1) pos.z = pos.z + side;
    }
    return total;
}

/* esvo.comp:23-28 */
static inline uint32_t cxor(uint32_t x, int ax, int ay, int az) {
    x ^= ax ? 4u : 0u;
    x ^= ay ? 2u : 0u;
    x ^= az ? 1u : 0u;
    return x;
}
static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float ffrom(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* esvo.comp:30-136 */
static V3 trace_esvo(Ctx* c, V3 ro, V3 rd) {
    const uint32_t depth = XO_STACK_DEPTH;
    uint32_t node_stack[XO_STACK_DEPTH + 1];
    R t_max_stack[XO_STACK_DEPTH + 1];
    memset(node_stack, 0, sizeof(node_stack));
    memset(t_max_stack, 0, sizeof(t_max_stack));

    V3 t_coeff = v3((R)1 / -rabs(rd.x), (R)1 / -rabs(rd.y), (R)1 / -rabs(rd.z));
    V3 t_bias = vmul(t_coeff, ro);
    int gx = rd.x > 0, gy = rd.y > 0, gz = rd.z > 0;
    {
        V3 alt = vsub(vscale(t_coeff, (R)3.0f), t_bias);
        if (gx) t_bias.x = alt.x;
        if (gy) t_bias.y = alt.y;
        if (gz) t_bias.z = alt.z;
    }
    uint32_t octant_mask = cxor(0, gx, gy, gz);
    R t_min = max_elem(vsub(vscale(t_coeff, (R)2.0f), t_bias));
    R t_max = min_elem(vsub(t_coeff, t_bias));
    R h = t_max;
    t_min = rmax(t_min, (R)0);
    t_max = rmin(t_max, (R)sqrtf(3.0f));

    uint32_t parent = 0, idx = 0;
    V3 pos = vs((R)1);
    uint32_t scale = depth - 1;
    R scale_exp2 = (R)0.5f;
    {
        V3 tc = vsub(vscale(t_coeff, (R)1.5f), t_bias);
        int ax = tc.x > t_min, ay = tc.y > t_min, az = tc.z > t_min;
        if (ax) pos.x = (R)1.5f;
        if (ay) pos.y = (R)1.5f;
        if (az) pos.z = (R)1.5f;
        idx = cxor(idx, ax, ay, az);
    }
    V3 total = vs((R)0);
    uint32_t iter = 0;
    while (scale < depth) {
        if (++iter > XO_SVO_MAX_ITER) { c->err |= XO_ERR_ITER; break; }
        V3 t_corner = vsub(vmul(pos, t_coeff), t_bias);
        R tc_max = min_elem(t_corner);
        if (t_min <= t_max) {
            R tv_max = rmin(t_max, tc_max);
            if (t_min <= tv_max) {
                if (!node_ok(c, parent)) break;
                uint32_t child = w_child(c, parent, idx ^ octant_mask);
                if (!node_ok(c, child)) break;
                if (w_leafdepth(c, child) >= LEAF_MASK) {
                    V3 color = unpack_rgb(w_color(c, child));
                    total = vadd(total, vscale(color, tv_max - t_min));
                } else {
                    if (tc_max < h) {
                        node_stack[scale] = parent;
                        t_max_stack[scale] = t_max;
                    }
                    h = tc_max;
                    parent = child;
                    --scale;
                    scale_exp2 *= (R)0.5f;
                    V3 t_center = vadd(vscale(t_coeff, scale_exp2), t_corner);
                    int ax = t_center.x > t_min, ay = t_center.y > t_min, az = t_center.z > t_min;
                    idx = cxor(0, ax, ay, az);
                    if (ax) pos.x = pos.x + scale_exp2;
                    if (ay) pos.y = pos.y + scale_exp2;
                    if (az) pos.z = pos.z + scale_exp2;
                    t_max = tv_max;
                    continue;
                }
            }
        }
        /* ADVANCE */
        int ax = t_corner.x <= tc_max, ay = t_corner.y <= tc_max, az = t_corner.z <= tc_max;
        uint32_t step_mask = cxor(0, ax, ay, az);
        if (ax) pos.x = pos.x - scale_exp2;
        if (ay) pos.y = pos.y - scale_exp2;
        if (az) pos.z = pos.z - scale_exp2;
        t_min = tc_max;
        idx ^= step_mask;
        if ((idx & step_mask) != 0) {
            /* POP; positions are dyadic with at most 23 fraction bits, so the
             * float bit patterns are exact in both the FP32 and FP64 builds. */
            uint32_t xx = fbits((float)pos.x) ^ fbits((float)(pos.x + scale_exp2));
            uint32_t xy = fbits((float)pos.y) ^ fbits((float)(pos.y + scale_exp2));
            uint32_t xz = fbits((float)pos.z) ^ fbits((float)(pos.z + scale_exp2));
            uint32_t dbits = (ax ? xx : 0u) | (ay ? xy : 0u) | (az ? xz : 0u);
            scale = (fbits((float)dbits) >> 23) - 127u;
            if (scale >= depth) break; /* the loop condition ends the ray */
            scale_exp2 = (R)ffrom((scale - depth + 127u) << 23);
            parent = node_stack[scale];
            t_max = t_max_stack[scale];
            uint32_t shx = fbits((float)pos.x) >> scale;
            uint32_t shy = fbits((float)pos.y) >> scale;
            uint32_t shz = fbits((float)pos.z) >> scale;
            pos = v3((R)ffrom(shx << scale), (R)ffrom(shy << scale), (R)ffrom(shz << scale));
            idx = (shx & 1u) * 4u + (shy & 1u) * 2u + (shz & 1u);
            h = 0;
        }
    }
    return total;
}

/* svo_rope.comp:29-48 */
static uint32_t find_relative(Ctx* c, uint32_t parent, V3 offset, V3 pos, V3* base, R* side) {
    if (!node_ok(c, parent)) return 0;
    int32_t d = (int32_t)(w_leafdepth(c, parent) & DEPTH_MASK);
    R extent = (R)ldexp(1.0, -(d > 1000 ? 1000 : d));
    offset = v3(offset.x - rmod(offset.x, extent), offset.y - rmod(offset.y, extent),
                offset.z - rmod(offset.z, extent));
    for (int level = 0;; ++level) {
        if (!node_ok(c, parent)) return 0;
        if (w_leafdepth(c, parent) >= LEAF_MASK) {
            *base = offset;
            *side = extent;
            return parent;
        }
        if (level >= XO_FIND_MAX_DEPTH) { c->err |= XO_ERR_ITER; return 0; }
        extent *= (R)0.5f;
        V3 oe = vadd(offset, vs(extent));
        int mx = pos.x >= oe.x, my = pos.y >= oe.y, mz = pos.z >= oe.z;
        uint32_t child = (uint32_t)(mx * 4 + my * 2 + mz);
        offset = vadd(offset, vmul(v3((R)mx, (R)my, (R)mz), vs(extent)));
        parent = w_child(c, parent, child);
    }
}

/* svo_rope.comp:50-63 */
static inline uint32_t neighbor_index(const uint32_t nb[3], V3 far, V3* mask) {
    if (far.x < rmin(far.y, far.z)) { *mask = v3(1, 0, 0); return nb[0]; }
    if (far.y < far.z) { *mask = v3(0, 1, 0); return nb[1]; }
    *mask = v3(0, 0, 1);
    return nb[2];
}

/* svo_rope.comp:65-135 */
static V3 trace_rope(Ctx* c, V3 ro, V3 rd) {
    V3 sgn = v3(rsign(rd.x), rsign(rd.y), rsign(rd.z));
    uint32_t nb[3] = {1u - (uint32_t)rmax(sgn.x, (R)0), 3u - (uint32_t)rmax(sgn.y, (R)0),
                      5u - (uint32_t)rmax(sgn.z, (R)0)};
    sgn = vadd(sgn, vs((R)0.1f));
    V3 rrd = vdiv(vs((R)1), rd);
    V3 bias = vmul(rrd, ro);
    V3 box_min = v3(-bias.x, -bias.y, -bias.z);
    V3 box_max = vsub(rrd, bias);
    R t_min = max_elem(vmin(box_min, box_max));
    R t_max = min_elem(vmax(box_min, box_max));
    if (t_min > t_max) return vs((R)0);
    t_min = rmax(t_min, (R)0);
    V3 pos = vadd(ro, vscale(rd, t_min));
    V3 offset;
    R side;
    uint32_t node = find(c, pos, &offset, &side);
    if (c->err) return vs((R)0);
    V3 node_min = vsub(vmul(offset, rrd), bias);
    V3 node_max = vsub(vmul(vadd(offset, vs(side)), rrd), bias);
    V3 far = vmax(node_min, node_max);
    R u_min = max_elem(vmin(node_min, node_max));
    R u_max = min_elem(far);
    R step = u_max - rmax(u_min, (R)0);
    V3 color = unpack_rgb(w_color(c, node));
    V3 total = vscale(color, step);
    V3 mask;
    uint32_t n = neighbor_index(nb, far, &mask);
    node = w_child(c, node, n);
    offset = vadd(offset, vscale(vmul(mask, sgn), side));
    uint32_t iter = 0;
    while (node != 0) {
        if (++iter > XO_SVO_MAX_ITER) { c->err |= XO_ERR_ITER; break; }
        pos = vadd(ro, vscale(rd, u_max));
        node = find_relative(c, node, offset, pos, &offset, &side);
        if (c->err) break;
        node_min = vsub(vmul(offset, rrd), bias);
        node_max = vsub(vmul(vadd(offset, vs(side)), rrd), bias);
        far = vmax(node_min, node_max);
        u_min = max_elem(vmin(node_min, node_max));
        u_max = min_elem(far);
        step = u_max - rmax(u_min, (R)0);
        color = unpack_rgb(w_color(c, node));
        total = vadd(total, vscale(color, step));
        n = neighbor_index(nb, far, &mask);
        node = w_child(c, node, n);
        offset = vadd(offset, vscale(vmul(mask, sgn), side));
    }
    return total;
}

/* esvo.comp:10-21 */
static inline void aabb_intersect(V3 bmin, V3 bmax, V3 ro, V3 rd, R* t0, R* t1) {
    const R e = (R)0.00000001f;
    V3 rrd = vdiv(vs((R)1), vadd(rd, vs(e)));
    V3 tbot = vmul(vsub(bmin, ro), rrd);
    V3 ttop = vmul(vsub(bmax, ro), rrd);
    V3 tmin = vmin(ttop, tbot);
    V3 tmax = vmax(ttop, tbot);
    *t0 = rmax(rmax(tmin.x, tmin.y), rmax(tmin.x, tmin.z));
    *t1 = rmin(rmin(tmax.x, tmax.y), rmin(tmax.x, tmax.z));
}

static inline uint8_t store_unorm(R x) {
    R cl = rmin(rmax(x, (R)0), (R)1);
    if (!(cl == cl)) cl = 0; /* NaN stores 0 */
    return (uint8_t)rfloor(cl * (R)255.0f + (R)0.5f);
}

typedef struct {
    int traversal;
    const xo_volume* vol;
    const xo_view* view;
    RaySetup setup;
    V3 translation; /* pre-divided by the voxel ratio, src/render/Renderer.cpp:62 */
    uint8_t* out_rgba;
    XO_REAL* out_emission;
    uint32_t* out_loads;
    uint8_t* out_err;
    uint32_t tiles_x, tiles_y;
    uint32_t next_tile; /* atomic */
    int64_t errors;     /* atomic */
} Job;

static void render_pixel(Job* j, uint32_t ix, uint32_t iy) {
    const xo_view* v = j->view;
    int32_t px = v->output_offset[0] + (int32_t)ix;
    int32_t py = v->output_offset[1] + (int32_t)iy;
    V3 rd = ray_dir(&j->setup, v, px, py);
    Ctx c = {j->vol, 0, 0};
    V3 color;
    switch (j->traversal) {
    case XO_DDA: {
        /* dda.comp:65-70 */
        uint32_t m = j->vol->dim[0];
        if (j->vol->dim[1] > m) m = j->vol->dim[1];
        if (j->vol->dim[2] > m) m = j->vol->dim[2];
        R side = (R)m;
        V3 ro = vscale(j->translation, side);
        R ec = voxel_emission_coeff(&j->setup, rd) / side;
        color = vscale(trace_dda(&c, ro, rd), ec);
        break;
    }
    case XO_SVO_NAIVE:
        color = vscale(trace_naive(&c, j->translation, rd), voxel_emission_coeff(&j->setup, rd));
        break;
    case XO_SVO_DF:
        color = vscale(trace_df(&c, j->translation, rd), voxel_emission_coeff(&j->setup, rd));
        break;
    case XO_SVO_ROPE:
        color = vscale(trace_rope(&c, j->translation, rd), voxel_emission_coeff(&j->setup, rd));
        break;
    case XO_ESVO:
    default: {
        /* esvo.comp:148-154 */
        V3 ro = vadd(j->translation, vs((R)1));
        R t0, t1;
        aabb_intersect(vs((R)1), vs((R)2), ro, rd, &t0, &t1);
        ro = vadd(ro, vscale(rd, rmax(t0, (R)0)));
        color = vscale(trace_esvo(&c, ro, rd), voxel_emission_coeff(&j->setup, rd));
        break;
    }
    }
    uint64_t o = (uint64_t)iy * v->output_extent[0] + ix;
    if (j->out_rgba) {
        uint8_t* p = j->out_rgba + 4 * o;
        p[0] = store_unorm(color.x);
        p[1] = store_unorm(color.y);
        p[2] = store_unorm(color.z);
        p[3] = 255;
    }
    if (j->out_emission) {
        j->out_emission[3 * o + 0] = color.x;
        j->out_emission[3 * o + 1] = color.y;
        j->out_emission[3 * o + 2] = color.z;
    }
    if (j->out_loads) j->out_loads[o] = c.loads;
    if (j->out_err) j->out_err[o] = c.err;
    if (c.err) __atomic_add_fetch(&j->errors, 1, __ATOMIC_RELAXED);
}

static void* worker(void* arg) {
    Job* j = (Job*)arg;
    const xo_view* v = j->view;
    uint32_t n = j->tiles_x * j->tiles_y;
    for (;;) {
        uint32_t t = __atomic_fetch_add(&j->next_tile, 1, __ATOMIC_RELAXED);
        if (t >= n) break;
        /* 8x8 tiles, the shaders' local size (common.glsl:23) */
        uint32_t tx = t % j->tiles_x, ty = t / j->tiles_x;
        for (uint32_t y = ty * 8; y < ty * 8 + 8 && y < v->output_extent[1]; ++y)
            for (uint32_t x = tx * 8; x < tx * 8 + 8 && x < v->output_extent[0]; ++x)
                render_pixel(j, x, y);
    }
    return NULL;
}

int64_t XO_ENTRY(int traversal, const xo_volume* vol, const xo_camera* cam, const xo_view* view,
                 uint8_t* out_rgba, XO_REAL* out_emission, uint32_t* out_loads, uint8_t* out_err,
                 int nthreads) {
    if (!vol || !cam || !view || traversal < 0 || traversal > 4) return -1;
    if (view->display_extent[0] == 0 || view->display_extent[1] == 0) return -1;
    if (traversal == XO_DDA && (!vol->rgba || !vol->dim[0] || !vol->dim[1] || !vol->dim[2])) return -1;
    if (traversal != XO_DDA && (!vol->nodes || vol->n_nodes == 0)) return -1;
    Job j;
    memset(&j, 0, sizeof(j));
    j.traversal = traversal;
    j.vol = vol;
    j.view = view;
    j.setup.fwd = v3((R)cam->forward[0], (R)cam->forward[1], (R)cam->forward[2]);
    j.setup.up = v3((R)cam->up[0], (R)cam->up[1], (R)cam->up[2]);
    j.setup.ratio = v3((R)view->voxel_ratio[0], (R)view->voxel_ratio[1], (R)view->voxel_ratio[2]);
    j.setup.aspect = (R)view->display_extent[1] / (R)view->display_extent[0];
    j.setup.ec = (R)view->emission_coeff;
    j.translation = vdiv(v3((R)cam->translation[0], (R)cam->translation[1], (R)cam->translation[2]),
                         j.setup.ratio);
    j.out_rgba = out_rgba;
    j.out_emission = out_emission;
    j.out_loads = out_loads;
    j.out_err = out_err;
    j.tiles_x = (view->output_extent[0] + 7) / 8;
    j.tiles_y = (view->output_extent[1] + 7) / 8;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nthreads == 1) {
        worker(&j);
    } else {
        pthread_t th[256];
        int started = 0;
        for (int i = 0; i < nthreads; ++i)
            if (pthread_create(&th[started], NULL, worker, &j) == 0) ++started;
        if (started == 0) worker(&j);
        for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    }
    return j.errors;
}
