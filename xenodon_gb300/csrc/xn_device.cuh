// Device-side math with the GLSL semantics of the reference shaders.
//
// The translation unit that includes this header is compiled with
// --fmad=false and IEEE division / square root, so `a*b + c` is a rounded
// multiply followed by a rounded add, exactly as in the C oracle built with
// -ffp-contract=off.  Where a fused multiply-add is wanted it is written as
// fmaf() explicitly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace xn {

struct V3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vs(float s) { return V3{s, s, s}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 vmin(V3 a, V3 b) { return V3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
__device__ __forceinline__ V3 vmax(V3 a, V3 b) { return V3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
// resources/common.glsl:58-64
// Three-input minimum and maximum (PTX min.f32 / max.f32 with three
// sources): the value of fminf(a, fminf(b, c)), resp. fmaxf, for the finite,
// non-NaN operands every caller passes, in one operation instead of two.
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min_elem(V3 v) { return min3f(v.x, v.y, v.z); }
__device__ __forceinline__ float max_elem(V3 v) { return max3f(v.x, v.y, v.z); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// GLSL normalize: v / length(v), IEEE divide and square root.
__device__ __forceinline__ V3 normalize3(V3 v) {
    float l = __fsqrt_rn(dot3(v, v));
    return V3{__fdiv_rn(v.x, l), __fdiv_rn(v.y, l), __fdiv_rn(v.z, l)};
}
__device__ __forceinline__ float gl_sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
// GLSL mod: x - y*floor(x/y)
__device__ __forceinline__ float gl_mod(float x, float y) { return x - y * floorf(__fdiv_rn(x, y)); }
// GLSL mod(x, y) for y a power of two: x/y is then exactly x * (1/y) (both
// the reciprocal and the product are exact while 1/y is a normal float), so
// the IEEE division of gl_mod is replaced by a multiply; any other y falls
// back to the division.  `inv` is __frcp_rn(y), computed when y changes.
__device__ __forceinline__ float gl_mod_pow2(float x, float y, float inv, bool exact) {
    return x - y * floorf(exact ? x * inv : __fdiv_rn(x, y));
}
// x - mod(x, y), the reference's snap of x down to a multiple of y.  On the
// exact path (y a power of two with a normal reciprocal) the remainder
// r = x - y*floor(x/y) is exact -- a multiple of the smaller of y and x's ulp,
// below y in magnitude -- so x - r is y*floor(x/y) exactly, with the same
// sign of zero: three operations instead of five.
__device__ __forceinline__ float snap_down_pow2(float x, float y, float inv, bool exact) {
    return exact ? y * floorf(x * inv) : x - gl_mod_pow2(x, y, inv, false);
}
// Whether y is a power of two whose reciprocal is a normal float.
__device__ __forceinline__ bool pow2_with_normal_reciprocal(float y) {
    const uint32_t b = __float_as_uint(y);
    const uint32_t e = (b >> 23) & 0xFFu;
    return (b & 0x807FFFFFu) == 0 && e >= 2 && e <= 252;
}

// float -> int truncation, clamped like the oracle (out-of-range values are
// never used by the shaders).
__device__ __forceinline__ int f2i(float x) {
    x = fminf(fmaxf(x, -1073741824.f), 1073741824.f);
    return __float2int_rz(x);
}

// byte/255, correctly rounded (the UNORM8 -> float conversion of
// unpackUnorm4x8 and of R8G8B8A8_UNORM texel reads).  A reciprocal multiply
// followed by one Newton/Markstein correction step is exact for all 256
// inputs (checked exhaustively against IEEE division).
__device__ __forceinline__ float unorm8(uint32_t c) {
    const float r = 1.0f / 255.0f;
    float cf = __uint2float_rn(c);
    float q0 = cf * r;
    float rem = fmaf(-q0, 255.0f, cf);
    return fmaf(rem, r, q0);
}
__device__ __forceinline__ V3 unpack_rgb(uint32_t col) {
    return V3{unorm8(col & 0xFFu), unorm8((col >> 8) & 0xFFu), unorm8((col >> 16) & 0xFFu)};
}
// The same values with the byte's float made without a conversion
// instruction: 2^23 + c has c in its low mantissa bits, and subtracting 2^23
// is exact, so cf equals the converted byte.
__device__ __forceinline__ float unorm8_bits(uint32_t c) {
    const float r = 1.0f / 255.0f;
    const float cf = __uint_as_float(0x4B000000u | c) - 8388608.0f;
    const float q0 = cf * r;
    const float rem = fmaf(-q0, 255.0f, cf);
    return fmaf(rem, r, q0);
}
__device__ __forceinline__ V3 unpack_rgb_bits(uint32_t col) {
    return V3{unorm8_bits(col & 0xFFu), unorm8_bits((col >> 8) & 0xFFu), unorm8_bits((col >> 16) & 0xFFu)};
}

// resources/common.glsl:40-43
__device__ __forceinline__ V3 adjust_ray(V3 rd) {
    const float eps = 1.0f / 8388608.0f;  // exp2(-23)
    if (fabsf(rd.x) < eps) rd.x = eps;
    if (fabsf(rd.y) < eps) rd.y = eps;
    if (fabsf(rd.z) < eps) rd.z = eps;
    return rd;
}

// Per-frame constants (push constant + UBO of resources/common.glsl:25-33).
struct Frame {
    V3 forward, up;
    V3 translation;  // already divided by voxel_ratio (src/render/Renderer.cpp:62)
    V3 voxel_ratio;
    float aspect;    // float(display.extent.y) / float(display.extent.x)
    float emission_coeff;
    int32_t out_x, out_y;
    uint32_t out_w, out_h;
    int32_t disp_x, disp_y;
    uint32_t disp_w, disp_h;
};

// resources/common.glsl:45-56 with uv from resources/dda.comp:62-63
__device__ __forceinline__ V3 primary_ray(const Frame& f, uint32_t ix, uint32_t iy) {
    int32_t px = f.out_x + (int32_t)ix;
    int32_t py = f.out_y + (int32_t)iy;
    float u = __fdiv_rn((float)(px - f.disp_x), (float)f.disp_w);
    float w = __fdiv_rn((float)(py - f.disp_y), (float)f.disp_h);
    u -= 0.5f;
    w -= 0.5f;
    w *= f.aspect;
    V3 right = normalize3(cross3(f.up, f.forward));
    V3 up = normalize3(cross3(right, f.forward));
    V3 rd = normalize3((right * u + up * w) + f.forward);
    return adjust_ray(normalize3(rd / f.voxel_ratio));
}

// resources/common.glsl:68-72
__device__ __forceinline__ float voxel_emission_coeff(const Frame& f, V3 rd) {
    V3 rd2 = rd * rd;
    V3 dim2 = f.voxel_ratio * f.voxel_ratio;
    return f.emission_coeff * __fsqrt_rn(__fdiv_rn(dot3(rd2, dim2), dot3(rd2, vs(1.0f))));
}

// RGBA8 UNORM store of imageStore(vec4(color, 1)): clamp, round to nearest.
__device__ __forceinline__ uint32_t store_unorm(float x) {
    float c = fminf(fmaxf(x, 0.0f), 1.0f);  // NaN -> 0
    return (uint32_t)floorf(c * 255.0f + 0.5f);
}
__device__ __forceinline__ uint32_t pack_rgba(V3 c) {
    return store_unorm(c.x) | (store_unorm(c.y) << 8) | (store_unorm(c.z) << 16) | 0xFF000000u;
}

}  // namespace xn
