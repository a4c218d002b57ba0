// GLSL 4.50 compute-shader subset as C++17 -- TEST INFRASTRUCTURE ONLY.
//
// The types, swizzles and built-ins that the reference's traversal shaders
// (resources/*.comp with common.glsl and octree.glsl) use, so that those
// sources compile and run on the CPU, one invocation per pixel.  The recipe
// (oracle/glsl_ref.py) streams each shader into the compiler after this
// header, with four mechanical rewrites and nothing else changed: the
// `#version` line dropped, `#include "*.glsl"` replaced by the file, an `out T
// name` parameter written `T& name`, and a buffer block's unsized array
// `T name[];` written `XoBuffer<T> name;`.  The GLSL qualifiers and block names become
// the C++ declarations below.
//
// Arithmetic is IEEE single precision, every operation (division and sqrt
// included) correctly rounded and none contracted (the recipe passes
// -ffp-contract=off); GLSL allows less exact division and square roots, and
// a GPU driver may fuse a multiply and an add, so this is one admissible
// evaluation of the shaders, the one the restatement and the CUDA kernels
// follow.  The built-ins follow their definitions in the GLSL 4.50
// specification: min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x,
// mod(x, y) = x - y * floor(x / y), length(x) = sqrt(dot(x, x)),
// normalize(x) = x / length(x), dot summed from the first component, cross as
// defined there, sign(x) in {-1, 0, 1}.  unpackUnorm4x8 and texelFetch of an
// RGBA8 texture give byte / 255, correctly rounded; texelFetch outside the
// texture gives 0 (robust image access).  imageStore to the rgba8 target keeps
// the float colour it is given and its RGBA8 form, round(clamp(c, 0, 1) *
// 255) with halves rounded up.
#pragma once

#include <cstdint>
#include <cstring>
#include <type_traits>

typedef uint32_t uint;

template <class T> constexpr bool xo_num = std::is_arithmetic_v<T> && !std::is_same_v<T, bool>;

// GLSL's implicit conversions: int -> uint, int -> float, uint -> float.
template <class From, class To>
constexpr bool xo_implicit = std::is_same_v<From, To> ||
                             (std::is_same_v<To, float> && (std::is_same_v<From, int> || std::is_same_v<From, uint>)) ||
                             (std::is_same_v<To, uint> && std::is_same_v<From, int>);

template <class T, int N> struct V;

// A read-only swizzle: the vector's components I... as a vector of their own.
template <class T, int N, int... I> struct Swz {
    T e[N];
    template <class U, std::enable_if_t<xo_implicit<T, U>, int> = 0>
    operator V<U, (int)sizeof...(I)>() const {
        return V<U, (int)sizeof...(I)>(U(e[I])...);
    }
};

#define XO_VEC_COMMON(N)                                                                                   \
    static constexpr int n = N;                                                                           \
    typedef T scalar;                                                                                     \
    V() : e{} {}                                                                                          \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    explicit V(S s) {                                                                                     \
        for (int i = 0; i < N; ++i) e[i] = T(s);                                                          \
    }                                                                                                     \
    template <class U, std::enable_if_t<!std::is_same_v<U, T> && xo_implicit<U, T>, int> = 0>             \
    V(const V<U, N>& o) {                                                                                 \
        for (int i = 0; i < N; ++i) e[i] = T(o.e[i]);                                                     \
    }                                                                                                     \
    template <class U, std::enable_if_t<!std::is_same_v<U, T> && !xo_implicit<U, T>, int> = 0>            \
    explicit V(const V<U, N>& o) {                                                                        \
        for (int i = 0; i < N; ++i) e[i] = T(o.e[i]);                                                     \
    }                                                                                                     \
    V& operator+=(const V& o) { for (int i = 0; i < N; ++i) e[i] += o.e[i]; return *this; }               \
    V& operator-=(const V& o) { for (int i = 0; i < N; ++i) e[i] -= o.e[i]; return *this; }               \
    V& operator*=(const V& o) { for (int i = 0; i < N; ++i) e[i] *= o.e[i]; return *this; }               \
    V& operator/=(const V& o) { for (int i = 0; i < N; ++i) e[i] /= o.e[i]; return *this; }               \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    V& operator+=(S s) { for (int i = 0; i < N; ++i) e[i] += T(s); return *this; }                        \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    V& operator-=(S s) { for (int i = 0; i < N; ++i) e[i] -= T(s); return *this; }                        \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    V& operator*=(S s) { for (int i = 0; i < N; ++i) e[i] *= T(s); return *this; }                        \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    V& operator/=(S s) { for (int i = 0; i < N; ++i) e[i] /= T(s); return *this; }                        \
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                                \
    V& operator%=(S s) { for (int i = 0; i < N; ++i) e[i] %= T(s); return *this; }

template <class T> struct V<T, 2> {
    union {
        T e[2];
        struct { T x, y; };
    };
    XO_VEC_COMMON(2)
    template <class A, class B, std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B>, int> = 0>
    V(A a, B b) : e{T(a), T(b)} {}
};

template <class T> struct V<T, 3> {
    union {
        T e[3];
        struct { T x, y, z; };
        struct { T r, g, b; };
        Swz<T, 3, 0, 1, 2> xyz;
        Swz<T, 3, 1, 2, 0> yzx;
        Swz<T, 3, 2, 0, 1> zxy;
        Swz<T, 3, 0, 0> xx;
        Swz<T, 3, 1, 2> yz;
        Swz<T, 3, 0, 1> xy;
    };
    XO_VEC_COMMON(3)
    template <class A, class B, class C,
              std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B> && std::is_arithmetic_v<C>, int> = 0>
    V(A a, B b, C c) : e{T(a), T(b), T(c)} {}
};

template <class T> struct V<T, 4> {
    union {
        T e[4];
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
        Swz<T, 4, 0, 1, 2> xyz;
        Swz<T, 4, 0, 1, 2> rgb;
    };
    XO_VEC_COMMON(4)
    template <class A, class B, class C, class D>
    V(A a, B b, C c, D d) : e{T(a), T(b), T(c), T(d)} {}
    template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
    V(const V<T, 3>& v, S s) : e{v.e[0], v.e[1], v.e[2], T(s)} {}
};

typedef V<float, 2> vec2;
typedef V<float, 3> vec3;
typedef V<float, 4> vec4;
typedef V<int, 2> ivec2;
typedef V<int, 3> ivec3;
typedef V<int, 4> ivec4;
typedef V<uint, 2> uvec2;
typedef V<uint, 3> uvec3;
typedef V<uint, 4> uvec4;
typedef V<bool, 2> bvec2;
typedef V<bool, 3> bvec3;

// ------------------------------------------------------------ operators ---

#define XO_BIN(VT, ST, op)                                                                         \
    inline VT operator op(const VT& p, const VT& q) {                                              \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = p.e[i] op q.e[i];                                 \
        return r;                                                                                  \
    }                                                                                              \
    inline VT operator op(const VT& p, ST s) {                                                     \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = p.e[i] op s;                                      \
        return r;                                                                                  \
    }                                                                                              \
    inline VT operator op(ST s, const VT& q) {                                                     \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = s op q.e[i];                                      \
        return r;                                                                                  \
    }

#define XO_ARITH(VT, ST) XO_BIN(VT, ST, +) XO_BIN(VT, ST, -) XO_BIN(VT, ST, *) XO_BIN(VT, ST, /)
#define XO_INTOPS(VT, ST) XO_BIN(VT, ST, %) XO_BIN(VT, ST, &) XO_BIN(VT, ST, |) XO_BIN(VT, ST, ^)

XO_ARITH(vec2, float)
XO_ARITH(vec3, float)
XO_ARITH(vec4, float)
XO_ARITH(ivec2, int)
XO_ARITH(ivec3, int)
XO_ARITH(uvec2, uint)
XO_ARITH(uvec3, uint)
XO_INTOPS(ivec3, int)
XO_INTOPS(uvec3, uint)

inline uvec3 operator<<(const uvec3& p, uint s) { return uvec3(p.x << s, p.y << s, p.z << s); }
inline uvec3 operator>>(const uvec3& p, uint s) { return uvec3(p.x >> s, p.y >> s, p.z >> s); }

template <class T, int N> inline V<T, N> operator-(const V<T, N>& p) {
    V<T, N> r;
    for (int i = 0; i < N; ++i) r.e[i] = -p.e[i];
    return r;
}

// ----------------------------------------------------------- relations ---

#define XO_REL(VT, BT, name, op)                                                                   \
    inline BT name(const VT& p, const VT& q) {                                                     \
        BT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = p.e[i] op q.e[i];                                 \
        return r;                                                                                  \
    }
#define XO_RELS(VT, BT)                                                                            \
    XO_REL(VT, BT, lessThan, <) XO_REL(VT, BT, lessThanEqual, <=) XO_REL(VT, BT, greaterThan, >)   \
    XO_REL(VT, BT, greaterThanEqual, >=) XO_REL(VT, BT, equal, ==) XO_REL(VT, BT, notEqual, !=)

XO_RELS(vec3, bvec3)
XO_RELS(uvec2, bvec2)
XO_RELS(uvec3, bvec3)
XO_RELS(ivec3, bvec3)

template <int N> inline bool any(const V<bool, N>& p) {
    for (int i = 0; i < N; ++i)
        if (p.e[i]) return true;
    return false;
}
template <int N> inline bool all(const V<bool, N>& p) {
    for (int i = 0; i < N; ++i)
        if (!p.e[i]) return false;
    return true;
}

// ------------------------------------------------------------ built-ins ---

template <class A, class B>
using xo_common = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<B>, float,
                                     std::conditional_t<std::is_unsigned_v<A> || std::is_unsigned_v<B>, uint, int>>;

inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline uint min(uint x, uint y) { return y < x ? y : x; }
inline uint max(uint x, uint y) { return x < y ? y : x; }
// a scalar and a literal of another type, as GLSL's implicit conversions
// (a float literal is single precision in GLSL)
template <class A, class B, std::enable_if_t<xo_num<A> && xo_num<B> && !std::is_same_v<A, B>, int> = 0>
inline xo_common<A, B> min(A x, B y) {
    return min(xo_common<A, B>(x), xo_common<A, B>(y));
}
template <class A, class B, std::enable_if_t<xo_num<A> && xo_num<B> && !std::is_same_v<A, B>, int> = 0>
inline xo_common<A, B> max(A x, B y) {
    return max(xo_common<A, B>(x), xo_common<A, B>(y));
}

#define XO_VMINMAX(VT)                                                                             \
    inline VT min(const VT& p, const VT& q) {                                                      \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = min(p.e[i], q.e[i]);                              \
        return r;                                                                                  \
    }                                                                                              \
    inline VT max(const VT& p, const VT& q) {                                                      \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = max(p.e[i], q.e[i]);                              \
        return r;                                                                                  \
    }
XO_VMINMAX(vec2)
XO_VMINMAX(vec3)
XO_VMINMAX(ivec3)

inline float mix(float x, float y, bool a) { return a ? y : x; }
inline int mix(int x, int y, bool a) { return a ? y : x; }
inline uint mix(uint x, uint y, bool a) { return a ? y : x; }
#define XO_VMIX(VT, BT)                                                                            \
    inline VT mix(const VT& p, const VT& q, const BT& a) {                                         \
        VT r;                                                                                      \
        for (int i = 0; i < VT::n; ++i) r.e[i] = a.e[i] ? q.e[i] : p.e[i];                         \
        return r;                                                                                  \
    }
XO_VMIX(vec3, bvec3)
XO_VMIX(ivec3, bvec3)
XO_VMIX(uvec3, bvec3)

inline float abs(float x) { return __builtin_fabsf(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float exp2(float x) { return __builtin_exp2f(x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : x < 0.0f ? -1.0f : 0.0f; }
inline float mod(float x, float y) { return x - y * floor(x / y); }

#define XO_VFUN(name)                                                                              \
    inline vec3 name(const vec3& p) { return vec3(name(p.x), name(p.y), name(p.z)); }
XO_VFUN(abs)
XO_VFUN(floor)
XO_VFUN(sign)
inline vec3 mod(const vec3& p, float y) { return vec3(mod(p.x, y), mod(p.y, y), mod(p.z, y)); }

inline float dot(const vec3& p, const vec3& q) { return p.x * q.x + p.y * q.y + p.z * q.z; }
inline float length(const vec3& p) { return sqrt(dot(p, p)); }
inline vec3 normalize(const vec3& p) { return p / length(p); }
inline vec3 cross(const vec3& p, const vec3& q) {
    return vec3(p.y * q.z - q.y * p.z, p.z * q.x - q.z * p.x, p.x * q.y - q.x * p.y);
}

inline uint floatBitsToUint(float x) {
    uint u;
    std::memcpy(&u, &x, 4);
    return u;
}
inline float uintBitsToFloat(uint u) {
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}
inline uvec3 floatBitsToUint(const vec3& p) {
    return uvec3(floatBitsToUint(p.x), floatBitsToUint(p.y), floatBitsToUint(p.z));
}
inline vec3 uintBitsToFloat(const uvec3& p) {
    return vec3(uintBitsToFloat(p.x), uintBitsToFloat(p.y), uintBitsToFloat(p.z));
}

inline vec4 unpackUnorm4x8(uint c) {
    return vec4(float(c & 0xFFu) / 255.0f, float((c >> 8) & 0xFFu) / 255.0f, float((c >> 16) & 0xFFu) / 255.0f,
                float(c >> 24) / 255.0f);
}

// --------------------------------------------------- resources of a pass ---

// Words the current invocation has read from the model: texels fetched and
// node buffer accesses.  In these shaders every `model.nodes[i]` expression
// is followed by one field (`children[k]`, `color` or `is_leaf_depth`), so
// each access of the buffer reads one 32-bit word.
static uint64_t xo_words_read;

// The node buffer's unsized array, written `XoBuffer<T> name;` by the recipe.
template <class T> struct XoBuffer {
    const T* p = nullptr;
    const T& operator[](uint64_t i) const {
        ++xo_words_read;
        return p[i];
    }
};

// An RGBA8 3D texture, x fastest, read with texelFetch.
struct sampler3D {
    const uint8_t* rgba = nullptr;
    int dx = 0, dy = 0, dz = 0;
};
inline vec4 texelFetch(const sampler3D& s, const ivec3& p, int) {
    ++xo_words_read;
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= s.dx || p.y >= s.dy || p.z >= s.dz) return vec4(0);
    const uint8_t* t = s.rgba + 4 * ((size_t)p.x + (size_t)s.dx * ((size_t)p.y + (size_t)s.dy * (size_t)p.z));
    return vec4(float(t[0]) / 255.0f, float(t[1]) / 255.0f, float(t[2]) / 255.0f, float(t[3]) / 255.0f);
}
inline ivec3 textureSize(const sampler3D& s, int) { return ivec3(s.dx, s.dy, s.dz); }

// The rgba8 storage image: the float colour and its RGBA8 form per pixel.
struct image2D {
    float* colour = nullptr;  // 4 floats per pixel, or null
    uint8_t* rgba = nullptr;  // 4 bytes per pixel, or null
    int width = 0;
};
inline uint8_t xo_unorm8(float c) {
    c = c > 0.0f ? (c < 1.0f ? c : 1.0f) : 0.0f;  // NaN -> 0
    return (uint8_t)__builtin_floorf(c * 255.0f + 0.5f);
}
inline void imageStore(image2D& im, const ivec2& p, const vec4& c) {
    const size_t i = (size_t)p.y * (size_t)im.width + (size_t)p.x;
    if (im.colour)
        for (int k = 0; k < 4; ++k) im.colour[4 * i + k] = c.e[k];
    if (im.rgba)
        for (int k = 0; k < 4; ++k) im.rgba[4 * i + k] = xo_unorm8(c.e[k]);
}

// The invocation's id, set by the entry point for every pixel.
static uvec3 gl_GlobalInvocationID;

// ------------------------------------------------ qualifiers and blocks ---

#define layout(...)
#define in
#define uniform
#define readonly
#define writeonly
#define restrict
#define buffer
#define PushConstant struct PushConstant_t
#define UniformBuffer struct UniformBuffer_t
#define Octree struct Octree_t
// the pass's model binding (a texture or the node buffer), set by the entry
#define model (*xo_model)
#define main xo_shader_main
