// glsl_shim.hpp - just enough GLSL, as C++, to compile the reference's
// compute shaders (shaders/taa.comp, shaders/sharpen.comp,
// shaders/antialias_fxaa_prepare.comp, shaders/antialias_fxaa.comp with
// shaders/Fxaa3_11_mod.h, shaders/post_process.comp) unmodified except for
// the mechanical rewrites oracle/ref_build.py applies.
//
// TEST INFRASTRUCTURE: it pins the oracle's restatement against the
// reference's own shader source; nothing in the product uses it.
//
// REAL is float (GLSL FP32; compile with -fsingle-precision-constant and
// -ffp-contract=off so literals and operations round as GLSL floats) or
// double (the FP64 reading of the same source).
//
// Sampler model (the same one the oracle documents): texelFetch and image
// loads clamp to the image; texture() is bilinear with clamp-to-edge and
// exact weights, except that a coordinate within GLSL_SNAP texels of a texel
// centre returns that texel (the hardware sampler's sub-texel rounding) and a
// NaN coordinate reads the edge texel.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#ifndef REAL
#define REAL float
#endif

namespace glsl {

using GReal = REAL;
typedef uint32_t uint;

template <class T> using if_arith = std::enable_if_t<std::is_arithmetic<T>::value, int>;
template <class T> using if_int = std::enable_if_t<std::is_integral<T>::value, int>;

struct ivec2;
struct uvec2;

// swizzle proxy over the storage of an N-vector: component indices I...
template <int N, class V, int... I> struct swz {
    GReal d[N];
    operator V() const { return V(d[I]...); }
    swz& operator=(const V& v) {
        const GReal src[] = {v[0], v[1], v[2], v[3]};
        int k = 0;
        ((d[I] = src[k++]), ...);
        return *this;
    }
    swz& operator+=(GReal s) {
        ((d[I] = d[I] + s), ...);
        return *this;
    }
};

struct vec2 {
    union {
        struct { GReal x, y; };
        struct { GReal r, g; };
        GReal d[2];
        swz<2, vec2, 0, 1> xy;
    };
    vec2() : x(0), y(0) {}
    template <class A, if_arith<A> = 0> explicit vec2(A a) : x(GReal(a)), y(GReal(a)) {}
    template <class A, class B, if_arith<A> = 0, if_arith<B> = 0> vec2(A a, B b) : x(GReal(a)), y(GReal(b)) {}
    vec2(const ivec2& v);
    vec2(const uvec2& v);
    GReal operator[](int i) const { return i < 2 ? d[i] : GReal(0); }
};

struct vec3 {
    union {
        struct { GReal x, y, z; };
        struct { GReal r, g, b; };
        GReal d[3];
        swz<3, vec2, 0, 1> xy;
        swz<3, vec2, 1, 2> gb;
    };
    vec3() : x(0), y(0), z(0) {}
    template <class A, if_arith<A> = 0> explicit vec3(A a) : x(GReal(a)), y(GReal(a)), z(GReal(a)) {}
    template <class A, class B, class C, if_arith<A> = 0, if_arith<B> = 0, if_arith<C> = 0>
    vec3(A a, B b, C c) : x(GReal(a)), y(GReal(b)), z(GReal(c)) {}
    template <class A, if_arith<A> = 0> vec3(const vec2& v, A s) : x(v.x), y(v.y), z(GReal(s)) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    GReal operator[](int i) const { return i < 3 ? d[i] : GReal(0); }
};

struct vec4 {
    union {
        struct { GReal x, y, z, w; };
        struct { GReal r, g, b, a; };
        GReal d[4];
        swz<4, vec2, 0, 1> xy;
        swz<4, vec2, 0, 1> rg;
        swz<4, vec3, 0, 1, 2> xyz;
        swz<4, vec3, 0, 1, 2> rgb;
        swz<4, vec2, 0, 2> rb;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    template <class A, if_arith<A> = 0> explicit vec4(A a) : x(GReal(a)), y(GReal(a)), z(GReal(a)), w(GReal(a)) {}
    template <class A, class B, class C, class D, if_arith<A> = 0, if_arith<B> = 0, if_arith<C> = 0, if_arith<D> = 0>
    vec4(A a_, B b_, C c_, D d_) : x(GReal(a_)), y(GReal(b_)), z(GReal(c_)), w(GReal(d_)) {}
    template <class A, if_arith<A> = 0> vec4(const vec3& v, A s) : x(v.x), y(v.y), z(v.z), w(GReal(s)) {}
    template <class A, class B, if_arith<A> = 0, if_arith<B> = 0>
    vec4(const vec2& v, A s, B t) : x(v.x), y(v.y), z(GReal(s)), w(GReal(t)) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    GReal operator[](int i) const { return d[i]; }
};

struct bvec2 { bool x, y; };
struct bvec3 { bool x, y, z; };

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    template <class A, if_int<A> = 0> explicit ivec2(A a) : x(int(a)), y(int(a)) {}
    template <class A, class B, if_arith<A> = 0, if_arith<B> = 0> ivec2(A a, B b) : x(int(a)), y(int(b)) {}
    explicit ivec2(const vec2& v) : x(int(v.x)), y(int(v.y)) {}
    explicit ivec2(const uvec2& v);
};
struct uvec2 {
    uint x, y;
};
struct uvec3 {
    uvec2 xy;  // the only access the shaders make (gl_GlobalInvocationID.xy)
    uint z;
};
struct uvec4 {
    union {
        struct { uint x, y, z, w; };
        struct { uint r, g, b, a; };
    };
    uvec4() : x(0), y(0), z(0), w(0) {}
    template <class A, class B, class C, class D> uvec4(A a_, B b_, C c_, D d_) : x(uint(a_)), y(uint(b_)), z(uint(c_)), w(uint(d_)) {}
};
// an integer 4-vector with the two swizzles the shaders read (.xy, .zw)
template <int A, int B> struct iswz {
    int d[4];
    operator ivec2() const { return ivec2(d[A], d[B]); }
};
struct ivec4 {
    union {
        struct { int x, y, z, w; };
        int d[4];
        iswz<0, 1> xy;
        iswz<2, 3> zw;
    };
    ivec4() : x(0), y(0), z(0), w(0) {}
    ivec4(int a_, int b_, int c_, int d_) : x(a_), y(b_), z(c_), w(d_) {}
};
inline ivec2::ivec2(const uvec2& v) : x(int(v.x)), y(int(v.y)) {}
inline vec2::vec2(const ivec2& v) : x(GReal(v.x)), y(GReal(v.y)) {}
inline vec2::vec2(const uvec2& v) : x(GReal(v.x)), y(GReal(v.y)) {}

struct mat4 {
    vec4 c[4];  // columns
};

// ---------------------------------------------------------------- arithmetic
#define GLSL_VEC_OPS(V, N)                                                                     \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.d[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b.d[i]; return r; } \
    inline V operator+(const V& a, GReal s) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + s; return r; }            \
    inline V operator-(const V& a, GReal s) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - s; return r; }            \
    inline V operator*(const V& a, GReal s) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s; return r; }            \
    inline V operator/(const V& a, GReal s) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / s; return r; }            \
    inline V operator+(GReal s, const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = s + a.d[i]; return r; }            \
    inline V operator-(GReal s, const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = s - a.d[i]; return r; }            \
    inline V operator*(GReal s, const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i]; return r; }            \
    inline V operator/(GReal s, const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = s / a.d[i]; return r; }            \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }                    \
    inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                                    \
    inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                                    \
    inline V& operator*=(V& a, GReal s) { a = a * s; return a; }                                                           \
    inline V& operator+=(V& a, GReal s) { a = a + s; return a; }                                                           \
    inline V min(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = b.d[i] < a.d[i] ? b.d[i] : a.d[i]; return r; } \
    inline V max(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] < b.d[i] ? b.d[i] : a.d[i]; return r; } \
    inline V clamp(const V& x, const V& lo, const V& hi) { return min(max(x, lo), hi); }                             \
    inline V abs(const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = std::fabs(a.d[i]); return r; }               \
    inline V sqrt(const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = std::sqrt(a.d[i]); return r; }              \
    inline V floor(const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = std::floor(a.d[i]); return r; }            \
    inline V fract(const V& a) { V r; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - std::floor(a.d[i]); return r; }   \
    inline GReal dot(const V& a, const V& b) { GReal s = a.d[0] * b.d[0]; for (int i = 1; i < N; ++i) s = s + a.d[i] * b.d[i]; return s; } \
    inline GReal length(const V& a) { return std::sqrt(dot(a, a)); }                                                       \
    inline V mix(const V& x, const V& y, GReal t) { V r; GReal u = GReal(1) - t; for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * u + y.d[i] * t; return r; }

GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)

// scalar helpers (GLSL semantics on finite values)
inline GReal min(GReal a, GReal b) { return b < a ? b : a; }
inline GReal max(GReal a, GReal b) { return a < b ? b : a; }
inline GReal clamp(GReal x, GReal lo, GReal hi) { return min(max(x, lo), hi); }
inline GReal mix(GReal x, GReal y, GReal t) { return x * (GReal(1) - t) + y * t; }
inline GReal abs(GReal a) { return std::fabs(a); }
inline GReal sqrt(GReal a) { return std::sqrt(a); }
inline GReal floor(GReal a) { return std::floor(a); }
inline GReal fract(GReal a) { return a - std::floor(a); }
inline GReal sin(GReal a) { return std::sin(a); }
inline GReal cos(GReal a) { return std::cos(a); }

// integer vectors
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.x - b.x, a.y - b.y); }
template <class I, if_int<I> = 0> ivec2 operator+(const ivec2& a, I s) { return ivec2(a.x + int(s), a.y + int(s)); }
template <class I, if_int<I> = 0> ivec2 operator-(const ivec2& a, I s) { return ivec2(a.x - int(s), a.y - int(s)); }
inline bool operator==(const ivec2& a, const ivec2& b) { return a.x == b.x && a.y == b.y; }
inline ivec2 min(const ivec2& a, const ivec2& b) { return ivec2(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y); }
inline ivec2 max(const ivec2& a, const ivec2& b) { return ivec2(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y); }
inline ivec2 clamp(const ivec2& x, const ivec2& lo, const ivec2& hi) { return min(max(x, lo), hi); }
// mixed integer / float vectors: the integer operand converts to float (GLSL 4.60 4.1.10)
inline vec2 operator+(const vec2& a, const ivec2& b) { return a + vec2(b); }
inline vec2 operator+(const ivec2& a, const vec2& b) { return vec2(a) + b; }
inline vec2 operator-(const vec2& a, const ivec2& b) { return a - vec2(b); }
inline vec2 operator-(const ivec2& a, const vec2& b) { return vec2(a) - b; }
inline vec2 operator*(const vec2& a, const ivec2& b) { return a * vec2(b); }
inline vec2 operator*(const ivec2& a, const vec2& b) { return vec2(a) * b; }
inline vec2 operator/(const vec2& a, const ivec2& b) { return a / vec2(b); }
inline vec2 operator/(const ivec2& a, const vec2& b) { return vec2(a) / b; }

// comparisons
inline bvec2 lessThan(const vec2& a, const vec2& b) { return {a.x < b.x, a.y < b.y}; }
inline bvec2 greaterThanEqual(const vec2& a, const vec2& b) { return {a.x >= b.x, a.y >= b.y}; }
inline bvec2 lessThan(const ivec2& a, const ivec2& b) { return {a.x < b.x, a.y < b.y}; }
inline bvec2 greaterThanEqual(const ivec2& a, const ivec2& b) { return {a.x >= b.x, a.y >= b.y}; }
inline bvec3 lessThan(const vec3& a, const vec3& b) { return {a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThan(const vec3& a, const vec3& b) { return {a.x > b.x, a.y > b.y, a.z > b.z}; }
inline bool any(bvec2 b) { return b.x || b.y; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }
inline bool all(bvec2 b) { return b.x && b.y; }

// column-major mat4 * vec4, rows accumulated left to right
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r.d[i] = m.c[0].d[i] * v.x + m.c[1].d[i] * v.y + m.c[2].d[i] * v.z + m.c[3].d[i] * v.w;
    return r;
}

// ---------------------------------------------------------------- resources
struct texture2D {
    const float* p = nullptr;  // RGBA or single-channel float texels
    int w = 0, h = 0, ch = 4;
};
struct sampler {};
struct sampler2D {
    const texture2D* t;
    sampler2D() : t(nullptr) {}  // a combined image sampler binding (bound by the driver code)
    explicit sampler2D(const texture2D* tex) : t(tex) {}
    sampler2D(const texture2D& tex, const sampler&) : t(&tex) {}
};
struct image2D {
    double* p = nullptr;  // RGBA outputs, written as the REAL values
    int w = 0, h = 0;
};
struct uimage2D {
    uint32_t* p = nullptr;
    int w = 0, h = 0;
};

#ifndef GLSL_SNAP
#define GLSL_SNAP 1e-4
#endif

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

inline vec4 texel(const texture2D& t, int x, int y) {
    if (!t.p) return vec4(0);
    x = clampi(x, 0, t.w - 1);
    y = clampi(y, 0, t.h - 1);
    const float* q = t.p + ((size_t)y * t.w + x) * t.ch;
    vec4 r(0);
    for (int c = 0; c < t.ch && c < 4; ++c) r.d[c] = GReal(q[c]);
    return r;
}
inline ivec2 textureSize(const texture2D& t, int) { return ivec2(t.w, t.h); }
inline vec4 texelFetch(const texture2D& t, const ivec2& c, int) { return texel(t, c.x, c.y); }

// bilinear, clamp to edge, exact weights; snaps to a centre within GLSL_SNAP texels
// (px, py): the footprint position in texel units (uv * size - 0.5)
inline vec4 texture_texels(const texture2D& t, double px, double py) {
    // a NaN coordinate reads the edge texel with weight 1 (taa.comp:535 divides
    // 0/0 at zero motion and then weights that tap by 0)
    if (px != px) px = -1e9;
    if (py != py) py = -1e9;
    double rx = std::floor(px + 0.5), ry = std::floor(py + 0.5);
    bool sx = std::fabs(px - rx) < GLSL_SNAP, sy = std::fabs(py - ry) < GLSL_SNAP;
    if (sx) px = rx;
    if (sy) py = ry;
    double fx0 = std::floor(px), fy0 = std::floor(py);
    GReal fx = GReal(px - fx0), fy = GReal(py - fy0);
    int x0 = int(std::fmax(std::fmin(fx0, 1e9), -1e9)), y0 = int(std::fmax(std::fmin(fy0, 1e9), -1e9));
    vec4 a = texel(t, x0, y0), b = texel(t, x0 + 1, y0), c = texel(t, x0, y0 + 1), d = texel(t, x0 + 1, y0 + 1);
    GReal gx = GReal(1) - fx, gy = GReal(1) - fy;
    vec4 top = a * gx + b * fx, bot = c * gx + d * fx;
    return top * gy + bot * fy;
}
inline vec4 texture(const sampler2D& s, const vec2& uv) {
    const texture2D& t = *s.t;
    return texture_texels(t, double(uv.x) * t.w - 0.5, double(uv.y) * t.h - 0.5);
}

// textureLod at level 0 of a single-level image is texture(); the offset
// variant moves the footprint by whole texels (GLSL 4.60 8.9.2).
inline vec4 textureLod(const sampler2D& s, const vec2& uv, GReal) { return texture(s, uv); }
inline vec4 textureLodOffset(const sampler2D& s, const vec2& uv, GReal, const ivec2& o) {
    const texture2D& t = *s.t;
    return texture_texels(t, double(uv.x) * t.w - 0.5 + o.x, double(uv.y) * t.h - 0.5 + o.y);
}
inline ivec2 textureSize(const sampler2D& s, int l) { return textureSize(*s.t, l); }
inline vec4 texelFetch(const sampler2D& s, const ivec2& c, int l) { return texelFetch(*s.t, c, l); }

inline void imageStore(image2D& im, const ivec2& c, const vec4& v) {
    if (!im.p || c.x < 0 || c.y < 0 || c.x >= im.w || c.y >= im.h) return;
    double* q = im.p + ((size_t)c.y * im.w + c.x) * 4;
    for (int i = 0; i < 4; ++i) q[i] = double(v.d[i]);
}
inline uvec4 imageLoad(const uimage2D& im, const ivec2& c) {
    if (!im.p) return uvec4(0, 0, 0, 0);
    return uvec4(im.p[(size_t)clampi(c.y, 0, im.h - 1) * im.w + clampi(c.x, 0, im.w - 1)], 0, 0, 0);
}
inline void imageStore(uimage2D& im, const ivec2& c, const uvec4& v) {
    if (!im.p || c.x < 0 || c.y < 0 || c.x >= im.w || c.y >= im.h) return;
    im.p[(size_t)c.y * im.w + c.x] = v.x;
}

}  // namespace glsl
