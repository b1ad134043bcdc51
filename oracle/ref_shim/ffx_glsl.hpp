// ffx_glsl.hpp - the GLSL that the FidelityFX headers need (shaders/ffx_a.h
// with A_GPU + A_GLSL, shaders/ffx_cas.h), as C++, so that the reference's
// shaders/sharpen_cas.comp compiles for the CPU unmodified except for the
// mechanical rewrites oracle/ref_build.py applies.
//
// TEST INFRASTRUCTURE: it pins the oracle's CAS restatement against the
// reference's own shader source; nothing in the product uses it.
//
// ffx_a.h defines a one-line helper for every scalar and vector type
// (float, uint, int; 1 to 4 components), and C++ type-checks all of them, so
// the vectors here are one template over element type and width with the
// component-wise operators, conversions and built-ins GLSL gives every
// vector.  Floats are GLSL FP32 (compile with -ffp-contract=off and
// -fsingle-precision-constant so that operations and literals round as
// GLSL's do).  Image loads clamp to the image (an out-of-range imageLoad is
// undefined in the reference); stores outside it are dropped.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace ffx_glsl {

typedef uint32_t uint;

template <class T, int N> struct gv;

// a swizzle: components I... of the storage of an N-vector of T, readable as a
// vector and assignable from one
template <class T, int N, int... I> struct sw {
    T d[N];
    operator gv<T, sizeof...(I)>() const { return gv<T, sizeof...(I)>(d[I]...); }
    sw& operator=(const gv<T, sizeof...(I)>& v) {
        int k = 0;
        ((d[I] = v.d[k++]), ...);
        return *this;
    }
};

template <class T> struct gv<T, 2> {
    union {
        struct { T x, y; };
        struct { T r, g; };
        T d[2];
    };
    gv() : x(0), y(0) {}
    explicit gv(T a) : x(a), y(a) {}
    template <class A, class B> gv(A a, B b) : x(T(a)), y(T(b)) {}
    template <class U> explicit gv(const gv<U, 2>& o) : x(T(o.x)), y(T(o.y)) {}
    gv(const gv& o) : x(o.x), y(o.y) {}
    gv& operator=(const gv& o) { x = o.x; y = o.y; return *this; }
    T& operator[](int i) { return d[i]; }
    T operator[](int i) const { return d[i]; }
};
template <class T> struct gv<T, 3> {
    union {
        struct { T x, y, z; };
        struct { T r, g, b; };
        T d[3];
        sw<T, 3, 0, 1> xy;
    };
    gv() : x(0), y(0), z(0) {}
    explicit gv(T a) : x(a), y(a), z(a) {}
    template <class A, class B, class C> gv(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <class A> gv(const gv<T, 2>& v, A s) : x(v.x), y(v.y), z(T(s)) {}
    template <class U> explicit gv(const gv<U, 3>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    gv(const gv& o) : x(o.x), y(o.y), z(o.z) {}
    gv& operator=(const gv& o) { x = o.x; y = o.y; z = o.z; return *this; }
    T& operator[](int i) { return d[i]; }
    T operator[](int i) const { return d[i]; }
};
template <class T> struct gv<T, 4> {
    union {
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
        T d[4];
        sw<T, 4, 0, 1> xy;
        sw<T, 4, 2, 3> zw;
        sw<T, 4, 0, 1, 2> xyz;
        sw<T, 4, 0, 1, 2> rgb;
    };
    gv() : x(0), y(0), z(0), w(0) {}
    explicit gv(T s) : x(s), y(s), z(s), w(s) {}
    template <class A, class B, class C, class D> gv(A a_, B b_, C c_, D d_) : x(T(a_)), y(T(b_)), z(T(c_)), w(T(d_)) {}
    template <class A> gv(const gv<T, 3>& v, A s) : x(v.x), y(v.y), z(v.z), w(T(s)) {}
    gv(const gv<T, 2>& p, const gv<T, 2>& q) : x(p.x), y(p.y), z(q.x), w(q.y) {}
    template <class U> explicit gv(const gv<U, 4>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    gv(const gv& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    gv& operator=(const gv& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    T& operator[](int i) { return d[i]; }
    T operator[](int i) const { return d[i]; }
};

using vec2 = gv<float, 2>;
using vec3 = gv<float, 3>;
using vec4 = gv<float, 4>;
using uvec2 = gv<uint, 2>;
using uvec3 = gv<uint, 3>;
using uvec4 = gv<uint, 4>;
using ivec2 = gv<int, 2>;
using ivec3 = gv<int, 3>;
using ivec4 = gv<int, 4>;
using bvec2 = gv<bool, 2>;
using bvec3 = gv<bool, 3>;
using bvec4 = gv<bool, 4>;

// component-wise f(a[i], b[i]) and f(a[i])
template <class T, int N, class F> gv<T, N> zip(const gv<T, N>& a, const gv<T, N>& b, F f) {
    gv<T, N> r;
    for (int i = 0; i < N; ++i) r.d[i] = f(a.d[i], b.d[i]);
    return r;
}
template <class T, int N, class F> gv<T, N> each(const gv<T, N>& a, F f) {
    gv<T, N> r;
    for (int i = 0; i < N; ++i) r.d[i] = f(a.d[i]);
    return r;
}

#define FFX_GLSL_BINOP(op)                                                                                    \
    template <class T, int N> gv<T, N> operator op(const gv<T, N>& a, const gv<T, N>& b) {                   \
        return zip(a, b, [](T p, T q) { return T(p op q); });                                                \
    }                                                                                                        \
    template <class T, int N, class S, std::enable_if_t<std::is_arithmetic<S>::value, int> = 0>              \
    gv<T, N> operator op(const gv<T, N>& a, S s) {                                                           \
        return each(a, [s](T p) { return T(p op T(s)); });                                                   \
    }                                                                                                        \
    template <class T, int N, class S, std::enable_if_t<std::is_arithmetic<S>::value, int> = 0>              \
    gv<T, N> operator op(S s, const gv<T, N>& a) {                                                           \
        return each(a, [s](T p) { return T(T(s) op p); });                                                   \
    }                                                                                                        \
    template <class T, int N> gv<T, N>& operator op##=(gv<T, N>& a, const gv<T, N>& b) { return a = a op b; } \
    template <class T, int N, class S, std::enable_if_t<std::is_arithmetic<S>::value, int> = 0>              \
    gv<T, N>& operator op##=(gv<T, N>& a, S s) {                                                             \
        return a = a op s;                                                                                   \
    }
FFX_GLSL_BINOP(+)
FFX_GLSL_BINOP(-)
FFX_GLSL_BINOP(*)
FFX_GLSL_BINOP(/)
FFX_GLSL_BINOP(&)
FFX_GLSL_BINOP(|)
FFX_GLSL_BINOP(^)
FFX_GLSL_BINOP(<<)
FFX_GLSL_BINOP(>>)
#undef FFX_GLSL_BINOP
template <class T, int N> gv<T, N> operator-(const gv<T, N>& a) { return each(a, [](T p) { return T(-p); }); }
template <class T, int N> gv<T, N> operator~(const gv<T, N>& a) { return each(a, [](T p) { return T(~p); }); }

// built-ins (GLSL 4.60 chapter 8) on scalars and vectors
template <class T, std::enable_if_t<std::is_arithmetic<T>::value, int> = 0> T min(T a, T b) { return b < a ? b : a; }
template <class T, std::enable_if_t<std::is_arithmetic<T>::value, int> = 0> T max(T a, T b) { return a < b ? b : a; }
template <class T, int N> gv<T, N> min(const gv<T, N>& a, const gv<T, N>& b) { return zip(a, b, [](T p, T q) { return min(p, q); }); }
template <class T, int N> gv<T, N> max(const gv<T, N>& a, const gv<T, N>& b) { return zip(a, b, [](T p, T q) { return max(p, q); }); }
template <class T> T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
inline float abs(float a) { return std::fabs(a); }
inline int abs(int a) { return a < 0 ? -a : a; }
template <class T, int N> gv<T, N> abs(const gv<T, N>& a) { return each(a, [](T p) { return abs(p); }); }
inline float floor(float a) { return std::floor(a); }
inline float fract(float a) { return a - std::floor(a); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float sin(float a) { return std::sin(a); }
inline float cos(float a) { return std::cos(a); }
inline float pow(float a, float b) { return std::pow(a, b); }
template <int N> gv<float, N> floor(const gv<float, N>& a) { return each(a, [](float p) { return floor(p); }); }
template <int N> gv<float, N> fract(const gv<float, N>& a) { return each(a, [](float p) { return fract(p); }); }
template <int N> gv<float, N> sqrt(const gv<float, N>& a) { return each(a, [](float p) { return sqrt(p); }); }
template <int N> gv<float, N> sin(const gv<float, N>& a) { return each(a, [](float p) { return sin(p); }); }
template <int N> gv<float, N> cos(const gv<float, N>& a) { return each(a, [](float p) { return cos(p); }); }
template <int N> gv<float, N> pow(const gv<float, N>& a, const gv<float, N>& b) {
    return zip(a, b, [](float p, float q) { return pow(p, q); });
}
// mix(x, y, a) = x * (1 - a) + y * a
inline float mix(float x, float y, float t) { return x * (1.0f - t) + y * t; }
template <int N> gv<float, N> mix(const gv<float, N>& x, const gv<float, N>& y, const gv<float, N>& t) {
    gv<float, N> r;
    for (int i = 0; i < N; ++i) r.d[i] = mix(x.d[i], y.d[i], t.d[i]);
    return r;
}
inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
template <int N> gv<uint, N> floatBitsToUint(const gv<float, N>& a) {
    gv<uint, N> r;
    for (int i = 0; i < N; ++i) r.d[i] = floatBitsToUint(a.d[i]);
    return r;
}
template <int N> gv<float, N> uintBitsToFloat(const gv<uint, N>& a) {
    gv<float, N> r;
    for (int i = 0; i < N; ++i) r.d[i] = uintBitsToFloat(a.d[i]);
    return r;
}
// binary16 bits of f, rounded to nearest even (finite inputs; CasSetup's GPU
// path packs its constants with it, which the CAS filter never calls)
inline uint half_bits(float f) {
    const uint u = floatBitsToUint(f), sign = (u >> 16) & 0x8000u;
    const float a = std::fabs(f);
    if (a >= 65520.0f) return sign | 0x7c00u;
    if (a < 6.103515625e-05f) return sign | (uint)std::nearbyint(a * 16777216.0f);  // subnormal: units of 2^-24
    int e;
    const float m = std::frexp(a, &e);               // a = m * 2^e, m in [0.5, 1)
    uint q = (uint)std::nearbyint(m * 2048.0f);      // 11 significant bits
    if (q == 2048u) { q = 1024u; ++e; }
    return sign | ((uint)(e + 14) << 10) | (q - 1024u);
}
inline uint packHalf2x16(const vec2& v) { return half_bits(v.x) | (half_bits(v.y) << 16); }

// bits [offset, offset + bits) of value, and value with them replaced by insert's low bits
inline uint bitfieldExtract(uint value, int offset, int bits) {
    return bits == 0 ? 0u : (value >> offset) & (bits == 32 ? 0xffffffffu : ((1u << bits) - 1u));
}
inline uint bitfieldInsert(uint base, uint insert, int offset, int bits) {
    const uint mask = (bits == 32 ? 0xffffffffu : ((1u << bits) - 1u)) << offset;
    return (base & ~mask) | ((insert << offset) & mask);
}

// ---------------------------------------------------------------- images
// an RGBA image of w x h float texels; imageLoad clamps the coordinate
struct image2D {
    const float* in = nullptr;
    double* out = nullptr;  // stores, as the FP32 values
    int w = 0, h = 0;
};
inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline vec4 imageLoad(const image2D& im, const ivec2& c) {
    const float* q = im.in + ((size_t)clampi(c.y, 0, im.h - 1) * im.w + clampi(c.x, 0, im.w - 1)) * 4;
    return vec4(q[0], q[1], q[2], q[3]);
}
inline void imageStore(image2D& im, const ivec2& c, const vec4& v) {
    if (c.x < 0 || c.y < 0 || c.x >= im.w || c.y >= im.h) return;
    double* q = im.out + ((size_t)c.y * im.w + c.x) * 4;
    for (int i = 0; i < 4; ++i) q[i] = double(v.d[i]);
}

}  // namespace ffx_glsl
