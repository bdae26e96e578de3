// A small C++ model of the GLSL compute-shader language: vector and matrix
// types, the built-in functions with the formulas the GLSL 4.60
// specification gives for them, images and samplers over host arrays, and
// the invocation ids.  Test infrastructure only: oracle/glsl/translate.py
// rewrites the reference's own compute shaders into C++ against this header
// so that they run on the host, and the tests compare the oracle with them.
//
// Conventions (all choices the GLSL specification leaves to the
// implementation, fixed here and used the same way by the oracle):
//  * float arithmetic is IEEE binary32 without contraction (built with
//    -ffp-contract=off) and floating literals are single precision
//    (-fsingle-precision-constant), as in GLSL;
//  * dot() sums left to right; mat * vec sums the columns left to right;
//    normalize(x) = x / length(x); length(x) = sqrt(dot(x, x));
//  * min / max / clamp return the non-NaN operand (IEEE minNum / maxNum,
//    what GPUs execute);
//  * transcendental functions are evaluated in binary64 and rounded once to
//    binary32 (the same bits on every host), except exp under GLSL_EXP_CW
//    (the sky and filter shaders), which is the oracle's Cody-Waite form;
//  * texture()/textureLod() filter bilinearly with clamp-to-edge addressing
//    and FP32 weights (x first, then y); texelFetch() reads the texel.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <atomic>
#include <initializer_list>
#include <thread>
#include <vector>
#include <type_traits>

namespace glsl {

using uint = uint32_t;

template <class T> struct tvec2;
template <class T> struct tvec3;
template <class T> struct tvec4;

template <class T> struct tvec2 {
    union {
        struct { T x, y; };
        struct { T r, g; };
    };
    tvec2() : x(T()), y(T()) {}
    tvec2(T s) : x(s), y(s) {}
    tvec2(T a, T b) : x(a), y(b) {}
    template <class U, class = std::enable_if_t<!std::is_same_v<U, T>>>
    tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
    tvec2 xy() const { return *this; }
    T& operator[](int i) { return i ? y : x; }
    T operator[](int i) const { return i ? y : x; }
};

template <class T> struct tvec3 {
    union {
        struct { T x, y, z; };
        struct { T r, g, b; };
    };
    tvec3() : x(T()), y(T()), z(T()) {}
    tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    tvec3(const tvec2<T>& v, T c) : x(v.x), y(v.y), z(c) {}
    explicit tvec3(const tvec4<T>& v);
    template <class U, class = std::enable_if_t<!std::is_same_v<U, T>>>
    tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    tvec2<T> xy() const { return {x, y}; }
    tvec3 xyz() const { return *this; }
    tvec3 rgb() const { return *this; }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T> struct tvec4 {
    union {
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
    };
    tvec4() : x(T()), y(T()), z(T()), w(T()) {}
    tvec4(T s) : x(s), y(s), z(s), w(s) {}
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    tvec4(const tvec2<T>& v, T c, T d) : x(v.x), y(v.y), z(c), w(d) {}
    template <class U, class = std::enable_if_t<!std::is_same_v<U, T>>>
    tvec4(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    tvec2<T> xy() const { return {x, y}; }
    tvec3<T> xyz() const { return {x, y, z}; }
    tvec3<T> rgb() const { return {x, y, z}; }
    void set_xyz(const tvec3<T>& v) { x = v.x; y = v.y; z = v.z; }
    void set_rgb(const tvec3<T>& v) { set_xyz(v); }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
template <class T> tvec3<T>::tvec3(const tvec4<T>& v) : x(v.x), y(v.y), z(v.z) {}

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using ivec2 = tvec2<int>;
using ivec3 = tvec3<int>;
using ivec4 = tvec4<int>;
using uvec2 = tvec2<uint>;
using uvec3 = tvec3<uint>;
using uvec4 = tvec4<uint>;
using bvec2 = tvec2<bool>;
using bvec3 = tvec3<bool>;
using bvec4 = tvec4<bool>;

// ---- component-wise operators (vector-vector, vector-scalar, scalar-vector)
template <class S> constexpr bool is_scalar_v = std::is_arithmetic_v<S>;

#define GLSL_BINOP(OP)                                                                                        \
    template <class T> tvec2<T> operator OP(const tvec2<T>& a, const tvec2<T>& b) {                          \
        return {T(a.x OP b.x), T(a.y OP b.y)};                                                                \
    }                                                                                                          \
    template <class T> tvec3<T> operator OP(const tvec3<T>& a, const tvec3<T>& b) {                          \
        return {T(a.x OP b.x), T(a.y OP b.y), T(a.z OP b.z)};                                                 \
    }                                                                                                          \
    template <class T> tvec4<T> operator OP(const tvec4<T>& a, const tvec4<T>& b) {                          \
        return {T(a.x OP b.x), T(a.y OP b.y), T(a.z OP b.z), T(a.w OP b.w)};                                  \
    }                                                                                                          \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec2<T> operator OP(const tvec2<T>& a, S s) { return a OP tvec2<T>(T(s)); }                               \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec3<T> operator OP(const tvec3<T>& a, S s) { return a OP tvec3<T>(T(s)); }                               \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec4<T> operator OP(const tvec4<T>& a, S s) { return a OP tvec4<T>(T(s)); }                               \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec2<T> operator OP(S s, const tvec2<T>& a) { return tvec2<T>(T(s)) OP a; }                               \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec3<T> operator OP(S s, const tvec3<T>& a) { return tvec3<T>(T(s)) OP a; }                               \
    template <class T, class S, class = std::enable_if_t<is_scalar_v<S>>>                                     \
    tvec4<T> operator OP(S s, const tvec4<T>& a) { return tvec4<T>(T(s)) OP a; }                               \
    template <class T, class B> tvec2<T>& operator OP##=(tvec2<T>& a, const B& b) { return a = a OP b; }      \
    template <class T, class B> tvec3<T>& operator OP##=(tvec3<T>& a, const B& b) { return a = a OP b; }      \
    template <class T, class B> tvec4<T>& operator OP##=(tvec4<T>& a, const B& b) { return a = a OP b; }

GLSL_BINOP(+)
GLSL_BINOP(-)
GLSL_BINOP(*)
GLSL_BINOP(/)
GLSL_BINOP(%)
#undef GLSL_BINOP

template <class T> tvec2<T> operator-(const tvec2<T>& a) { return {T(-a.x), T(-a.y)}; }
template <class T> tvec3<T> operator-(const tvec3<T>& a) { return {T(-a.x), T(-a.y), T(-a.z)}; }
template <class T> tvec4<T> operator-(const tvec4<T>& a) { return {T(-a.x), T(-a.y), T(-a.z), T(-a.w)}; }

inline float dot(const tvec3<float>& a, const tvec3<float>& b);

// ---- matrices (column-major; m[c] is column c)
struct mat3 {
    vec3 c[3];
    mat3() {}
    mat3(const vec3& a, const vec3& b, const vec3& d) : c{a, b, d} {}
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    mat4() {}
    mat4(const vec4& a, const vec4& b, const vec4& d, const vec4& e) : c{a, b, d, e} {}
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline vec4 operator*(const mat4& m, const vec4& v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w;
}
// row vector times matrix: component i is dot(v, column i)
inline vec3 operator*(const vec3& v, const mat3& m) { return {dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])}; }
inline mat4 operator*(const mat4& a, const mat4& b) { return {a * b.c[0], a * b.c[1], a * b.c[2], a * b.c[3]}; }
inline mat3 operator*(const mat3& a, const mat3& b) { return {a * b.c[0], a * b.c[1], a * b.c[2]}; }

// ---- built-in functions: scalar forms, then component-wise vector forms
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float floor(float x) { return std::floor(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float round(float x) { return std::round(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
// IEEE minNum / maxNum (a NaN operand yields the other one), as GPUs execute
// GLSL's min / max; the specification leaves NaN inputs undefined
inline float min(float x, float y) { return std::fmin(x, y); }
inline float max(float x, float y) { return std::fmax(x, y); }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline uint min(uint x, uint y) { return y < x ? y : x; }
inline uint max(uint x, uint y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float pow(float x, float y) { return float(std::pow(double(x), double(y))); }
#ifdef GLSL_EXP_CW
// e^x by Cody-Waite reduction x = n ln2 + r (ln2 split into a 16-bit head
// and a tail), the degree-7 Taylor polynomial of e^r in Horner form with
// fma, and an exact scale by 2^n: the exp the oracle and the CUDA kernels
// use for the sky, within GLSL's bound for exp (3 + 2|x| ulp).
inline float exp(float x) {
    if (!(x > -87.0f)) return std::isnan(x) ? x : 0.0f;
    if (x > 88.0f) return INFINITY;
    const float n = std::nearbyint(x * 1.44269502f);
    float r = std::fma(-n, 0.693145752f, x);
    r = std::fma(-n, 1.42860677e-6f, r);
    float q = 1.98412701e-4f;
    q = std::fma(q, r, 1.38888892e-3f);
    q = std::fma(q, r, 8.33333377e-3f);
    q = std::fma(q, r, 4.16666679e-2f);
    q = std::fma(q, r, 1.66666672e-1f);
    q = std::fma(q, r, 0.5f);
    q = std::fma(q, r, 1.0f);
    q = std::fma(q, r, 1.0f);
    const int e = int(n);
    if (e < -126) return 0.0f;
    return q * std::ldexp(1.0f, e);
}
#else
inline float exp(float x) { return float(std::exp(double(x))); }
#endif
inline float exp2(float x) { return float(std::exp2(double(x))); }
inline float log(float x) { return float(std::log(double(x))); }
inline float log2(float x) { return float(std::log2(double(x))); }
inline float sin(float x) { return float(std::sin(double(x))); }
inline float cos(float x) { return float(std::cos(double(x))); }
inline float tan(float x) { return float(std::tan(double(x))); }
inline float asin(float x) { return float(std::asin(double(x))); }
inline float acos(float x) { return float(std::acos(double(x))); }
inline float atan(float y, float x) { return float(std::atan2(double(y), double(x))); }
inline float atan(float x) { return float(std::atan(double(x))); }

#define GLSL_UNARY(F)                                                                                         \
    inline vec2 F(const vec2& v) { return {F(v.x), F(v.y)}; }                                                 \
    inline vec3 F(const vec3& v) { return {F(v.x), F(v.y), F(v.z)}; }                                         \
    inline vec4 F(const vec4& v) { return {F(v.x), F(v.y), F(v.z), F(v.w)}; }
GLSL_UNARY(abs)
GLSL_UNARY(sign)
GLSL_UNARY(floor)
GLSL_UNARY(ceil)
GLSL_UNARY(round)
GLSL_UNARY(fract)
GLSL_UNARY(sqrt)
GLSL_UNARY(inversesqrt)
GLSL_UNARY(exp)
GLSL_UNARY(exp2)
GLSL_UNARY(log)
GLSL_UNARY(log2)
GLSL_UNARY(sin)
GLSL_UNARY(cos)
GLSL_UNARY(acos)
#undef GLSL_UNARY

#define GLSL_BINARY(F)                                                                                        \
    inline vec2 F(const vec2& a, const vec2& b) { return {F(a.x, b.x), F(a.y, b.y)}; }                         \
    inline vec3 F(const vec3& a, const vec3& b) { return {F(a.x, b.x), F(a.y, b.y), F(a.z, b.z)}; }            \
    inline vec4 F(const vec4& a, const vec4& b) {                                                              \
        return {F(a.x, b.x), F(a.y, b.y), F(a.z, b.z), F(a.w, b.w)};                                           \
    }                                                                                                          \
    inline vec2 F(const vec2& a, float b) { return F(a, vec2(b)); }                                            \
    inline vec3 F(const vec3& a, float b) { return F(a, vec3(b)); }                                            \
    inline vec4 F(const vec4& a, float b) { return F(a, vec4(b)); }
GLSL_BINARY(min)
GLSL_BINARY(max)
GLSL_BINARY(pow)
GLSL_BINARY(mod)
#undef GLSL_BINARY
inline vec2 step(float e, const vec2& x) { return {step(e, x.x), step(e, x.y)}; }
inline vec3 step(float e, const vec3& x) { return {step(e, x.x), step(e, x.y), step(e, x.z)}; }
inline vec3 step(const vec3& e, const vec3& x) { return {step(e.x, x.x), step(e.y, x.y), step(e.z, x.z)}; }
inline vec3 smoothstep(float e0, float e1, const vec3& x) {
    return {smoothstep(e0, e1, x.x), smoothstep(e0, e1, x.y), smoothstep(e0, e1, x.z)};
}
inline vec2 clamp(const vec2& x, float lo, float hi) { return {clamp(x.x, lo, hi), clamp(x.y, lo, hi)}; }
inline vec3 clamp(const vec3& x, float lo, float hi) { return {clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi)}; }
inline vec3 clamp(const vec3& x, const vec3& lo, const vec3& hi) {
    return {clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z)};
}
inline vec4 clamp(const vec4& x, float lo, float hi) {
    return {clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi), clamp(x.w, lo, hi)};
}
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(const vec4& x, const vec4& y, float a) { return x * (1.0f - a) + y * a; }

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline float length(float x) { return std::fabs(x); }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec2 normalize(const vec2& v) { return v / length(v); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }

template <class T> bvec2 greaterThanEqual(const tvec2<T>& a, const tvec2<T>& b) { return {a.x >= b.x, a.y >= b.y}; }
template <class T> bvec2 greaterThan(const tvec2<T>& a, const tvec2<T>& b) { return {a.x > b.x, a.y > b.y}; }
template <class T> bvec2 lessThan(const tvec2<T>& a, const tvec2<T>& b) { return {a.x < b.x, a.y < b.y}; }
inline bool any(const bvec2& b) { return b.x || b.y; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }
inline bool all(const bvec2& b) { return b.x && b.y; }

// ---- constant arrays: an index past the end reads a zero element
template <class T, unsigned N> struct carray {
    T a[N];
    carray(std::initializer_list<T> l) {
        unsigned i = 0;
        for (const T& v : l) a[i++] = v;
    }
    const T& operator[](uint i) const {
        static const T zero{};
        return i < N ? a[i] : zero;
    }
};

// ---- images and samplers over host arrays (4 components per texel)
struct image2D {
    int w = 0, h = 0;
    float* px = nullptr;
};
struct uimage2D {
    int w = 0, h = 0;
    uint* px = nullptr;
};
struct sampler2D {
    int w = 0, h = 0;
    const float* px = nullptr;
};
struct usampler2D {
    int w = 0, h = 0;
    const uint* px = nullptr;
};
inline ivec2 imageSize(const image2D& i) { return {i.w, i.h}; }
inline ivec2 imageSize(const uimage2D& i) { return {i.w, i.h}; }
inline void imageStore(image2D& i, const ivec2& p, const vec4& v) {
    float* q = i.px + 4 * (size_t(p.y) * size_t(i.w) + size_t(p.x));
    q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = v.w;
}
inline void imageStore(uimage2D& i, const ivec2& p, const uvec4& v) {
    uint* q = i.px + 4 * (size_t(p.y) * size_t(i.w) + size_t(p.x));
    q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = v.w;
}
inline ivec2 textureSize(const sampler2D& s, int) { return {s.w, s.h}; }
inline ivec2 textureSize(const usampler2D& s, int) { return {s.w, s.h}; }
inline vec4 texelFetch(const sampler2D& s, const ivec2& p, int) {
    const float* q = s.px + 4 * (size_t(p.y) * size_t(s.w) + size_t(p.x));
    return {q[0], q[1], q[2], q[3]};
}
inline uvec4 texelFetch(const usampler2D& s, const ivec2& p, int) {
    const uint* q = s.px + 4 * (size_t(p.y) * size_t(s.w) + size_t(p.x));
    return {q[0], q[1], q[2], q[3]};
}
// bilinear with clamp-to-edge addressing and FP32 weights, interpolating
// along x, then y (a NaN coordinate reads texel 0)
inline vec4 textureLod(const sampler2D& s, const vec2& uv, float) {
    float u = uv.x * float(s.w) - 0.5f, v = uv.y * float(s.h) - 0.5f;
    if (std::isnan(u)) u = 0.0f;
    if (std::isnan(v)) v = 0.0f;
    u = std::fmin(std::fmax(u, -1.0f), float(s.w));
    v = std::fmin(std::fmax(v, -1.0f), float(s.h));
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    auto cl = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
    const int i0 = cl(int(fu), s.w), i1 = cl(int(fu) + 1, s.w), j0 = cl(int(fv), s.h), j1 = cl(int(fv) + 1, s.h);
    const vec4 t00 = texelFetch(s, {i0, j0}, 0), t10 = texelFetch(s, {i1, j0}, 0);
    const vec4 t01 = texelFetch(s, {i0, j1}, 0), t11 = texelFetch(s, {i1, j1}, 0);
    const vec4 top = t00 * (1.0f - a) + t10 * a, bot = t01 * (1.0f - a) + t11 * a;
    return top * (1.0f - b) + bot * b;
}
inline vec4 texture(const sampler2D& s, const vec2& uv) { return textureLod(s, uv, 0.0f); }

// ---- workgroup barrier: the dispatcher runs a workgroup's invocations as
// threads and points each at the workgroup's std::barrier
struct WorkgroupBarrier {
    virtual void wait() = 0;
};
inline thread_local WorkgroupBarrier* gl_workgroup_barrier = nullptr;
inline void barrier() {
    if (gl_workgroup_barrier) gl_workgroup_barrier->wait();
}

// ---- dispatch of a w x h grid of invocations: rows spread over `threads`
// host threads (the invocation ids are thread-local; a shader's globals are
// set before and only read during the dispatch)
template <class F> void dispatch_rows(int w, int y0, int y1, int threads, F&& f);
template <class F> void dispatch_2d(int w, int h, int threads, F&& f);
// the thread count the shims dispatch with (shared by every translation unit)
inline std::atomic<int>& ref_thread_count() {
    static std::atomic<int> n{1};
    return n;
}
inline int ref_threads() { return ref_thread_count().load(); }
inline int ref_dispatch_threads_set(int n) {
    if (n >= 1) ref_thread_count().store(n);
    return ref_threads();
}

// ---- invocation ids (set by the dispatcher before each invocation)
inline thread_local uvec3 gl_GlobalInvocationID;
inline thread_local uvec3 gl_LocalInvocationID;
inline thread_local uvec3 gl_WorkGroupID;
inline thread_local uint gl_LocalInvocationIndex;

template <class F> void dispatch_rows(int w, int y0, int y1, int threads, F&& f) {
    auto rows = [&](int r0, int r1) {
        for (int y = r0; y < r1; ++y)
            for (int x = 0; x < w; ++x) {
                gl_GlobalInvocationID = uvec3(uint(x), uint(y), 0u);
                f();
            }
    };
    if (threads <= 1 || y1 - y0 < 2) {
        rows(y0, y1);
        return;
    }
    std::vector<std::thread> pool;
    std::atomic<int> next{y0};
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (int y; (y = next.fetch_add(1)) < y1;) rows(y, y + 1);
        });
    for (auto& t : pool) t.join();
}
template <class F> void dispatch_2d(int w, int h, int threads, F&& f) { dispatch_rows(w, 0, h, threads, f); }

} // namespace glsl
