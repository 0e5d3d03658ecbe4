// glsl_shim.hpp -- TEST INFRASTRUCTURE ONLY (pins the CPU oracle).
//
// The subset of GLSL 4.60 that the reference's path-tracing shaders and
// their include files use -- scalar and vector types with the .xy / .xyz /
// .rgb swizzles, mat3 / mat4 / mat4x3, the arithmetic operators and the
// built-in functions they call, storage images and a combined image sampler
// -- so that those files compile unchanged as C++ inside a namespace. The
// built-ins GLSL leaves implementation-defined take the oracle's definitions
// (oracle_math.hpp), which are also the device's: sin, cos, asin, acos,
// atan, normalize = v * (1 / length(v)), mix(x, y, a) = x * (1 - a) + y * a,
// pow(x, 5) = ((x * x) * (x * x)) * x, radians(x) = x * 0.017453292,
// min / max at equal operands, inverse(mat3) by cofactors in double, and
// texture() as bilinear REPEAT filtering with texel centres at (i + 0.5) / n.
// GLSL's float literals are single precision: the translation unit that
// includes this header is compiled with -fsingle-precision-constant,
// -ffp-contract=off and -fno-strict-aliasing (the swizzles share storage
// with the components through unions).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "oracle_math.hpp"

namespace glsl {

using uint = std::uint32_t;

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct uvec2;
struct uvec3;
struct uvec4;
template <class T, int N> struct VecOf;
template <> struct VecOf<float, 2> { using type = vec2; };
template <> struct VecOf<float, 3> { using type = vec3; };
template <> struct VecOf<float, 4> { using type = vec4; };
template <> struct VecOf<int, 2> { using type = ivec2; };
template <> struct VecOf<uint, 2> { using type = uvec2; };
template <> struct VecOf<uint, 3> { using type = uvec3; };
template <> struct VecOf<uint, 4> { using type = uvec4; };

// A swizzle: components I... of the N-component storage it overlays.
template <class T, int N, int... I>
struct Swz {
    T d[N];
    using V = typename VecOf<T, int(sizeof...(I))>::type;
    operator V() const { return V(d[I]...); }
    Swz& operator=(const V& v) {
        int k = 0;
        ((d[I] = v[k++]), ...);
        return *this;
    }
    Swz& operator=(const Swz& o) { return *this = V(o); }
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        float v_[2];
    };
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(float a) : x(a), y(a) {}
    explicit vec2(const ivec2& o);
    explicit vec2(const uvec2& o);
    float& operator[](int i) { return v_[i]; }
    float operator[](int i) const { return v_[i]; }
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        Swz<float, 3, 0, 1> xy;
        Swz<float, 3, 0, 1, 2> xyz, rgb;
        float v_[3];
    };
    vec3() = default;
    vec3(const vec3& o) { std::memcpy(v_, o.v_, sizeof v_); }
    vec3& operator=(const vec3& o) { std::memcpy(v_, o.v_, sizeof v_); return *this; }
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(float a) : x(a), y(a), z(a) {}
    vec3(const vec2& a, float c) : x(a.x), y(a.y), z(c) {}
    explicit vec3(const vec4& o);
    float& operator[](int i) { return v_[i]; }
    float operator[](int i) const { return v_[i]; }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        Swz<float, 4, 0, 1> xy;
        Swz<float, 4, 0, 1, 2> xyz, rgb;
        float v_[4];
    };
    vec4() = default;
    vec4(const vec4& o) { std::memcpy(v_, o.v_, sizeof v_); }
    vec4& operator=(const vec4& o) { std::memcpy(v_, o.v_, sizeof v_); return *this; }
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    explicit vec4(float a) : x(a), y(a), z(a), w(a) {}
    vec4(const vec3& o, float d) : x(o.x), y(o.y), z(o.z), w(d) {}
    vec4(const vec2& o, float c, float d) : x(o.x), y(o.y), z(c), w(d) {}
    float& operator[](int i) { return v_[i]; }
    float operator[](int i) const { return v_[i]; }
};
inline vec3::vec3(const vec4& o) : x(o.x), y(o.y), z(o.z) {}

struct ivec2 {
    int x, y;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(int a) : x(a), y(a) {}
    explicit ivec2(const vec2& o) : x(int(o.x)), y(int(o.y)) {}
    explicit ivec2(const uvec2& o);
    int& operator[](int i) { return i ? y : x; }
    int operator[](int i) const { return i ? y : x; }
};
struct uvec2 {
    uint x, y;
    uvec2() = default;
    uvec2(uint a, uint b) : x(a), y(b) {}
    explicit uvec2(const ivec2& o) : x(uint(o.x)), y(uint(o.y)) {}
    uint& operator[](int i) { return i ? y : x; }
    uint operator[](int i) const { return i ? y : x; }
};
inline vec2::vec2(const ivec2& o) : x(float(o.x)), y(float(o.y)) {}
inline vec2::vec2(const uvec2& o) : x(float(o.x)), y(float(o.y)) {}
inline ivec2::ivec2(const uvec2& o) : x(int(o.x)), y(int(o.y)) {}

struct uvec3 {
    union {
        struct { uint x, y, z; };
        Swz<uint, 3, 0, 1> xy;
        uint v_[3];
    };
    uvec3() = default;
    uvec3(const uvec3& o) { std::memcpy(v_, o.v_, sizeof v_); }
    uvec3& operator=(const uvec3& o) { std::memcpy(v_, o.v_, sizeof v_); return *this; }
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    uint& operator[](int i) { return v_[i]; }
    uint operator[](int i) const { return v_[i]; }
};
struct uvec4 {
    union {
        struct { uint x, y, z, w; };
        Swz<uint, 4, 0, 1> xy;
        uint v_[4];
    };
    uvec4() = default;
    uvec4(const uvec4& o) { std::memcpy(v_, o.v_, sizeof v_); }
    uvec4& operator=(const uvec4& o) { std::memcpy(v_, o.v_, sizeof v_); return *this; }
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
    uint& operator[](int i) { return v_[i]; }
    uint operator[](int i) const { return v_[i]; }
};

// ---- arithmetic (component-wise, in the order GLSL defines) ----
#define OHAO_GLSL_VEC_OPS(V, N)                                                                         \
    inline V operator+(V a, const V& b) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] + b.v_[i]; return a; } \
    inline V operator-(V a, const V& b) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] - b.v_[i]; return a; } \
    inline V operator*(V a, const V& b) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] * b.v_[i]; return a; } \
    inline V operator/(V a, const V& b) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] / b.v_[i]; return a; } \
    inline V operator+(V a, float s) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] + s; return a; }          \
    inline V operator-(V a, float s) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] - s; return a; }          \
    inline V operator*(V a, float s) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] * s; return a; }          \
    inline V operator/(V a, float s) { for (int i = 0; i < N; ++i) a.v_[i] = a.v_[i] / s; return a; }          \
    inline V operator+(float s, V a) { for (int i = 0; i < N; ++i) a.v_[i] = s + a.v_[i]; return a; }          \
    inline V operator-(float s, V a) { for (int i = 0; i < N; ++i) a.v_[i] = s - a.v_[i]; return a; }          \
    inline V operator*(float s, V a) { for (int i = 0; i < N; ++i) a.v_[i] = s * a.v_[i]; return a; }          \
    inline V operator/(float s, V a) { for (int i = 0; i < N; ++i) a.v_[i] = s / a.v_[i]; return a; }          \
    inline V operator-(V a) { for (int i = 0; i < N; ++i) a.v_[i] = -a.v_[i]; return a; }                     \
    inline V& operator+=(V& a, const V& b) { return a = a + b; }                                            \
    inline V& operator-=(V& a, const V& b) { return a = a - b; }                                            \
    inline V& operator*=(V& a, const V& b) { return a = a * b; }                                            \
    inline V& operator/=(V& a, const V& b) { return a = a / b; }                                            \
    inline V& operator+=(V& a, float s) { return a = a + s; }                                               \
    inline V& operator-=(V& a, float s) { return a = a - s; }                                               \
    inline V& operator*=(V& a, float s) { return a = a * s; }                                               \
    inline V& operator/=(V& a, float s) { return a = a / s; }
OHAO_GLSL_VEC_OPS(vec2, 2)
OHAO_GLSL_VEC_OPS(vec3, 3)
OHAO_GLSL_VEC_OPS(vec4, 4)
#undef OHAO_GLSL_VEC_OPS

inline ivec2 operator+(ivec2 a, ivec2 b) { return {a.x + b.x, a.y + b.y}; }
inline ivec2 operator-(ivec2 a, ivec2 b) { return {a.x - b.x, a.y - b.y}; }
inline ivec2 operator*(ivec2 a, ivec2 b) { return {a.x * b.x, a.y * b.y}; }
inline ivec2 operator+(ivec2 a, int s) { return {a.x + s, a.y + s}; }
inline ivec2 operator-(ivec2 a, int s) { return {a.x - s, a.y - s}; }
inline ivec2 operator*(ivec2 a, int s) { return {a.x * s, a.y * s}; }

// ---- matrices (column-major; m[c] is column c) ----
struct mat4x3 {
    vec3 c[4];
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat3 {
    vec3 c[3];
    mat3() = default;
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit mat3(const mat4x3& m) { c[0] = m.c[0]; c[1] = m.c[1]; c[2] = m.c[2]; }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int i = 0; i < 3; ++i) r.v_[i] = m.c[0].v_[i] * v.x + m.c[1].v_[i] * v.y + m.c[2].v_[i] * v.z;
    return r;
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r.v_[i] = m.c[0].v_[i] * v.x + m.c[1].v_[i] * v.y + m.c[2].v_[i] * v.z + m.c[3].v_[i] * v.w;
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = a * b.c[j];
    return r;
}
inline mat3 transpose(const mat3& m) {
    mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.c[i].v_[j] = m.c[j].v_[i];
    return r;
}
// Cofactors over the determinant in double, rounded to float: the oracle's
// instance normal-matrix computation.
inline mat3 inverse(const mat3& m) {
    const double a = m.c[0].x, b = m.c[1].x, c = m.c[2].x;   // row 0
    const double d = m.c[0].y, e = m.c[1].y, f = m.c[2].y;   // row 1
    const double g = m.c[0].z, h = m.c[1].z, i = m.c[2].z;   // row 2
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    const double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    const double det = a * A + b * B + c * C;
    const double inv[9] = {A / det, D / det, G / det, B / det, E / det, H / det, C / det, F / det, I / det};
    mat3 r;
    for (int row = 0; row < 3; ++row)
        for (int col = 0; col < 3; ++col) r.c[col].v_[row] = static_cast<float>(inv[row * 3 + col]);
    return r;
}
// General 4x4 inverse (Gauss-Jordan with partial pivoting, double); the
// shaders use it only for the motion-vector and depth outputs.
inline mat4 inverse(const mat4& m) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) { a[r][k] = m.c[k].v_[r]; a[r][k + 4] = r == k ? 1.0 : 0.0; }
    for (int col = 0; col < 4; ++col) {
        int p = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[p][col])) p = r;
        for (int k = 0; k < 8; ++k) std::swap(a[col][k], a[p][k]);
        const double piv = a[col][col];
        for (int k = 0; k < 8; ++k) a[col][k] /= piv;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            const double f = a[r][col];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[col][k];
        }
    }
    mat4 r;
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) r.c[col].v_[row] = static_cast<float>(a[row][col + 4]);
    return r;
}

// ---- built-in functions ----
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline float length(const vec2& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { float inv = 1.0f / length(a); return a * inv; }
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline vec3 abs(const vec3& a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float floor(float x) { return std::floor(x); }
inline float exp(float x) { return std::exp(x); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline vec3 max(const vec3& a, const vec3& b) { return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
inline vec3 min(const vec3& a, const vec3& b) { return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
inline vec3 max(const vec3& a, float b) { return {max(a.x, b), max(a.y, b), max(a.z, b)}; }
inline vec3 min(const vec3& a, float b) { return {min(a.x, b), min(a.y, b), min(a.z, b)}; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline vec3 clamp(const vec3& x, float lo, float hi) { return {clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi)}; }
inline ivec2 clamp(const ivec2& x, const ivec2& lo, const ivec2& hi) {
    return {clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y)};
}
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(const vec4& x, const vec4& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) {
    return {mix(x.x, y.x, a.x), mix(x.y, y.y, a.y), mix(x.z, y.z, a.z)};
}
// smoothstep as the GLSL specification writes it: t * t * (3 - 2 t)
inline float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
// GLSL leaves pow's precision to exp2(y * log2(x)) of the implementation:
// the oracle's definition (pow5 for the Schlick exponent, else exp2 / log2
// from their series).
inline float pow(float x, float y) { return orc::pow_def(x, y); }
inline vec3 pow(const vec3& x, const vec3& y) { return {pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)}; }
inline vec3 reflect(const vec3& i, const vec3& n) { float d = 2.0f * dot(n, i); return i - n * d; }
inline float radians(float deg) { return deg * 0.017453292f; }
inline float sin(float x) { return orc::sin_f(x); }
inline float cos(float x) { return orc::cos_f(x); }
inline float asin(float x) { return orc::asin_f(x); }
inline float acos(float x) { return orc::acos_f(x); }
inline float atan(float y, float x) { return orc::atan2_f(y, x); }
inline uint floatBitsToUint(float f) { return orc::f2u(f); }
inline float uintBitsToFloat(uint u) { return orc::u2f(u); }
template <class T> inline T nonuniformEXT(T x) { return x; }

// ---- resources ----
// env_sampling.glsl's CDF buffers as a helper-only translation unit binds
// them; the shader translation units declare their own.
struct FloatBuffer {
    const float* data;
};

// Storage image: RGBA32F texels, row-major (formats narrower than RGBA32F
// are stored unquantised; the comparisons read only RGBA32F images).
struct image2D {
    vec4* texels = nullptr;
    int width = 0, height = 0;
};
inline vec4 imageLoad(const image2D& im, ivec2 p) { return im.texels[static_cast<size_t>(p.y) * im.width + p.x]; }
inline void imageStore(image2D& im, ivec2 p, const vec4& v) { im.texels[static_cast<size_t>(p.y) * im.width + p.x] = v; }

// Combined image sampler: bilinear, REPEAT, texel centres at (i + 0.5) / n.
struct sampler2D {
    const float* rgba = nullptr;   // width * height RGBA32F texels
    int width = 0, height = 0;
};
inline vec4 texture(const sampler2D& s, const vec2& uv) {
    const int W = s.width, H = s.height;
    const float x = uv.x * float(W) - 0.5f;
    const float y = uv.y * float(H) - 0.5f;
    const float fx0 = std::floor(x), fy0 = std::floor(y);
    const float fx = x - fx0, fy = y - fy0;
    auto wrap = [](long long i, int n) { long long m = i % n; return static_cast<int>(m < 0 ? m + n : m); };
    const long long ix = static_cast<long long>(fx0), iy = static_cast<long long>(fy0);
    const int x0 = wrap(ix, W), x1 = wrap(ix + 1, W), y0 = wrap(iy, H), y1 = wrap(iy + 1, H);
    auto tex = [&](int xx, int yy) {
        const float* p = &s.rgba[(static_cast<size_t>(yy) * W + xx) * 4];
        return vec3(p[0], p[1], p[2]);
    };
    const vec3 top = tex(x0, y0) * (1.0f - fx) + tex(x1, y0) * fx;
    const vec3 bot = tex(x0, y1) * (1.0f - fx) + tex(x1, y1) * fx;
    auto alpha = [&](int xx, int yy) { return s.rgba[(static_cast<size_t>(yy) * W + xx) * 4 + 3]; };
    const float atop = alpha(x0, y0) * (1.0f - fx) + alpha(x1, y0) * fx;
    const float abot = alpha(x0, y1) * (1.0f - fx) + alpha(x1, y1) * fx;
    return vec4(top * (1.0f - fy) + bot * fy, atop * (1.0f - fy) + abot * fy);
}

}  // namespace glsl
