// glsl_shim.hpp -- TEST INFRASTRUCTURE ONLY (pins the CPU oracle).
//
// The subset of GLSL 4.60 types and built-ins that the reference's shader
// include files use (scalar uint/int/float, vec2, vec3, uvec2; dot, cross,
// normalize, inversesqrt, sqrt, abs, min, max, clamp, sin, cos, acos and
// two-argument atan), so that those files compile unchanged as C++ inside
// namespace glsl. The built-ins GLSL leaves implementation-defined take the
// oracle's definitions (oracle_math.hpp), which are also the device's: the
// comparison then checks the order of operations the oracle restates, not a
// math library. GLSL's float literals are single precision: the translation
// unit that includes this header is compiled with -fsingle-precision-constant
// and -ffp-contract=off.
#pragma once
#include <cmath>
#include <cstdint>

#include "oracle_math.hpp"

namespace glsl {

using uint = std::uint32_t;

struct vec2 {
    float x, y;
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(float a) : x(a), y(a) {}
};
struct vec3 {
    float x, y, z;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(float a) : x(a), y(a), z(a) {}
};
struct uvec2 {
    uint x, y;
    uvec2() = default;
    uvec2(uint a, uint b) : x(a), y(b) {}
};

inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator*(vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(vec3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }

inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
// the oracle's (and the device's) normalize: v * (1 / length(v))
inline vec3 normalize(vec3 a) { float inv = 1.0f / length(a); return a * inv; }
inline float abs(float x) { return std::fabs(x); }
// max/min: the oracle's (and the device's) choice at equal operands, where
// GLSL leaves the sign of a zero result open
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float sin(float x) { return orc::sin_f(x); }
inline float cos(float x) { return orc::cos_f(x); }
inline float acos(float x) { return orc::acos_f(x); }
inline float atan(float y, float x) { return orc::atan2_f(y, x); }

// env_sampling.glsl reads the CDFs through two storage buffers the including
// shader declares (`envMarg.data[]`, `envCond.data[]`).
struct FloatBuffer {
    const float* data;
};
inline FloatBuffer envMarg{nullptr}, envCond{nullptr};

}  // namespace glsl
