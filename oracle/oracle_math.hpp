// oracle_math.hpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// Scalar/vector arithmetic for the CPU restatement of OHAO's path-tracing
// shaders. Only tests/, the smoke check and bench.py's CPU-baseline leg load
// the oracle; the product library never links it.
//
// Floating-point contract (shared, by specification, with the CUDA kernels):
//   * every expression is evaluated left to right exactly as written, with no
//     FMA contraction (the oracle is compiled with -ffp-contract=off; the
//     device code is compiled with -fmad=false); fused multiply-adds appear
//     only where `fma_` is written explicitly;
//   * division and sqrt are IEEE-754 round-to-nearest on both sides;
//   * the transcendental functions GLSL leaves implementation-defined
//     (sin, cos, atan, asin, acos, pow) are defined here from their Taylor
//     series after Cody-Waite / half-angle style range reduction, so that the
//     CPU and the GPU evaluate the same formula.
// The GLSL built-ins are restated from the GLSL 4.60 specification
// (mix(x,y,a) = x*(1-a) + y*a, reflect(I,N) = I - 2*dot(N,I)*N, ...).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace orc {

inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// ---- float transcendental functions (definitions shared with the device) ----
// pi/2 split for Cody-Waite reduction with FMA: hi = fl(pi/2), mid/lo = the
// rounded remainders.
constexpr float kPio2Hi = 0x1.921fb6p+0f;
constexpr float kPio2Mid = -0x1.777a5cp-25f;
constexpr float kPio2Lo = -0x1.ee59dap-50f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPiF = 0x1.921fb6p+1f;
constexpr float kPiHalfF = 0x1.921fb6p+0f;
constexpr float kPiSixthF = 0x1.0c1524p-1f;
constexpr float kSqrt3F = 0x1.bb67aep+0f;
constexpr float kTanPi12F = 0x1.126146p-2f;

// sin and cos of x for |x| < 2^17: k = rint(x*2/pi), r = x - k*pi/2 (three
// FMA steps), Taylor polynomials of degree 9 (sin) and 10 (cos) on
// |r| <= pi/4, quadrant selected by k mod 4.
inline void sincos_f(float x, float* s_out, float* c_out) {
    float k = std::rint(x * kTwoOverPi);
    float r = fma_(-k, kPio2Hi, x);
    r = fma_(-k, kPio2Mid, r);
    r = fma_(-k, kPio2Lo, r);
    int q = static_cast<int>(k) & 3;
    float r2 = r * r;
    float ps = 1.0f / 362880.0f;
    ps = fma_(ps, r2, -1.0f / 5040.0f);
    ps = fma_(ps, r2, 1.0f / 120.0f);
    ps = fma_(ps, r2, -1.0f / 6.0f);
    float s = fma_(r2 * r, ps, r);
    float pc = -1.0f / 3628800.0f;
    pc = fma_(pc, r2, 1.0f / 40320.0f);
    pc = fma_(pc, r2, -1.0f / 720.0f);
    pc = fma_(pc, r2, 1.0f / 24.0f);
    pc = fma_(pc, r2, -0.5f);
    float c = fma_(pc, r2, 1.0f);
    float so, co;
    switch (q) {
        case 0: so = s; co = c; break;
        case 1: so = c; co = -s; break;
        case 2: so = -s; co = -c; break;
        default: so = -c; co = s; break;
    }
    *s_out = so;
    *c_out = co;
}
inline float sin_f(float x) { float s, c; sincos_f(x, &s, &c); return s; }
inline float cos_f(float x) { float s, c; sincos_f(x, &s, &c); return c; }

// atan2: reduce to a = min/max in [0,1]; if a > tan(pi/12) use
// atan(a) = pi/6 + atan((a*sqrt3 - 1)/(a + sqrt3)); Taylor series to z^15.
inline float atan2_f(float y, float x) {
    float ax = std::fabs(x), ay = std::fabs(y);
    float mx = std::max(ax, ay), mn = std::min(ax, ay);
    float a = (mx > 0.0f) ? mn / mx : 0.0f;
    float off = 0.0f;
    float z = a;
    if (a > kTanPi12F) {
        z = (a * kSqrt3F - 1.0f) / (a + kSqrt3F);
        off = kPiSixthF;
    }
    float z2 = z * z;
    float p = -1.0f / 15.0f;
    p = fma_(p, z2, 1.0f / 13.0f);
    p = fma_(p, z2, -1.0f / 11.0f);
    p = fma_(p, z2, 1.0f / 9.0f);
    p = fma_(p, z2, -1.0f / 7.0f);
    p = fma_(p, z2, 1.0f / 5.0f);
    p = fma_(p, z2, -1.0f / 3.0f);
    float r = off + fma_(z2 * z, p, z);
    if (ay > ax) r = kPiHalfF - r;
    if (x < 0.0f) r = kPiF - r;
    if (std::signbit(y)) r = -r;
    return r;
}
inline float asin_f(float x) { return atan2_f(x, std::sqrt((1.0f - x) * (1.0f + x))); }
inline float acos_f(float x) { return atan2_f(std::sqrt((1.0f - x) * (1.0f + x)), x); }

// GLSL pow(x, 5.0) as used by the Schlick terms: ((x*x)*(x*x))*x.
template <class T> inline T pow5(T x) { T x2 = x * x; T x4 = x2 * x2; return x4 * x; }

// pow(x, y) for x >= 0 as exp2(y * log2(x)), each defined here (GLSL leaves
// pow's precision to exp2 and log2 of the implementation):
//   log2(x): x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s),
//            s = (m - 1) / (m + 1), by the atanh series to s^11 (|s| < 0.172;
//            Abramowitz & Stegun 4.1.27); log2 x = e + ln m / ln 2.
//   exp2(y): y = n + f, n = rint(y), |f| <= 1/2; 2^f = e^(f ln 2) by its
//            Taylor series to degree 9; times 2^n built from the exponent
//            bits (results below 2^-126 flush to 0).
constexpr float kLn2F = 0x1.62e430p-1f;
constexpr float kLog2eF = 0x1.715476p+0f;
inline float log2_def(float x) {
    int e = 0;
    if (x < 0x1p-126f) { x = x * 0x1p23f; e = -23; }
    const uint32_t b = f2u(x);
    e += static_cast<int>((b >> 23) & 0xFFu) - 127;
    float m = u2f((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 1.0f / 11.0f;
    p = fma_(p, s2, 1.0f / 9.0f);
    p = fma_(p, s2, 1.0f / 7.0f);
    p = fma_(p, s2, 1.0f / 5.0f);
    p = fma_(p, s2, 1.0f / 3.0f);
    const float lnm = 2.0f * fma_(s2 * s, p, s);
    return fma_(lnm, kLog2eF, static_cast<float>(e));
}
inline float exp2_def(float y) {
    if (!(y >= -126.0f)) return y != y ? y : 0.0f;
    if (y > 127.0f) return INFINITY;
    const float n = std::rint(y);
    const float z = (y - n) * kLn2F;
    float p = 1.0f / 362880.0f;
    p = fma_(p, z, 1.0f / 40320.0f);
    p = fma_(p, z, 1.0f / 5040.0f);
    p = fma_(p, z, 1.0f / 720.0f);
    p = fma_(p, z, 1.0f / 120.0f);
    p = fma_(p, z, 1.0f / 24.0f);
    p = fma_(p, z, 1.0f / 6.0f);
    p = fma_(p, z, 0.5f);
    p = fma_(p, z, 1.0f);
    p = fma_(p, z, 1.0f);
    return p * u2f(static_cast<uint32_t>(static_cast<int>(n) + 127) << 23);
}
inline float pow_def(float x, float y) {
    if (y == 5.0f) return pow5(x);
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : INFINITY);
    if (x == 1.0f || y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return NAN;
    return exp2_def(y * log2_def(x));
}

// ---- Real-dispatched scalar functions ----
inline float m_sin(float x) { return sin_f(x); }
inline float m_cos(float x) { return cos_f(x); }
inline float m_atan2(float y, float x) { return atan2_f(y, x); }
inline float m_asin(float x) { return asin_f(x); }
inline float m_acos(float x) { return acos_f(x); }
inline float m_sqrt(float x) { return std::sqrt(x); }
inline double m_sin(double x) { return std::sin(x); }
inline double m_cos(double x) { return std::cos(x); }
inline double m_atan2(double y, double x) { return std::atan2(y, x); }
inline double m_asin(double x) { return std::asin(x); }
inline double m_acos(double x) { return std::acos(x); }
inline double m_sqrt(double x) { return std::sqrt(x); }
inline float m_pow(float x, float y) { return pow_def(x, y); }
inline double m_pow(double x, double y) { return y == 5.0 ? (x * x) * (x * x) * x : std::pow(x, y); }

// GLSL min/max/clamp (IEEE fmin/fmax semantics for non-NaN inputs).
template <class T> inline T gmax(T a, T b) { return a > b ? a : b; }
template <class T> inline T gmin(T a, T b) { return a < b ? a : b; }
template <class T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline T gmix(T a, T b, T t) { return a * (T(1) - t) + b * t; }

template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    template <class U> explicit V3(const V3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> inline V3<T> operator+(T s, V3<T> a) { return {s + a.x, s + a.y, s + a.z}; }
template <class T> inline V3<T> operator-(T s, V3<T> a) { return {s - a.x, s - a.y, s - a.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T length(V3<T> a) { return m_sqrt(dot(a, a)); }
// normalize(v) = v * (1/length(v)).
template <class T> inline V3<T> normalize(V3<T> a) { T inv = T(1) / length(a); return a * inv; }
template <class T> inline V3<T> reflect(V3<T> i, V3<T> n) { T d = T(2) * dot(n, i); return i - n * d; }
template <class T> inline V3<T> vmix(V3<T> a, V3<T> b, T t) { return a * (T(1) - t) + b * t; }
template <class T> inline V3<T> vmix(V3<T> a, V3<T> b, V3<T> t) {
    return {gmix(a.x, b.x, t.x), gmix(a.y, b.y, t.y), gmix(a.z, b.z, t.z)};
}
template <class T> inline T maxc(V3<T> a) { return gmax(a.x, gmax(a.y, a.z)); }
template <class T> inline T lum(V3<T> a) { return dot(a, V3<T>(T(0.2126f), T(0.7152f), T(0.0722f))); }

}  // namespace orc
