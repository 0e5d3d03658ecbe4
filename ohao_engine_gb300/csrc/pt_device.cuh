// pt_device.cuh -- device math, scene view and BVH traversal for sm_103a.
//
// Floating-point contract: this code is compiled with -fmad=false, so every
// a*b+c is two IEEE operations; fused multiply-adds appear only as explicit
// fmaf(). Division and sqrt are IEEE round-to-nearest (no fast-math). The
// transcendental functions GLSL leaves implementation-defined are defined
// here from Taylor series after Cody-Waite reduction (sin/cos) and a
// pi/6-shift reduction (atan2), so results are reproducible bit-for-bit by a
// host implementation of the same definitions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pt_types.hpp"

namespace ohao {

#define OHAO_HD __host__ __device__ __forceinline__
#define OHAO_D __device__ __forceinline__

// ---------------------------------------------------------------------------
// math
// ---------------------------------------------------------------------------
constexpr float kPio2Hi = 0x1.921fb6p+0f;
constexpr float kPio2Mid = -0x1.777a5cp-25f;
constexpr float kPio2Lo = -0x1.ee59dap-50f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPiF = 0x1.921fb6p+1f;
constexpr float kPiHalfF = 0x1.921fb6p+0f;
constexpr float kPiSixthF = 0x1.0c1524p-1f;
constexpr float kSqrt3F = 0x1.bb67aep+0f;
constexpr float kTanPi12F = 0x1.126146p-2f;

OHAO_D void sincos_f(float x, float* s_out, float* c_out) {
    float k = rintf(x * kTwoOverPi);
    float r = fmaf(-k, kPio2Hi, x);
    r = fmaf(-k, kPio2Mid, r);
    r = fmaf(-k, kPio2Lo, r);
    int q = static_cast<int>(k) & 3;
    float r2 = r * r;
    float ps = 1.0f / 362880.0f;
    ps = fmaf(ps, r2, -1.0f / 5040.0f);
    ps = fmaf(ps, r2, 1.0f / 120.0f);
    ps = fmaf(ps, r2, -1.0f / 6.0f);
    float s = fmaf(r2 * r, ps, r);
    float pc = -1.0f / 3628800.0f;
    pc = fmaf(pc, r2, 1.0f / 40320.0f);
    pc = fmaf(pc, r2, -1.0f / 720.0f);
    pc = fmaf(pc, r2, 1.0f / 24.0f);
    pc = fmaf(pc, r2, -0.5f);
    float c = fmaf(pc, r2, 1.0f);
    float so = (q == 0) ? s : (q == 1) ? c : (q == 2) ? -s : -c;
    float co = (q == 0) ? c : (q == 1) ? -s : (q == 2) ? -c : s;
    *s_out = so;
    *c_out = co;
}
OHAO_D float sin_f(float x) { float s, c; sincos_f(x, &s, &c); return s; }
OHAO_D float cos_f(float x) { float s, c; sincos_f(x, &s, &c); return c; }

OHAO_D float atan2_f(float y, float x) {
    float ax = fabsf(x), ay = fabsf(y);
    float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    float a = (mx > 0.0f) ? mn / mx : 0.0f;
    float off = 0.0f;
    float z = a;
    if (a > kTanPi12F) {
        z = (a * kSqrt3F - 1.0f) / (a + kSqrt3F);
        off = kPiSixthF;
    }
    float z2 = z * z;
    float p = -1.0f / 15.0f;
    p = fmaf(p, z2, 1.0f / 13.0f);
    p = fmaf(p, z2, -1.0f / 11.0f);
    p = fmaf(p, z2, 1.0f / 9.0f);
    p = fmaf(p, z2, -1.0f / 7.0f);
    p = fmaf(p, z2, 1.0f / 5.0f);
    p = fmaf(p, z2, -1.0f / 3.0f);
    float r = off + fmaf(z2 * z, p, z);
    if (ay > ax) r = kPiHalfF - r;
    if (x < 0.0f) r = kPiF - r;
    if (signbit(y)) r = -r;
    return r;
}
OHAO_D float asin_f(float x) { return atan2_f(x, sqrtf((1.0f - x) * (1.0f + x))); }
OHAO_D float acos_f(float x) { return atan2_f(sqrtf((1.0f - x) * (1.0f + x)), x); }

// pow(x, y) for x >= 0 as exp2(y * log2(x)), both defined here (GLSL leaves
// pow's precision to the implementation): log2 by the atanh series of
// s = (m - 1)/(m + 1) for x = m 2^e, m in [sqrt(1/2), sqrt(2)) (Abramowitz &
// Stegun 4.1.27, to s^11); exp2 by reduction to |f| <= 1/2 and the Taylor
// series of e^(f ln 2) to degree 9, scaled by 2^n from the exponent bits
// (below 2^-126 flushed to 0). The host oracle evaluates the same steps.
constexpr float kLn2F = 0x1.62e430p-1f;
constexpr float kLog2eF = 0x1.715476p+0f;
OHAO_D float log2_def(float x) {
    int e = 0;
    if (x < 0x1p-126f) { x = x * 0x1p23f; e = -23; }
    const uint32_t b = __float_as_uint(x);
    e += static_cast<int>((b >> 23) & 0xFFu) - 127;
    float m = __uint_as_float((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 1.0f / 11.0f;
    p = fmaf(p, s2, 1.0f / 9.0f);
    p = fmaf(p, s2, 1.0f / 7.0f);
    p = fmaf(p, s2, 1.0f / 5.0f);
    p = fmaf(p, s2, 1.0f / 3.0f);
    const float lnm = 2.0f * fmaf(s2 * s, p, s);
    return fmaf(lnm, kLog2eF, static_cast<float>(e));
}
OHAO_D float exp2_def(float y) {
    if (!(y >= -126.0f)) return y != y ? y : 0.0f;
    if (y > 127.0f) return INFINITY;
    const float n = rintf(y);
    const float z = (y - n) * kLn2F;
    float p = 1.0f / 362880.0f;
    p = fmaf(p, z, 1.0f / 40320.0f);
    p = fmaf(p, z, 1.0f / 5040.0f);
    p = fmaf(p, z, 1.0f / 720.0f);
    p = fmaf(p, z, 1.0f / 120.0f);
    p = fmaf(p, z, 1.0f / 24.0f);
    p = fmaf(p, z, 1.0f / 6.0f);
    p = fmaf(p, z, 0.5f);
    p = fmaf(p, z, 1.0f);
    p = fmaf(p, z, 1.0f);
    return p * __uint_as_float(static_cast<uint32_t>(static_cast<int>(n) + 127) << 23);
}
OHAO_D float pow5f(float x);
OHAO_D float pow_def(float x, float y) {
    if (y == 5.0f) return pow5f(x);
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : INFINITY);
    if (x == 1.0f || y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return NAN;
    return exp2_def(y * log2_def(x));
}

OHAO_D float gmaxf(float a, float b) { return a > b ? a : b; }
OHAO_D float gminf(float a, float b) { return a < b ? a : b; }
OHAO_D float gclampf(float x, float lo, float hi) { return gminf(gmaxf(x, lo), hi); }
OHAO_D float gmixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
OHAO_D float pow5f(float x) { float x2 = x * x; float x4 = x2 * x2; return x4 * x; }

struct V3 {
    float x, y, z;
};
OHAO_D V3 v3(float x, float y, float z) { return V3{x, y, z}; }
OHAO_D V3 v3s(float s) { return V3{s, s, s}; }
OHAO_D V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
OHAO_D V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
OHAO_D V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
OHAO_D V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
OHAO_D V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
OHAO_D V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
OHAO_D V3 operator-(float s, V3 a) { return {s - a.x, s - a.y, s - a.z}; }
OHAO_D V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
OHAO_D float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
OHAO_D V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
OHAO_D float length(V3 a) { return sqrtf(dot(a, a)); }
OHAO_D V3 normalize(V3 a) { float inv = 1.0f / length(a); return a * inv; }
OHAO_D V3 reflect(V3 i, V3 n) { float d = 2.0f * dot(n, i); return i - n * d; }
OHAO_D V3 vmix(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
OHAO_D float maxc(V3 a) { return gmaxf(a.x, gmaxf(a.y, a.z)); }
OHAO_D float lum(V3 a) { return dot(a, V3{0.2126f, 0.7152f, 0.0722f}); }
OHAO_D V3 ld3(const float4& f) { return {f.x, f.y, f.z}; }

// ---------------------------------------------------------------------------
// rays and triangles
// ---------------------------------------------------------------------------
struct RayPre {
    float o[3];
    float d[3];
    float invd[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

OHAO_D float sel3(const float v[3], int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

constexpr float kTinyDir = 0x1p-80f;

OHAO_D RayPre ray_pre(V3 o, V3 d) {
    RayPre r;
    r.o[0] = o.x; r.o[1] = o.y; r.o[2] = o.z;
    r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float dd = fabsf(r.d[k]) > kTinyDir ? r.d[k] : copysignf(kTinyDir, r.d[k]);
        r.invd[k] = 1.0f / dd;
    }
    int kz = 0;
    if (fabsf(d.y) > fabsf(d.x)) kz = 1;
    if (fabsf(d.z) > fabsf(sel3(r.d, kz))) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (sel3(r.d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    float dz = sel3(r.d, kz);
    r.Sx = sel3(r.d, kx) / dz;
    r.Sy = sel3(r.d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}

// Woop-Benthin-Wald watertight ray/triangle test (JCGT 2013), t in (tmin,tmax).
OHAO_D bool tri_intersect(const RayPre& r, float4 v0, float4 v1, float4 v2, float tmin, float tmax, float& t_out,
                          float& u_out, float& v_out) {
    float A[3] = {v0.x - r.o[0], v0.y - r.o[1], v0.z - r.o[2]};
    float B[3] = {v1.x - r.o[0], v1.y - r.o[1], v1.z - r.o[2]};
    float C[3] = {v2.x - r.o[0], v2.y - r.o[1], v2.z - r.o[2]};
    const float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    float Ax = sel3(A, r.kx) - r.Sx * Akz;
    float Ay = sel3(A, r.ky) - r.Sy * Akz;
    float Bx = sel3(B, r.kx) - r.Sx * Bkz;
    float By = sel3(B, r.ky) - r.Sy * Bkz;
    float Cx = sel3(C, r.kx) - r.Sx * Ckz;
    float Cy = sel3(C, r.ky) - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = static_cast<double>(Cx) * static_cast<double>(By);
        double CyBx = static_cast<double>(Cy) * static_cast<double>(Bx);
        U = static_cast<float>(__dsub_rn(CxBy, CyBx));
        double AxCy = static_cast<double>(Ax) * static_cast<double>(Cy);
        double AyCx = static_cast<double>(Ay) * static_cast<double>(Cx);
        V = static_cast<float>(__dsub_rn(AxCy, AyCx));
        double BxAy = static_cast<double>(Bx) * static_cast<double>(Ay);
        double ByAx = static_cast<double>(By) * static_cast<double>(Ax);
        W = static_cast<float>(__dsub_rn(BxAy, ByAx));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * Akz;
    float Bz = r.Sz * Bkz;
    float Cz = r.Sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// ---------------------------------------------------------------------------
// bindless textures: RGBA8 UNORM texel c read as c / 255, sampled LINEAR /
// REPEAT at LOD 0 with texel centres at (i + 0.5) / size (the hardware
// sampler of the reference's texture array, restated in float)
// ---------------------------------------------------------------------------
OHAO_D int wrap_texel(long long i, int n) {
    const long long m = i % n;
    return static_cast<int>(m < 0 ? m + n : m);
}
OHAO_D float4 unorm4(uchar4 c) {
    return make_float4(static_cast<float>(c.x) / 255.0f, static_cast<float>(c.y) / 255.0f,
                       static_cast<float>(c.z) / 255.0f, static_cast<float>(c.w) / 255.0f);
}
OHAO_D float4 tex_sample(const DScene& sc, uint32_t idx, float u, float v) {
    const uint4 ti = __ldg(sc.tex_info + idx);
    const int W = static_cast<int>(ti.y), H = static_cast<int>(ti.z);
    const float x = u * static_cast<float>(W) - 0.5f;
    const float y = v * static_cast<float>(H) - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float fx = x - fx0, fy = y - fy0;
    const long long ix = static_cast<long long>(fx0), iy = static_cast<long long>(fy0);
    const int x0 = wrap_texel(ix, W), x1 = wrap_texel(ix + 1, W), y0 = wrap_texel(iy, H), y1 = wrap_texel(iy + 1, H);
    const uchar4* t = sc.tex + ti.x;
    const float4 t00 = unorm4(t[static_cast<size_t>(y0) * W + x0]), t10 = unorm4(t[static_cast<size_t>(y0) * W + x1]);
    const float4 t01 = unorm4(t[static_cast<size_t>(y1) * W + x0]), t11 = unorm4(t[static_cast<size_t>(y1) * W + x1]);
    float4 r;
    const float top_x = t00.x * (1.0f - fx) + t10.x * fx, bot_x = t01.x * (1.0f - fx) + t11.x * fx;
    const float top_y = t00.y * (1.0f - fx) + t10.y * fx, bot_y = t01.y * (1.0f - fx) + t11.y * fx;
    const float top_z = t00.z * (1.0f - fx) + t10.z * fx, bot_z = t01.z * (1.0f - fx) + t11.z * fx;
    const float top_w = t00.w * (1.0f - fx) + t10.w * fx, bot_w = t01.w * (1.0f - fx) + t11.w * fx;
    r.x = top_x * (1.0f - fy) + bot_x * fy;
    r.y = top_y * (1.0f - fy) + bot_y * fy;
    r.z = top_z * (1.0f - fy) + bot_z * fy;
    r.w = top_w * (1.0f - fy) + bot_w * fy;
    return r;
}

// pt_anyhit.rahit:17-50 for rays traced without gl_RayFlagsOpaqueEXT: a
// candidate hit on a non-opaque instance whose material's diffuse texture
// has alpha < 0.5 at the hit's UV is ignored. Opaque instances, materials
// without a diffuse texture and the tile albedo map (no alpha) accept.
// Out of line: it runs only for candidate hits of non-opaque geometry, and
// inlined into the traversal loops it would raise their register count.
OHAO_D bool alpha_accept(const DScene& sc, uint32_t inst, uint32_t prim, float u, float v) {
    const DInst& in = sc.inst[inst];
    if (!(__ldg(&in.mask) & kInstNoOpaque)) return true;
    const uint32_t gtri = (__ldg(&in.custom) & 0xFFFFFFu) + prim;
    const uint32_t mid = __ldg(sc.mat_ids + gtri);
    const uint32_t dtex = __float_as_uint(__ldg(&sc.mats[mid * 3].w));
    if (dtex == 0xFFFFFFFFu || (dtex == 0u && sc.map_w > 0)) return true;
    const uint32_t i0 = __ldg(sc.indices + gtri * 3), i1 = __ldg(sc.indices + gtri * 3 + 1),
                   i2 = __ldg(sc.indices + gtri * 3 + 2);
    const float2 uv0 = __ldg(sc.uvs + i0), uv1 = __ldg(sc.uvs + i1), uv2 = __ldg(sc.uvs + i2);
    const float w = 1.0f - u - v;
    const float tu = w * uv0.x + u * uv1.x + v * uv2.x;
    const float tv = w * uv0.y + u * uv1.y + v * uv2.y;
    return !(tex_sample(sc, dtex, tu, tv).w < 0.5f);
}

}  // namespace ohao

#include "pt_traverse.cuh"
