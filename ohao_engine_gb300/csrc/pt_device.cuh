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
// 8-wide node: 80 bytes = 5 x uint4 (layout of ohao_bvh8_node)
// ---------------------------------------------------------------------------
constexpr float kTravRelSlack = 0x1p-14f;
constexpr float kTravAbsScale = 0x1p-21f;
constexpr int kStackSize = 64;

OHAO_D uint32_t byte_of(uint32_t lo4, uint32_t hi4, int i) {
    uint32_t w = (i < 4) ? lo4 : hi4;
    return (w >> ((i & 3) * 8)) & 0xFFu;
}

struct NodeHits {
    uint32_t hitmask;     // slots whose box the ray overlaps
    float tn[8];
};

// Slab test of the 8 child boxes in the node's quantized frame, with
// conservative per-axis margins folded into the offsets.
OHAO_D void node_test(const uint4 q0, const uint4 q1, const uint4 q2, const uint4 q3, const uint4 q4, const RayPre& r,
                      float tmin, float tbest, NodeHits& h) {
    const float org[3] = {__uint_as_float(q0.x), __uint_as_float(q0.y), __uint_as_float(q0.z)};
    float a[3], bn[3], bf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int e = static_cast<int>(static_cast<int8_t>((q0.w >> (8 * k)) & 0xFFu));
        float s = __int_as_float((e + 127) << 23);
        a[k] = s * r.invd[k];
        float b = (org[k] - r.o[k]) * r.invd[k];
        float m = 255.0f * fabsf(a[k]) + fabsf(b);
        m = m * kTravAbsScale;
        bn[k] = b - m;
        bf[k] = b + m;
    }
    const float tlimit = tbest + tbest * kTravRelSlack;
    h.hitmask = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t meta = byte_of(q1.z, q1.w, i);
        const float lox = static_cast<float>(byte_of(q2.x, q2.y, i));
        const float loy = static_cast<float>(byte_of(q2.z, q2.w, i));
        const float loz = static_cast<float>(byte_of(q3.x, q3.y, i));
        const float hix = static_cast<float>(byte_of(q3.z, q3.w, i));
        const float hiy = static_cast<float>(byte_of(q4.x, q4.y, i));
        const float hiz = static_cast<float>(byte_of(q4.z, q4.w, i));
        const float nx = r.invd[0] < 0.0f ? hix : lox, fx = r.invd[0] < 0.0f ? lox : hix;
        const float ny = r.invd[1] < 0.0f ? hiy : loy, fy = r.invd[1] < 0.0f ? loy : hiy;
        const float nz = r.invd[2] < 0.0f ? hiz : loz, fz = r.invd[2] < 0.0f ? loz : hiz;
        float tn = fmaxf(fmaxf(fmaf(nx, a[0], bn[0]), fmaf(ny, a[1], bn[1])), fmaf(nz, a[2], bn[2]));
        float tf = fminf(fminf(fmaf(fx, a[0], bf[0]), fmaf(fy, a[1], bf[1])), fmaf(fz, a[2], bf[2]));
        h.tn[i] = tn;
        if (meta != 0u && tn <= tf && tn <= tlimit && tf >= tmin) h.hitmask |= 1u << i;
    }
}

struct Hit {
    float t, u, v;
    uint32_t inst, prim;
};

OHAO_D bool key_less(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb) {
    return ia < ib || (ia == ib && pa < pb);
}

struct TravCount {
    uint32_t nodes, tris;
};

// Closest-hit traversal of one BVH (flat, or a BLAS with inst_override).
// `stack_base` lets a BLAS traversal run above the TLAS entries.
template <bool kStats>
OHAO_D void bvh_closest(const uint4* __restrict__ nodes, const float4* __restrict__ tris, const RayPre& r,
                        float tmin, float tmax, Hit& best, uint32_t inst_override, uint32_t* st_node, float* st_t,
                        int stack_base, TravCount& cnt, int& err) {
    if (stack_base >= kStackSize) { err = 1; return; }
    int sp = stack_base;
    st_node[sp] = 0u;
    st_t[sp] = -INFINITY;
    sp++;
    while (sp > stack_base) {
        sp--;
        const uint32_t ni = st_node[sp];
        const float tn0 = st_t[sp];
        {
            const float tb = best.prim != 0xFFFFFFFFu ? best.t : tmax;
            if (tn0 > tb + tb * kTravRelSlack) continue;
        }
        const uint4* np = nodes + static_cast<size_t>(ni) * 5;
        const uint4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
        if (kStats) cnt.nodes++;
        NodeHits h;
        node_test(q0, q1, q2, q3, q4, r, tmin, best.prim != 0xFFFFFFFFu ? best.t : tmax, h);
        const uint32_t imask = q0.w >> 24;
        uint32_t leafmask = h.hitmask & ~imask;
        while (leafmask) {
            const int i = __ffs(leafmask) - 1;
            leafmask &= leafmask - 1;
            const uint32_t meta = byte_of(q1.z, q1.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const float4* tp = tris + static_cast<size_t>(q1.y + off + q) * 3;
                const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                if (kStats) cnt.tris++;
                float t, u, v;
                if (!tri_intersect(r, v0, v1, v2, tmin, tmax, t, u, v)) continue;
                const uint32_t prim = __float_as_uint(v0.w);
                const uint32_t inst = (inst_override != 0xFFFFFFFFu) ? inst_override : __float_as_uint(v1.w);
                if (best.prim == 0xFFFFFFFFu || t < best.t || (t == best.t && key_less(inst, prim, best.inst, best.prim))) {
                    best.t = t; best.u = u; best.v = v; best.inst = inst; best.prim = prim;
                }
            }
        }
        // internal children: stable sort by tnear descending, push far first
        const uint32_t inner = h.hitmask & imask;
        if (inner) {
            float key[8];
            uint32_t id[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const bool c = (inner >> i) & 1u;
                key[i] = c ? h.tn[i] : -INFINITY;
                id[i] = q1.x + (byte_of(q1.z, q1.w, i) & 7u);
            }
            // compact candidates to the front keeping slot order
            float k2[8];
            uint32_t i2[8];
            int n = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) { k2[i] = -INFINITY; i2[i] = 0u; }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const bool c = (inner >> i) & 1u;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (c && j == n) { k2[j] = key[i]; i2[j] = id[i]; }
                }
                n += c ? 1 : 0;
            }
#pragma unroll
            for (int i = 1; i < 8; ++i) {
#pragma unroll
                for (int j = i; j > 0; --j) {
                    if (j < n && k2[j] > k2[j - 1]) {
                        float tk = k2[j]; k2[j] = k2[j - 1]; k2[j - 1] = tk;
                        uint32_t ti = i2[j]; i2[j] = i2[j - 1]; i2[j - 1] = ti;
                    }
                }
            }
            if (sp + n > kStackSize) { err = 1; return; }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (i < n) { st_node[sp] = i2[i]; st_t[sp] = k2[i]; sp++; }
            }
        }
    }
}

template <bool kStats>
OHAO_D bool bvh_any(const uint4* __restrict__ nodes, const float4* __restrict__ tris, const RayPre& r, float tmin,
                    float tmax, uint32_t* st_node, int stack_base, TravCount& cnt, int& err) {
    if (stack_base >= kStackSize) { err = 1; return false; }
    int sp = stack_base;
    st_node[sp++] = 0u;
    while (sp > stack_base) {
        const uint32_t ni = st_node[--sp];
        const uint4* np = nodes + static_cast<size_t>(ni) * 5;
        const uint4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
        if (kStats) cnt.nodes++;
        NodeHits h;
        node_test(q0, q1, q2, q3, q4, r, tmin, tmax, h);
        const uint32_t imask = q0.w >> 24;
        uint32_t m = h.hitmask;
        while (m) {
            const int i = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t meta = byte_of(q1.z, q1.w, i);
            if ((imask >> i) & 1u) {
                if (sp >= kStackSize) { err = 1; return false; }
                st_node[sp++] = q1.x + (meta & 7u);
                continue;
            }
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const float4* tp = tris + static_cast<size_t>(q1.y + off + q) * 3;
                const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                if (kStats) cnt.tris++;
                float t, u, v;
                if (tri_intersect(r, v0, v1, v2, tmin, tmax, t, u, v)) return true;
            }
        }
    }
    return false;
}

OHAO_D void xform_point(const float m[12], V3 p, V3& o) {
    o.x = ((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3];
    o.y = ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7];
    o.z = ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11];
}
OHAO_D void xform_dir(const float m[12], V3 d, V3& o) {
    o.x = (m[0] * d.x + m[1] * d.y) + m[2] * d.z;
    o.y = (m[4] * d.x + m[5] * d.y) + m[6] * d.z;
    o.z = (m[8] * d.x + m[9] * d.y) + m[10] * d.z;
}

// Scene-level closest hit (flat or two-level). tmax <= tmin means no hit.
template <bool kStats>
OHAO_D Hit scene_closest(const DScene& sc, V3 o, V3 d, float tmin, float tmax, TravCount& cnt, int& err) {
    Hit best;
    best.t = 0.0f; best.u = 0.0f; best.v = 0.0f;
    best.inst = 0xFFFFFFFFu; best.prim = 0xFFFFFFFFu;
    if (!(tmax > tmin) || sc.nnodes == 0) return best;
    uint32_t st_node[kStackSize];
    float st_t[kStackSize];
    const RayPre r = ray_pre(o, d);
    if (!sc.two_level) {
        bvh_closest<kStats>(sc.nodes, sc.tris, r, tmin, tmax, best, 0xFFFFFFFFu, st_node, st_t, 0, cnt, err);
        return best;
    }
    int sp = 0;
    st_node[sp] = 0u; st_t[sp] = -INFINITY; sp++;
    while (sp > 0) {
        sp--;
        const uint32_t ni = st_node[sp];
        const float tn0 = st_t[sp];
        {
            const float tb = best.prim != 0xFFFFFFFFu ? best.t : tmax;
            if (tn0 > tb + tb * kTravRelSlack) continue;
        }
        const uint4* np = sc.nodes + static_cast<size_t>(ni) * 5;
        const uint4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
        if (kStats) cnt.nodes++;
        NodeHits h;
        node_test(q0, q1, q2, q3, q4, r, tmin, best.prim != 0xFFFFFFFFu ? best.t : tmax, h);
        const uint32_t imask = q0.w >> 24;
        uint32_t leafmask = h.hitmask & ~imask;
        while (leafmask) {
            const int i = __ffs(leafmask) - 1;
            leafmask &= leafmask - 1;
            const uint32_t meta = byte_of(q1.z, q1.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const uint32_t ii = __ldg(sc.tlas_inst + q1.y + off + q);
                const DInst& in = sc.inst[ii];
                const DBlas bl = sc.blas[in.blas];
                V3 oo, od;
                xform_point(in.w2o, o, oo);
                xform_dir(in.w2o, d, od);
                const RayPre ro = ray_pre(oo, od);
                bvh_closest<kStats>(sc.blas_nodes + static_cast<size_t>(bl.node_off) * 5,
                                    sc.blas_tris + static_cast<size_t>(bl.tri_off) * 3, ro, tmin, tmax, best, ii,
                                    st_node, st_t, sp, cnt, err);
                if (err) return best;
            }
        }
        const uint32_t inner = h.hitmask & imask;
        if (inner) {
            float k2[8];
            uint32_t i2[8];
            int n = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) { k2[i] = -INFINITY; i2[i] = 0u; }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const bool c = (inner >> i) & 1u;
                const float key = h.tn[i];
                const uint32_t id = q1.x + (byte_of(q1.z, q1.w, i) & 7u);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (c && j == n) { k2[j] = key; i2[j] = id; }
                }
                n += c ? 1 : 0;
            }
#pragma unroll
            for (int i = 1; i < 8; ++i) {
#pragma unroll
                for (int j = i; j > 0; --j) {
                    if (j < n && k2[j] > k2[j - 1]) {
                        float tk = k2[j]; k2[j] = k2[j - 1]; k2[j - 1] = tk;
                        uint32_t ti = i2[j]; i2[j] = i2[j - 1]; i2[j - 1] = ti;
                    }
                }
            }
            if (sp + n > kStackSize) { err = 1; return best; }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (i < n) { st_node[sp] = i2[i]; st_t[sp] = k2[i]; sp++; }
            }
        }
    }
    return best;
}

template <bool kStats>
OHAO_D bool scene_occluded(const DScene& sc, V3 o, V3 d, float tmin, float tmax, TravCount& cnt, int& err) {
    if (!(tmax > tmin) || sc.nnodes == 0) return false;
    uint32_t st_node[kStackSize];
    const RayPre r = ray_pre(o, d);
    if (!sc.two_level) return bvh_any<kStats>(sc.nodes, sc.tris, r, tmin, tmax, st_node, 0, cnt, err);
    int sp = 0;
    st_node[sp++] = 0u;
    while (sp > 0) {
        const uint32_t ni = st_node[--sp];
        const uint4* np = sc.nodes + static_cast<size_t>(ni) * 5;
        const uint4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
        if (kStats) cnt.nodes++;
        NodeHits h;
        node_test(q0, q1, q2, q3, q4, r, tmin, tmax, h);
        const uint32_t imask = q0.w >> 24;
        uint32_t m = h.hitmask;
        while (m) {
            const int i = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t meta = byte_of(q1.z, q1.w, i);
            if ((imask >> i) & 1u) {
                if (sp >= kStackSize) { err = 1; return false; }
                st_node[sp++] = q1.x + (meta & 7u);
                continue;
            }
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const uint32_t ii = __ldg(sc.tlas_inst + q1.y + off + q);
                const DInst& in = sc.inst[ii];
                const DBlas bl = sc.blas[in.blas];
                V3 oo, od;
                xform_point(in.w2o, o, oo);
                xform_dir(in.w2o, d, od);
                const RayPre ro = ray_pre(oo, od);
                if (bvh_any<kStats>(sc.blas_nodes + static_cast<size_t>(bl.node_off) * 5,
                                    sc.blas_tris + static_cast<size_t>(bl.tri_off) * 3, ro, tmin, tmax, st_node, sp,
                                    cnt, err))
                    return true;
                if (err) return false;
            }
        }
    }
    return false;
}

}  // namespace ohao
