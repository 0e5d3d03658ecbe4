// pt_path.cuh -- the reference path estimator as a resumable per-bounce step.
//
// Restates shaders/rt/pt_raygen.rgen main() (stages A/B/C, 126-1186),
// pt_closesthit.rchit (37-162), pt_miss.rmiss (52-81) and
// includes/rt/env_sampling.glsl (16-94) for CUDA. A path is a small state
// machine so that the wavefront driver can keep it in SoA arrays between
// kernels and the persistent driver can keep it in registers:
//   phase 0  primary ray pending          (stage A)
//   phase 1  specular chain, bounce b     (stage B, 503-827)
//   phase 2  diffuse chain, bounce b      (stage C, 830-1133)
//   phase 3  done
// The shadow rays a step emits (light NEE, env NEE) are resolved before the
// next step of the same path, so radiance is summed in the shader's order.
#pragma once
#include "env_guide.hpp"
#include "pt_device.cuh"

namespace ohao {

// Sobol direction numbers, dimensions 0-3 x 32 bits: the table of
// shaders/includes/rt/sampler_sobol_tables.glsl:10-47 (data, not derivable:
// dimension 2 is not the textbook Joe-Kuo dimension). Initialised statically
// so that every translation unit that includes this header carries it.
__constant__ uint32_t c_sobol_dirs[128] = {
    0x80000000u, 0x40000000u, 0x20000000u, 0x10000000u, 0x08000000u, 0x04000000u, 0x02000000u, 0x01000000u,
    0x00800000u, 0x00400000u, 0x00200000u, 0x00100000u, 0x00080000u, 0x00040000u, 0x00020000u, 0x00010000u,
    0x00008000u, 0x00004000u, 0x00002000u, 0x00001000u, 0x00000800u, 0x00000400u, 0x00000200u, 0x00000100u,
    0x00000080u, 0x00000040u, 0x00000020u, 0x00000010u, 0x00000008u, 0x00000004u, 0x00000002u, 0x00000001u,
    0x80000000u, 0xC0000000u, 0xA0000000u, 0xF0000000u, 0x88000000u, 0xCC000000u, 0xAA000000u, 0xFF000000u,
    0x80800000u, 0xC0C00000u, 0xA0A00000u, 0xF0F00000u, 0x88880000u, 0xCCCC0000u, 0xAAAA0000u, 0xFFFF0000u,
    0x80008000u, 0xC000C000u, 0xA000A000u, 0xF000F000u, 0x88008800u, 0xCC00CC00u, 0xAA00AA00u, 0xFF00FF00u,
    0x80808080u, 0xC0C0C0C0u, 0xA0A0A0A0u, 0xF0F0F0F0u, 0x88888888u, 0xCCCCCCCCu, 0xAAAAAAAAu, 0xFFFFFFFFu,
    0x80000000u, 0x40000000u, 0xE0000000u, 0x50000000u, 0x98000000u, 0xBC000000u, 0xAE000000u, 0x25000000u,
    0x5B800000u, 0x91400000u, 0x65600000u, 0x2E500000u, 0x91180000u, 0x88D40000u, 0xDD360000u, 0x02950000u,
    0x4C888000u, 0x09EB4000u, 0x86CA6000u, 0x13B15000u, 0x42ADD800u, 0x3DF8D400u, 0x2FE57E00u, 0x56EB8100u,
    0x8C41A680u, 0xE68455C0u, 0x3C9CE8E0u, 0xB44DBFF0u, 0x7C27F6C8u, 0x5239A6ACu, 0x853B0EDEu, 0x52EB2EF9u,
    0x80000000u, 0xC0000000u, 0x20000000u, 0x50000000u, 0xF8000000u, 0x74000000u, 0xA2000000u, 0x93000000u,
    0xD8800000u, 0x25400000u, 0x59E00000u, 0xE6D00000u, 0x78080000u, 0xB40C0000u, 0x82020000u, 0xC3050000u,
    0x208F8000u, 0x51CBC000u, 0xFBEA2000u, 0x75AD5000u, 0xA00AF800u, 0x90077400u, 0xD800A200u, 0x25009300u,
    0x59E08480u, 0xE6D0CEC0u, 0x78088520u, 0xB40CEBB0u, 0x82028348u, 0xC305C274u, 0x208FB552u, 0x51CB9AE9u,
};

constexpr uint32_t kSamplerPCG = 0, kSamplerSobol = 1;
constexpr uint32_t kFlagFirefly = 1u << 2;
constexpr uint32_t kFlagEnvFixedV = 1u << 8;
constexpr uint32_t kFlagVndf = 1u << 9;

// ---------------------------------------------------------------------------
// samplers (sampler_pcg.glsl:9-29, sampler_sobol.glsl:13-82)
// ---------------------------------------------------------------------------
OHAO_D uint32_t owen_scramble(uint32_t v, uint32_t seed) {
    v = __brev(v);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    return __brev(v);
}
OHAO_D uint32_t sobol_hash_pixel(uint32_t px, uint32_t py) {
    uint32_t h = (px * 0x1b873593u) ^ (py * 0xcc9e2d51u);
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}
OHAO_D float sobol_sample(uint32_t index, uint32_t seed, uint32_t dim) {
    const uint32_t pad = dim >> 2, local = dim & 3u;
    const uint32_t s = seed ^ (pad * 0x9e3779b9u);
    uint32_t r = 0;
    for (uint32_t bit = 0; index != 0; bit++, index >>= 1)
        if (index & 1u) r ^= c_sobol_dirs[local * 32 + bit];
    const uint32_t v = owen_scramble(r, s);
    return static_cast<float>(v >> 8) * (1.0f / 16777216.0f);
}
OHAO_D uint32_t pcg_next(uint32_t& st) {
    st = st * 747796405u + 2891336453u;
    const uint32_t w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (w >> 22u) ^ w;
}

struct Rng {
    uint32_t type, state, index, seed;
    OHAO_D float s1(uint32_t dim) {
        if (type == kSamplerPCG) return static_cast<float>(pcg_next(state)) / 4294967296.0f;
        return sobol_sample(index, seed, dim);
    }
};
OHAO_D uint32_t pcg_init(uint32_t px, uint32_t py, uint32_t s) { return px * 1973u + py * 9277u + s * 26699u + 1u; }

// ---------------------------------------------------------------------------
// surface / miss shading
// ---------------------------------------------------------------------------
constexpr float kPI = 3.14159265358979f;      // OHAO_PI
constexpr float kTWOPI = 6.28318530717959f;   // OHAO_TWOPI

struct Surf {
    bool hit;
    V3 color, pos, N, albedo;
    float rough, metal, dist, env_pdf;
    uint32_t gtri, matid;
    float tu, tv;
};

// env_sampling.glsl:15-37: the first CDF entry >= u (the last entry if
// none), searched between a guide table's bounds where the scene has one.
OHAO_D int search_marg(const DScene& sc, float u) {
    if (sc.guide_marg)
        return ohao_env_guide::search([&](int i) { return __ldg(sc.marg + i); },
                                      [&](uint32_t j) { return static_cast<int>(__ldg(sc.guide_marg + j)); },
                                      sc.guide_mm, u);
    int lo = 0, hi = static_cast<int>(sc.env_h) - 1;
    while (lo < hi) { int mid = (lo + hi) / 2; if (__ldg(sc.marg + mid) < u) lo = mid + 1; else hi = mid; }
    return lo;
}
OHAO_D int search_cond(const DScene& sc, uint32_t row, uint32_t base, float u) {
    if (sc.guide_cond) {
        const uint16_t* g = sc.guide_cond + static_cast<size_t>(row) * (sc.guide_mc + 1);
        return ohao_env_guide::search([&](int i) { return __ldg(sc.cond + base + i); },
                                      [&](uint32_t j) { return static_cast<int>(__ldg(g + j)); }, sc.guide_mc, u);
    }
    int lo = 0, hi = static_cast<int>(sc.env_w) - 1;
    while (lo < hi) { int mid = (lo + hi) / 2; if (__ldg(sc.cond + base + mid) < u) lo = mid + 1; else hi = mid; }
    return lo;
}
// env_sampling.glsl:52-74
OHAO_D void sample_env(const DScene& sc, float u1, float u2, V3& dir, float& pdf) {
    const uint32_t W = sc.env_w, H = sc.env_h;
    const int y = search_marg(sc, u1);
    const uint32_t base = static_cast<uint32_t>(y) * W;
    const int x = search_cond(sc, static_cast<uint32_t>(y), base, u2);
    const float u = (static_cast<float>(x) + 0.5f) / static_cast<float>(W);
    const float v = (static_cast<float>(y) + 0.5f) / static_cast<float>(H);
    const float phi = (u - 0.5f) * kTWOPI;
    const float theta = v * kPI;
    const float sinT = sin_f(theta);
    dir = v3(sinT * cos_f(phi), cos_f(theta), sinT * sin_f(phi));
    const float theta2 = (static_cast<float>(y) + 0.5f) / static_cast<float>(H) * kPI;
    const float sinT2 = gmaxf(sin_f(theta2), 1e-4f);
    const float condDiff = __ldg(sc.cond + base + x) - (x > 0 ? __ldg(sc.cond + base + x - 1) : 0.0f);
    const float margDiff = __ldg(sc.marg + y) - (y > 0 ? __ldg(sc.marg + y - 1) : 0.0f);
    const float pdfUV = condDiff * margDiff * static_cast<float>(W) * static_cast<float>(H);
    pdf = pdfUV / (kTWOPI * kPI * sinT2);
    pdf = gmaxf(pdf, 0.0f);
}
// env_sampling.glsl:77-94
OHAO_D float pdf_env(const DScene& sc, V3 dir) {
    const uint32_t W = sc.env_w, H = sc.env_h;
    const float theta = acos_f(gclampf(dir.y, -1.0f, 1.0f));
    const float phi = atan2_f(dir.z, dir.x);
    const float u = phi / kTWOPI + 0.5f;
    const float v = theta / kPI;
    int x = static_cast<int>(u * static_cast<float>(W));
    x = x < 0 ? 0 : (x > static_cast<int>(W) - 1 ? static_cast<int>(W) - 1 : x);
    int y = static_cast<int>(v * static_cast<float>(H));
    y = y < 0 ? 0 : (y > static_cast<int>(H) - 1 ? static_cast<int>(H) - 1 : y);
    const uint32_t base = static_cast<uint32_t>(y) * W;
    const float condDiff = __ldg(sc.cond + base + x) - (x > 0 ? __ldg(sc.cond + base + x - 1) : 0.0f);
    const float margDiff = __ldg(sc.marg + y) - (y > 0 ? __ldg(sc.marg + y - 1) : 0.0f);
    const float pdfUV = condDiff * margDiff * static_cast<float>(W) * static_cast<float>(H);
    const float sinT = gmaxf(sin_f(theta), 1e-4f);
    return gmaxf(pdfUV / (kTWOPI * kPI * sinT), 0.0f);
}
OHAO_D int wrapi(int i, int n) { int m = i % n; return m < 0 ? m + n : m; }
// LINEAR/REPEAT texture fetch restated in float (texel centres at (i+0.5)/N)
OHAO_D V3 env_texture(const DScene& sc, float u, float v) {
    const int W = static_cast<int>(sc.env_w), H = static_cast<int>(sc.env_h);
    const float x = u * static_cast<float>(W) - 0.5f;
    const float y = v * static_cast<float>(H) - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float fx = x - fx0, fy = y - fy0;
    const long long ix = static_cast<long long>(fx0), iy = static_cast<long long>(fy0);
    const int x0 = wrapi(static_cast<int>(ix % W), W), x1 = wrapi(static_cast<int>((ix + 1) % W), W);
    const int y0 = wrapi(static_cast<int>(iy % H), H), y1 = wrapi(static_cast<int>((iy + 1) % H), H);
    const V3 t00 = ld3(__ldg(sc.env + static_cast<size_t>(y0) * W + x0));
    const V3 t10 = ld3(__ldg(sc.env + static_cast<size_t>(y0) * W + x1));
    const V3 t01 = ld3(__ldg(sc.env + static_cast<size_t>(y1) * W + x0));
    const V3 t11 = ld3(__ldg(sc.env + static_cast<size_t>(y1) * W + x1));
    const V3 top = t00 * (1.0f - fx) + t10 * fx;
    const V3 bot = t01 * (1.0f - fx) + t11 * fx;
    return top * (1.0f - fy) + bot * fy;
}
// pt_miss.rmiss:52-81
OHAO_D void miss_shade(const DScene& sc, const PathParams& pp, V3 rd, Surf& s) {
    s.hit = false;
    s.dist = -1.0f;
    if (sc.has_env) {
        const V3 dir = normalize(rd);
        const float phi = atan2_f(dir.z, dir.x);
        const float u = phi / 6.2831853f + 0.5f;
        float v;
        if (pp.flags & kFlagEnvFixedV) v = acos_f(gclampf(dir.y, -1.0f, 1.0f)) / 3.1415926f;
        else v = asin_f(gclampf(dir.y, -1.0f, 1.0f)) / 3.1415926f + 0.5f;
        const float envS = (sc.env_intensity > 0.0f) ? sc.env_intensity : 1.0f;
        s.color = env_texture(sc, u, v) * envS;
    } else {
        s.color = v3s(0.0f);
    }
    s.env_pdf = (sc.has_env && sc.has_cdf) ? pdf_env(sc, normalize(rd)) : 0.0f;
}
// diff_map.hpp:40-67
OHAO_D V3 albedo_map_sample(const float* __restrict__ map, uint32_t mw, uint32_t mh, float u, float v) {
    const int w = static_cast<int>(mw), h = static_cast<int>(mh);
    u = gclampf(u, 0.0f, 1.0f);
    v = gclampf(v, 0.0f, 1.0f);
    const float x = u * static_cast<float>(w - 1);
    const float y = v * static_cast<float>(h - 1);
    const int x0 = static_cast<int>(x), y0 = static_cast<int>(y);
    const int x1 = min(x0 + 1, w - 1), y1 = min(y0 + 1, h - 1);
    const float tx = x - static_cast<float>(x0), ty = y - static_cast<float>(y0);
    float out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a = __ldg(map + (static_cast<size_t>(y0) * w + x0) * 3 + c) * (1.0f - tx) +
                        __ldg(map + (static_cast<size_t>(y0) * w + x1) * 3 + c) * tx;
        const float b = __ldg(map + (static_cast<size_t>(y1) * w + x0) * 3 + c) * (1.0f - tx) +
                        __ldg(map + (static_cast<size_t>(y1) * w + x1) * 3 + c) * tx;
        out[c] = a * (1.0f - ty) + b * ty;
    }
    return v3(out[0], out[1], out[2]);
}
// Emission of a surface point: the sRGB-decoded emissive texture
// (pt_closesthit.rchit:150-156) plus the material's slot-2 emission (not the
// reference's). m2 = the material's third float4, etex its emissive texture.
template <bool kTex>
OHAO_D V3 emission_of(const DScene& sc, uint32_t etex, float4 m2, float tu, float tv) {
    V3 emis = v3s(0.0f);
    if (kTex && etex != 0xFFFFFFFFu) {
        const float4 c = tex_sample(sc, etex, tu, tv);
        emis = v3(pow_def(c.x, 2.2f), pow_def(c.y, 2.2f), pow_def(c.z, 2.2f));
    }
    return emis + v3(m2.y, m2.z, m2.w);
}

// pt_closesthit.rchit:37-162
// kTex: bindless textures compiled in (scenes without them keep the shading
// step at its register count; the tile albedo map is read either way).
template <bool kTex = true>
OHAO_D void hit_shade(const DScene& sc, V3 o, V3 d, const Hit& h, Surf& s) {
    s.hit = true;
    const float t = h.t;
    s.pos = o + d * t;
    s.dist = t;
    const DInst& in = sc.inst[h.inst];
    const float u = h.u, v = h.v;
    const float w = 1.0f - u - v;
    const uint32_t gtri = (in.custom & 0xFFFFFFu) + h.prim;
    s.gtri = gtri;
    const uint32_t i0 = __ldg(sc.indices + gtri * 3), i1 = __ldg(sc.indices + gtri * 3 + 1),
                   i2 = __ldg(sc.indices + gtri * 3 + 2);
    const float2 uv0 = __ldg(sc.uvs + i0), uv1 = __ldg(sc.uvs + i1), uv2 = __ldg(sc.uvs + i2);
    s.tu = w * uv0.x + u * uv1.x + v * uv2.x;
    s.tv = w * uv0.y + u * uv1.y + v * uv2.y;
    const V3 n0 = ld3(__ldg(sc.normals + i0)), n1 = ld3(__ldg(sc.normals + i1)), n2 = ld3(__ldg(sc.normals + i2));
    const V3 interp = n0 * w + n1 * u + n2 * v;
    const float* m = in.nrm;
    V3 wn;
    if (dot(interp, interp) > 0.0001f) {
        const V3 x = normalize(interp);
        wn = normalize(v3(m[0] * x.x + m[1] * x.y + m[2] * x.z, m[3] * x.x + m[4] * x.y + m[5] * x.z,
                          m[6] * x.x + m[7] * x.y + m[8] * x.z));
    } else {
        V3 oo, od;
        xform_point(in.w2o, o, oo);
        xform_dir(in.w2o, d, od);
        const V3 hl = oo + od * t;
        const V3 al = v3(fabsf(hl.x), fabsf(hl.y), fabsf(hl.z));
        auto sgn = [](float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); };
        V3 ln;
        if (al.x >= al.y && al.x >= al.z) ln = v3(sgn(hl.x), 0.0f, 0.0f);
        else if (al.y >= al.z) ln = v3(0.0f, sgn(hl.y), 0.0f);
        else ln = v3(0.0f, 0.0f, sgn(hl.z));
        wn = normalize(v3(m[0] * ln.x + m[1] * ln.y + m[2] * ln.z, m[3] * ln.x + m[4] * ln.y + m[5] * ln.z,
                          m[6] * ln.x + m[7] * ln.y + m[8] * ln.z));
        if (dot(wn, d) > 0.0f) wn = -wn;
    }
    const uint32_t mid = __ldg(sc.mat_ids + gtri);
    s.matid = mid;
    const float4 m0 = __ldg(sc.mats + mid * 3), m1 = __ldg(sc.mats + mid * 3 + 1), m2 = __ldg(sc.mats + mid * 3 + 2);
    const uint32_t dtex = __float_as_uint(m0.w), ntex = __float_as_uint(m1.z), etex = __float_as_uint(m1.w),
                   rmtex = __float_as_uint(m2.x);
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    // albedo: base colour times the sRGB-decoded diffuse texture
    // (pt_closesthit.rchit:108-113); diffuse index 0 is the tile albedo map
    // when one is set (linear, diff_map.hpp:40-67)
    V3 alb = v3(m0.x, m0.y, m0.z);
    if (dtex != kNone) {
        if (dtex == 0u && sc.map_w > 0) {
            alb = alb * albedo_map_sample(sc.albedo_map, sc.map_w, sc.map_h, s.tu, s.tv);
        } else if (kTex) {
            const float4 c = tex_sample(sc, dtex, s.tu, s.tv);
            alb = alb * v3(pow_def(c.x, 2.2f), pow_def(c.y, 2.2f), pow_def(c.z, 2.2f));
        }
    }
    // tangent-space normal map in the Frisvad basis of the shading normal
    // (pt_closesthit.rchit:116-133)
    if (kTex && ntex != kNone) {
        const float4 c = tex_sample(sc, ntex, s.tu, s.tv);
        const V3 mapN = normalize(v3(c.x * 2.0f - 1.0f, c.y * 2.0f - 1.0f, c.z * 2.0f - 1.0f));
        V3 T, B;
        if (wn.z < -0.9999f) {
            T = v3(0.0f, -1.0f, 0.0f);
            B = v3(-1.0f, 0.0f, 0.0f);
        } else {
            const float a = 1.0f / (1.0f + wn.z);
            const float d = -wn.x * wn.y * a;
            T = v3(1.0f - wn.x * wn.x * a, d, -wn.x);
            B = v3(d, 1.0f - wn.y * wn.y * a, -wn.y);
        }
        wn = normalize(T * mapN.x + B * mapN.y + wn * mapN.z);
    }
    s.N = wn;
    s.albedo = alb;
    // roughness / metallic factors from the ORM texture's G and B
    // (pt_closesthit.rchit:139-148)
    float rough = m1.x, metal = m1.y;
    if (kTex && rmtex != kNone) {
        const float4 c = tex_sample(sc, rmtex, s.tu, s.tv);
        rough = rough * c.y;
        metal = metal * c.z;
    }
    rough = gmaxf(rough, 0.04f);
    s.color = emission_of<kTex>(sc, etex, m2, s.tu, s.tv);
    // payload.attenuation = (rough, clamp(metal,0,1), curv) -> unpackHitPbr
    const float ax = rough, ay = gclampf(metal, 0.0f, 1.0f);
    float rr, mm;
    if (ax < 0.0f && ay < 1e-4f) {
        rr = -ax; if (rr >= 10.0f) rr = rr - 10.0f; rr = gmaxf(rr, 0.01f); mm = 1.0f;
    } else {
        rr = fabsf(ax); if (rr >= 10.0f) rr = rr - 10.0f; rr = gmaxf(rr, 0.01f); mm = gclampf(ay, 0.0f, 1.0f);
    }
    s.rough = rr;
    s.metal = mm;
}

// ---------------------------------------------------------------------------
// BSDF helpers
// ---------------------------------------------------------------------------
// pt_raygen.rgen:90-97
OHAO_D V3 cos_hemi(V3 N, float u0, float u1) {
    const V3 up = fabsf(N.y) < 0.999f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    const V3 T = normalize(cross(up, N));
    const V3 B = cross(N, T);
    const float r = sqrtf(u0);
    const float phi = 6.2831853f * u1;
    float sp, cp;
    sincos_f(phi, &sp, &cp);
    return normalize(T * r * cp + B * r * sp + N * sqrtf(gmaxf(0.0f, 1.0f - r * r)));
}
// GGX visible-normal sampling and its Smith terms (ggx_aniso.glsl:56-133,
// Heitz 2018), alpha = roughness^2; inversesqrt as 1 / sqrt.
OHAO_D float ggx_d_iso(float NdotH, float alpha) {
    const float a2 = alpha * alpha;
    const float denom = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
    return a2 / (3.14159265f * denom * denom + 1e-8f);
}
OHAO_D float smith_lambda(float c, float alpha) {
    const float c2 = c * c;
    const float tan2 = gmaxf(0.0f, 1.0f - c2) / gmaxf(c2, 1e-8f);
    return 0.5f * (-1.0f + sqrtf(1.0f + alpha * alpha * tan2));
}
OHAO_D float smith_g1(float c, float alpha) { return 1.0f / (1.0f + smith_lambda(c, alpha)); }
OHAO_D float smith_g2_over_g1(float NdotV, float NdotL, float alpha) {
    const float lv = smith_lambda(NdotV, alpha), ll = smith_lambda(NdotL, alpha);
    return (1.0f + lv) / (1.0f + lv + ll + 1e-8f);
}
OHAO_D V3 sample_vndf(V3 Ve, float ax, float ay, float u0, float u1) {
    const V3 Vh = normalize(v3(ax * Ve.x, ay * Ve.y, Ve.z));
    const float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    const V3 T1 = lensq > 0.0f ? v3(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : v3(1.0f, 0.0f, 0.0f);
    const V3 T2 = cross(Vh, T1);
    const float r = sqrtf(u0);
    const float phi = 2.0f * 3.14159265f * u1;
    float sp, cp;
    sincos_f(phi, &sp, &cp);
    const float t1 = r * cp;
    float t2 = r * sp;
    const float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * sqrtf(gmaxf(0.0f, 1.0f - t1 * t1)) + s * t2;
    const V3 Nh = T1 * t1 + T2 * t2 + Vh * sqrtf(gmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
    return normalize(v3(ax * Nh.x, ay * Nh.y, gmaxf(0.0f, Nh.z)));
}

// ggx_aniso.glsl:31-55
OHAO_D float ggxD(const PathParams& pp, V3 N, V3 H, float NdotH, float rough) {
    const float an = pp.aniso;
    if (an < 0.001f) {
        const float a = rough * rough, a2 = a * a;
        const float denom = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
        return a2 / (3.14159265f * denom * denom + 0.0001f);
    }
    const V3 up = v3(0.0f, 1.0f, 0.0f);
    const V3 ref = fabsf(dot(up, N)) > 0.97f ? v3(1.0f, 0.0f, 0.0f) : up;
    const V3 T = normalize(ref - N * dot(ref, N));
    const V3 B = cross(N, T);
    float s, c;
    sincos_f(pp.aniso_rot, &s, &c);
    const V3 Tr = T * c + B * s;
    const V3 Br = B * c - T * s;
    const float r2 = rough * rough;
    const float aspect = sqrtf(1.0f - an * 0.9f);
    const float rT = gmaxf(r2 / aspect, 0.001f);
    const float rB = gmaxf(r2 * aspect, 0.001f);
    const float TdotH = dot(Tr, H), BdotH = dot(Br, H);
    const float dd = (TdotH * TdotH / rT) + (BdotH * BdotH / rB) + NdotH * NdotH;
    return 1.0f / (3.14159265f * rT * rB * dd * dd + 0.0001f);
}
OHAO_D float mis_balance(float a, float b) { return a / gmaxf(a + b, 1e-6f); }   // mis.glsl:7-9

OHAO_D V3 firefly(const PathParams& pp, V3 c) {
    if ((pp.flags & kFlagFirefly) && pp.clamp_lum > 0.0f) {
        const float l = lum(c);
        if (l > pp.clamp_lum) c = c * (pp.clamp_lum / l);
    }
    return c;
}

// A pending shadow query: visible => radiance += contrib.
struct ShadowReq {
    V3 org;
    V3 dir;
    float tmax;
    V3 contrib;
    bool valid;
};

// Light choice and sample point of a light NEE (the draws and geometry of
// pt_raygen.rgen:305-383), shared by the forward step and the adjoint.
// mis_pdf: the solid-angle pdf of the sample when the emitter can also be
// reached by a BSDF ray (emitter MIS: emissive triangles, sphere and area
// lights), else 0.
struct LightSample {
    bool valid;       // NdotL > 0 && weight > 0
    V3 L, Le;
    float weight, shadowDist, NdotL, n, mis_pdf;
};

// Number of choices of the light NEE: the analytic lights, plus the emissive
// triangles as one more choice under emitter MIS.
template <bool kMis>
OHAO_D uint32_t light_choices(const DScene& sc) {
    return sc.nlights + ((kMis && sc.nemis != 0u) ? 1u : 0u);
}

// First entry of the emissive-triangle CDF above u (the last when none is).
OHAO_D uint32_t emis_search(const DScene& sc, float u) {
    uint32_t lo = 0, hi = sc.nemis - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(sc.emis_cdf + mid) <= u) lo = mid + 1u;
        else hi = mid;
    }
    return lo;
}

// Emission of triangle prim of instance inst at barycentrics (u, v): the
// value hit_shade gives a ray that hits that point.
template <bool kTex>
OHAO_D V3 emission_at(const DScene& sc, uint32_t inst, uint32_t prim, float u, float v) {
    const uint32_t gtri = (sc.inst[inst].custom & 0xFFFFFFu) + prim;
    const uint32_t mid = __ldg(sc.mat_ids + gtri);
    const float4 m1 = __ldg(sc.mats + mid * 3 + 1), m2 = __ldg(sc.mats + mid * 3 + 2);
    const uint32_t etex = __float_as_uint(m1.w);
    float tu = 0.0f, tv = 0.0f;
    if (kTex && etex != 0xFFFFFFFFu) {
        const float w = 1.0f - u - v;
        const uint32_t i0 = __ldg(sc.indices + gtri * 3), i1 = __ldg(sc.indices + gtri * 3 + 1),
                       i2 = __ldg(sc.indices + gtri * 3 + 2);
        const float2 uv0 = __ldg(sc.uvs + i0), uv1 = __ldg(sc.uvs + i1), uv2 = __ldg(sc.uvs + i2);
        tu = w * uv0.x + u * uv1.x + v * uv2.x;
        tv = w * uv0.y + u * uv1.y + v * uv2.y;
    }
    return emission_of<kTex>(sc, etex, m2, tu, tv);
}

template <bool kTex = true, bool kMis = false>
OHAO_D LightSample sample_light(const DScene& sc, Rng& rng, uint32_t& dim, V3 P, V3 N) {
    LightSample out;
    out.mis_pdf = 0.0f;
    const uint32_t n = light_choices<kMis>(sc);
    const float usel = rng.s1(dim);
    uint32_t li = static_cast<uint32_t>(usel * static_cast<float>(n));
    dim += 1;
    li = min(li, n - 1u);
    V3 L, Le;
    float shadowDist, weight;
    if (kMis && li == sc.nlights) {
        // an emissive triangle, chosen by power with what is left of the
        // choice's draw, at a uniform point (barycentrics sqrt(a0)(1 - a1),
        // sqrt(a0) a1); both faces emit
        const uint32_t e = emis_search(sc, usel * static_cast<float>(n) - static_cast<float>(sc.nlights));
        const float4 A = __ldg(sc.emis_tri + 3 * e), B = __ldg(sc.emis_tri + 3 * e + 1),
                     C = __ldg(sc.emis_tri + 3 * e + 2);
        const float a0 = rng.s1(dim), a1 = rng.s1(dim + 1);
        dim += 2;
        const float su = sqrtf(a0);
        const float b1 = su * (1.0f - a1), b2 = su * a1;
        const V3 e1 = v3(B.x, B.y, B.z), e2 = v3(C.x, C.y, C.z);
        const V3 lp = v3(A.x, A.y, A.z) + e1 * b1 + e2 * b2;
        const V3 ng = normalize(cross(e1, e2));
        const V3 tl = lp - P;
        const float ld = length(tl);
        L = tl / ld;
        const float lcos = fabsf(dot(L, ng));
        Le = emission_at<kTex>(sc, __float_as_uint(B.w), __float_as_uint(C.w), b1, b2);
        weight = lcos / (A.w * (ld * ld));
        shadowDist = ld - 0.02f;
        out.mis_pdf = A.w * (ld * ld) / (lcos * static_cast<float>(n));
    } else {
        const float4 L0 = __ldg(sc.lights + li * 5), L1 = __ldg(sc.lights + li * 5 + 1),
                     L2 = __ldg(sc.lights + li * 5 + 2), L3 = __ldg(sc.lights + li * 5 + 3),
                     L4 = __ldg(sc.lights + li * 5 + 4);
        const float ltype = L0.w;
        const V3 lc = v3(L0.x, L0.y, L0.z);
        const V3 lcol = v3(L1.x, L1.y, L1.z);
        const float lint = L1.w;
        const float lrad = L2.w;
        const V3 ldir = normalize(v3(L2.x, L2.y, L2.z));
        const float outerAngle = L3.w;
        const float r = gmaxf(lrad, 0.01f);
        const float area = 4.0f * 3.14159f * r * r;
        Le = lcol * lint / gmaxf(area, 0.01f);
        if (ltype < 0.5f) {
            const float u1 = rng.s1(dim), u2 = rng.s1(dim + 1);
            dim += 2;
            const float cosT = 1.0f - 2.0f * u1;
            const float sinT = sqrtf(gmaxf(0.0f, 1.0f - cosT * cosT));
            const float phi = 6.2831853f * u2;
            float sp, cp;
            sincos_f(phi, &sp, &cp);
            const V3 off = v3(sinT * cp, sinT * sp, cosT) * r;
            const V3 lp = lc + off;
            const V3 ln = normalize(off);
            const V3 tl = lp - P;
            const float ld = length(tl);
            L = tl / ld;
            const float lcos = gmaxf(dot(-L, ln), 0.0f);
            const float la = 4.0f * 3.14159f * r * r;
            weight = lcos * la / (ld * ld);
            shadowDist = ld - 0.02f;
            if (kMis) out.mis_pdf = (ld * ld) / (lcos * la * static_cast<float>(n));
        } else if (ltype < 1.5f) {
            L = -ldir;
            weight = 1.0f;
            shadowDist = 10000.0f;
        } else if (ltype < 2.5f) {
            const float u1 = rng.s1(dim), u2 = rng.s1(dim + 1);
            dim += 2;
            const float cosT = 1.0f - 2.0f * u1;
            const float sinT = sqrtf(gmaxf(0.0f, 1.0f - cosT * cosT));
            const float phi = 6.2831853f * u2;
            float sp, cp;
            sincos_f(phi, &sp, &cp);
            const V3 off = v3(sinT * cp, sinT * sp, cosT) * r;
            const V3 lp = lc + off;
            const V3 tl = lp - P;
            const float ld = length(tl);
            L = tl / ld;
            shadowDist = ld - 0.02f;
            const float cosA = dot(-L, ldir);
            const float innerCos = cos_f(lrad * 0.017453292f);
            const float outerCos = cos_f(outerAngle * 0.017453292f);
            float spot = gclampf((cosA - outerCos) / (innerCos - outerCos + 0.001f), 0.0f, 1.0f);
            spot = spot * spot;
            const float la = 4.0f * 3.14159f * r * r;
            weight = la / (ld * ld) * spot;
        } else {
            const V3 e1 = v3(L3.x, L3.y, L3.z);
            const V3 e2 = v3(L4.x, L4.y, L4.z);
            const float ar = L4.w;
            const float a0 = rng.s1(dim), a1 = rng.s1(dim + 1);
            dim += 2;
            const V3 lp = lc + e1 * a0 + e2 * a1;
            const V3 ln = normalize(cross(e1, e2));
            const V3 tl = lp - P;
            const float ld = length(tl);
            L = tl / ld;
            const float lcos = gmaxf(dot(-L, ln), 0.0f);
            weight = lcos * ar / (ld * ld);
            shadowDist = ld - 0.02f;
            if (kMis) out.mis_pdf = (ld * ld) / (lcos * ar * static_cast<float>(n));
        }
    }
    out.NdotL = gmaxf(dot(N, L), 0.0f);
    out.valid = out.NdotL > 0.0f && weight > 0.0f;
    out.L = L;
    out.Le = Le;
    out.weight = weight;
    out.shadowDist = shadowDist;
    out.n = static_cast<float>(n);
    return out;
}

// The BSDF pdf the estimator gives direction L at a surface (the one its env
// MIS uses, pt_raygen.rgen:466-479): the diffuse and GGX lobes mixed by the
// specular choice probability.
OHAO_D float bsdf_pdf(V3 inDir, V3 N, V3 F0, float rough, float metal, float NdotL, float NdotH, float VdotH,
                      float D) {
    const float cosI = fabsf(dot(normalize(inDir), N));
    const V3 fres = F0 + (1.0f - F0) * pow5f(1.0f - cosI);
    float sp = maxc(fres) * (1.0f - rough * 0.9f);
    sp = gmixf(sp, 1.0f, metal);
    const float pdfD = NdotL / kPI;
    const float pdfS = D * NdotH / (4.0f * VdotH + 1e-4f);
    return gmixf(pdfD, pdfS, sp);
}

// Analytic light NEE; contribution precomputed as if visible. thr == null at
// bounce 0 (pt_raygen.rgen:305-434; 585-705; 893-1013). Under emitter MIS a
// sample of an emitter that BSDF rays can reach is weighted by the balance
// heuristic against bsdf_pdf.
template <bool kTex = true, bool kMis = false>
OHAO_D void nee_light(const DScene& sc, const PathParams& pp, Rng& rng, uint32_t& dim, V3 P, V3 N, V3 inDir, V3 albedo,
                      float rough, float metal, V3 F0, const V3* thr, ShadowReq& req) {
    req.valid = false;
    const LightSample ls = sample_light<kTex, kMis>(sc, rng, dim, P, N);
    if (!ls.valid) return;
    const V3 L = ls.L, Le = ls.Le;
    const float NdotL = ls.NdotL, weight = ls.weight, shadowDist = ls.shadowDist;
    const float n = ls.n;
    const V3 V = normalize(-inDir);
    const V3 H = normalize(L + V);
    const float NdotH = gmaxf(dot(N, H), 0.001f);
    const float NdotV = gmaxf(dot(N, V), 0.001f);
    const float VdotH = gmaxf(dot(V, H), 0.001f);
    float D;
    if (thr == nullptr) {
        D = ggxD(pp, N, H, NdotH, rough);
    } else {
        const float a = rough * rough, a2 = a * a;
        const float denom = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
        D = a2 / (3.14159f * denom * denom + 0.0001f);
    }
    const V3 F = F0 + (1.0f - F0) * pow5f(1.0f - VdotH);
    const float k = (rough + 1.0f) * (rough + 1.0f) / 8.0f;
    const float G = (NdotL / (NdotL * (1.0f - k) + k)) * (NdotV / (NdotV * (1.0f - k) + k));
    const V3 spec = D * F * G / (4.0f * NdotV * NdotL + 0.001f);
    const V3 kD = (1.0f - F) * (1.0f - metal);
    const V3 diff = kD * albedo / 3.14159f;
    V3 c;
    if (thr == nullptr) c = Le * (diff + spec) * NdotL * weight * n;
    else c = *thr * Le * (diff + spec) * NdotL * weight * n;
    if (kMis && ls.mis_pdf > 0.0f)
        c = c * mis_balance(ls.mis_pdf, bsdf_pdf(inDir, N, F0, rough, metal, NdotL, NdotH, VdotH, D));
    req.valid = true;
    req.org = P + N * 0.01f;
    req.dir = L;
    req.tmax = shadowDist;
    req.contrib = firefly(pp, c);
}

// Emitter MIS, BSDF side: the sphere and area lights that the ray (ro, rd)
// crosses before tmax (lights stay transparent to it, as to every ray of the
// reference, so each one crossed counts), each seen from its emitting side
// and weighted against its light-NEE pdf (weight 1 after a delta bounce).
OHAO_D V3 light_hits(const DScene& sc, V3 ro, V3 rd, float tmax, bool delta, float last_pdf, float n) {
    V3 sum = v3s(0.0f);
    for (uint32_t li = 0; li < sc.nlights; ++li) {
        const float4 L0 = __ldg(sc.lights + li * 5);
        const float ltype = L0.w;
        if (ltype >= 0.5f && ltype < 2.5f) continue;   // directional and spot lights cannot be hit
        const float4 L1 = __ldg(sc.lights + li * 5 + 1), L2 = __ldg(sc.lights + li * 5 + 2);
        const V3 lc = v3(L0.x, L0.y, L0.z);
        const float r = gmaxf(L2.w, 0.01f);
        const float area = 4.0f * 3.14159f * r * r;
        const V3 Le = v3(L1.x, L1.y, L1.z) * L1.w / gmaxf(area, 0.01f);
        float t, lcos, la;
        if (ltype < 0.5f) {
            const V3 oc = ro - lc;
            const float b = dot(oc, rd);
            const float c = dot(oc, oc) - r * r;
            const float disc = b * b - c;
            if (!(disc >= 0.0f)) continue;
            t = -b - sqrtf(disc);
            if (!(t > 0.001f && t < tmax)) continue;
            const V3 ln = normalize(ro + rd * t - lc);
            lcos = dot(-rd, ln);
            la = 4.0f * 3.14159f * r * r;
        } else {
            const float4 L3 = __ldg(sc.lights + li * 5 + 3), L4 = __ldg(sc.lights + li * 5 + 4);
            const V3 e1 = v3(L3.x, L3.y, L3.z), e2 = v3(L4.x, L4.y, L4.z);
            const V3 nn = cross(e1, e2);
            const V3 ln = normalize(nn);
            lcos = dot(-rd, ln);
            if (!(lcos > 0.0f)) continue;
            t = dot(lc - ro, ln) / -lcos;
            if (!(t > 0.001f && t < tmax)) continue;
            const V3 rel = ro + rd * t - lc;
            const float inv = 1.0f / dot(nn, nn);
            const float a = dot(cross(rel, e2), nn) * inv;
            const float b = dot(cross(e1, rel), nn) * inv;
            if (!(a >= 0.0f && a <= 1.0f && b >= 0.0f && b <= 1.0f)) continue;
            la = L4.w;
        }
        if (!(lcos > 0.0f)) continue;
        float w = 1.0f;
        if (!delta) w = mis_balance(last_pdf, (t * t) / (lcos * la * n));
        sum = sum + Le * w;
    }
    return sum;
}

// Emitter MIS, BSDF side: the light-NEE pdf of a ray (direction rd) that hit
// global triangle gtri of instance inst at distance t, or 0 when that
// triangle is not in the emissive table.
OHAO_D float emis_pdf_at(const DScene& sc, uint32_t inst, uint32_t gtri, V3 rd, float t, float n) {
    const uint32_t r = __ldg(sc.emis_rank + gtri);
    if (!(r & 0x80000000u)) return 0.0f;
    const uint2 ib = __ldg(sc.emis_inst + inst);
    if (ib.x == 0xFFFFFFFFu) return 0.0f;
    const uint32_t e = ib.x + (r & 0x7FFFFFFFu) - ib.y;
    const float4 A = __ldg(sc.emis_tri + 3 * e), B = __ldg(sc.emis_tri + 3 * e + 1), C = __ldg(sc.emis_tri + 3 * e + 2);
    if (!(A.w > 0.0f)) return 0.0f;
    const V3 ng = normalize(cross(v3(B.x, B.y, B.z), v3(C.x, C.y, C.z)));
    const float lcos = fabsf(dot(rd, ng));
    return A.w * (t * t) / (lcos * n);
}

// Env NEE sample (pt_raygen.rgen:439-451): direction, pdf, and the radiance
// the miss shader returns for it.
struct EnvSample {
    bool valid;       // NdotL > 0 && pdf > 0
    V3 dir, rad;
    float pdf, NdotL;
};

OHAO_D EnvSample sample_env_nee(const DScene& sc, const PathParams& pp, Rng& rng, uint32_t& dim, V3 N) {
    EnvSample out;
    const float u1 = rng.s1(dim), u2 = rng.s1(dim + 1);
    dim += 2;
    sample_env(sc, u1, u2, out.dir, out.pdf);
    out.NdotL = gmaxf(dot(N, out.dir), 0.0f);
    out.valid = out.NdotL > 0.0f && out.pdf > 0.0f;
    if (out.valid) {
        Surf ms;
        miss_shade(sc, pp, out.dir, ms);
        out.rad = ms.color;
    }
    return out;
}

// Env NEE with balance MIS (pt_raygen.rgen:438-500, 708-763, 1016-1071).
OHAO_D void nee_env(const DScene& sc, const PathParams& pp, Rng& rng, uint32_t& dim, V3 P, V3 N, V3 inDir, V3 albedo,
                    float rough, float metal, V3 F0, const V3* thr, ShadowReq& req) {
    req.valid = false;
    const EnvSample es = sample_env_nee(sc, pp, rng, dim, N);
    if (!es.valid) return;
    const V3 envDir = es.dir;
    const float envPdf = es.pdf, NdotL = es.NdotL;
    const V3 envRad = es.rad;
    const V3 V = normalize(-inDir);
    const V3 H = normalize(envDir + V);
    const float NdotH = gmaxf(dot(N, H), 0.001f);
    const float NdotV = gmaxf(dot(N, V), 0.001f);
    const float VdotH = gmaxf(dot(V, H), 0.001f);
    float D;
    if (thr == nullptr) {
        D = ggxD(pp, N, H, NdotH, rough);
    } else {
        const float a = rough * rough, a2 = a * a;
        const float denom = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
        D = a2 / (kPI * denom * denom + 0.0001f);
    }
    const V3 F = F0 + (1.0f - F0) * pow5f(1.0f - VdotH);
    const float k = (rough + 1.0f) * (rough + 1.0f) / 8.0f;
    const float G = (NdotL / (NdotL * (1.0f - k) + k)) * (NdotV / (NdotV * (1.0f - k) + k));
    const V3 spec = D * F * G / (4.0f * NdotV * NdotL + 0.001f);
    const V3 kD = (1.0f - F) * (1.0f - metal);
    const V3 diff = kD * albedo / kPI;
    const V3 brdf = diff + spec;
    const float cosI = fabsf(dot(normalize(inDir), N));
    const V3 fres = F0 + (1.0f - F0) * pow5f(1.0f - cosI);
    float sp = maxc(fres) * (1.0f - rough * 0.9f);
    sp = gmixf(sp, 1.0f, metal);
    const float pdfD = NdotL / kPI;
    const float pdfS = D * NdotH / (4.0f * VdotH + 1e-4f);
    const float bsdfPdf = gmixf(pdfD, pdfS, sp);
    const float w = mis_balance(envPdf, bsdfPdf);
    V3 c;
    if (thr == nullptr) c = envRad * brdf * NdotL * w / envPdf;
    else c = *thr * envRad * brdf * NdotL * w / envPdf;
    req.valid = true;
    req.org = P + N * 0.01f;
    req.dir = envDir;
    req.tmax = 10000.0f;
    req.contrib = firefly(pp, c);
}

// Specular jitter lobe (pt_raygen.rgen:516-525, 784-793).
OHAO_D V3 spec_dir(Rng& rng, uint32_t& dim, V3 inDir, V3 N, float rough) {
    V3 refl = reflect(inDir, N);
    if (rough > 0.01f) {
        const float j0 = rng.s1(dim), j1 = rng.s1(dim + 1);
        dim += 2;
        const V3 jit = cos_hemi(refl, j0, j1) * rough;
        refl = normalize(refl + jit);
        if (dot(refl, N) < 0.0f) {
            const float f0 = rng.s1(dim), f1 = rng.s1(dim + 1);
            dim += 2;
            refl = cos_hemi(N, f0, f1);
        }
    }
    return refl;
}

// ---------------------------------------------------------------------------
// path state and the per-bounce step
// ---------------------------------------------------------------------------
struct PathState {
    uint32_t rng, dim;
    uint32_t phase, bounce;
    bool delta;
    V3 ro, rd;
    float last_pdf;
    V3 thr, rad;
    V3 fhP, fhN, fhAlb;
};

constexpr uint32_t kPhasePrimary = 0, kPhaseSpec = 1, kPhaseDiff = 2, kPhaseDone = 3;

OHAO_D Rng make_rng(const PathParams& pp, uint32_t px, uint32_t py, uint32_t sidx, uint32_t state) {
    Rng r;
    r.type = pp.sampler;
    r.state = state;
    r.index = sidx;
    r.seed = (pp.sampler == kSamplerSobol) ? sobol_hash_pixel(px, py) : 0u;
    return r;
}

// Camera ray for (px, py, sample) and initial state (pt_raygen.rgen:138-163).
OHAO_D void path_start(const ViewParams& vw, const PathParams& pp, uint32_t px, uint32_t py, uint32_t sidx,
                       PathState& ps) {
    Rng rng = make_rng(pp, px, py, sidx, pcg_init(px, py, sidx));
    uint32_t dim = 0;
    const float jx = rng.s1(dim) - 0.5f, jy = rng.s1(dim + 1) - 0.5f;
    dim += 2;
    const float uvx = (static_cast<float>(px) + 0.5f + jx + 0.0f) / static_cast<float>(vw.width);
    const float uvy = (static_cast<float>(py) + 0.5f + jy + 0.0f) / static_cast<float>(vw.height);
    const float ndcx = uvx * 2.0f - 1.0f, ndcy = uvy * 2.0f - 1.0f;
    const float* iv = vw.inv_view;
    const V3 camPos = v3(iv[12], iv[13], iv[14]);
    const V3 fwd = -v3(iv[8], iv[9], iv[10]);
    const V3 right = v3(iv[0], iv[1], iv[2]);
    const V3 up = v3(iv[4], iv[5], iv[6]);
    const float aspect = static_cast<float>(vw.width) / static_cast<float>(vw.height);
    const float tanY = fabsf(vw.inv_proj[5]);
    const float tanX = tanY * aspect;
    ps.rd = normalize(fwd + right * ndcx * tanX - up * ndcy * tanY);
    ps.ro = camPos;
    ps.rng = rng.state;
    ps.dim = dim;
    ps.phase = kPhasePrimary;
    ps.bounce = 0;
    ps.delta = false;
    ps.last_pdf = 0.0f;
    ps.thr = v3s(1.0f);
    ps.rad = v3s(0.0f);
    ps.fhP = ps.fhN = ps.fhAlb = v3s(0.0f);
}

struct AovOut {
    V3 albedo, normal;
    float depth, hit, rough, metal;
};

// First-hit features of a camera ray's surface (or of its miss).
OHAO_D void aov_of(const Surf& s, const ViewParams& vw, AovOut& ao) {
    if (s.hit) {
        ao.albedo = s.albedo;
        ao.normal = s.N * 0.5f + v3s(0.5f);
        // view-space depth: -(inverse(invView) * pos).z for a rigid invView
        const float* iv = vw.inv_view;
        const V3 c = v3(iv[12], iv[13], iv[14]);
        const V3 fz = v3(iv[8], iv[9], iv[10]);
        ao.depth = dot(s.pos - c, fz) * -1.0f;
        ao.hit = 1.0f;
        ao.rough = s.rough;
        ao.metal = s.metal;
    } else {
        ao.albedo = s.color;
        ao.normal = v3s(0.0f);
        ao.depth = 1e30f;
        ao.hit = 0.0f;
        ao.rough = 0.0f;
        ao.metal = 0.0f;
    }
}

// Starts the diffuse chain from the stored first hit (pt_raygen.rgen:836-853).
OHAO_D void start_diffuse_chain(const PathParams& pp, Rng& rng, uint32_t& dim, PathState& ps) {
    const float d0 = rng.s1(dim), d1 = rng.s1(dim + 1);
    dim += 2;
    const V3 dd = cos_hemi(ps.fhN, d0, d1);
    ps.thr = ps.fhAlb;
    ps.last_pdf = gmaxf(dot(dd, ps.fhN), 0.0f) / kPI;
    ps.delta = false;
    ps.ro = ps.fhP + ps.fhN * 0.01f;
    ps.rd = dd;
    ps.phase = kPhaseDiff;
    ps.bounce = 1;
    if (pp.max_bounces == 0) ps.phase = kPhaseDone;
}

// One step: consume the closest-hit result of the path's current ray, add
// the radiance terms the shader adds here, emit up to two shadow queries and
// set up the next ray (or finish). Returns true when a next ray is pending.
// kMis: emitter MIS (OHAO_PT_FLAG_EMITTER_MIS) compiled in. kPhase: 0 any
// path, 1 only paths at their camera ray, 2 only paths in a chain (a caller
// that knows its queue holds one kind compiles the other branch out).
template <bool kTex = true, bool kMis = false, int kPhase = 0>
OHAO_D bool path_step(const DScene& sc, const PathParams& pp, const ViewParams& vw, uint32_t px, uint32_t py,
                      uint32_t sidx, PathState& ps, const Hit& h, ShadowReq& qL, ShadowReq& qE, AovOut* aov) {
    qL.valid = false;
    qE.valid = false;
    Rng rng = make_rng(pp, px, py, sidx, ps.rng);
    uint32_t dim = ps.dim;
    Surf s;
    if (h.prim != 0xFFFFFFFFu) hit_shade<kTex>(sc, ps.ro, ps.rd, h, s);
    else miss_shade(sc, pp, ps.rd, s);

    if (kPhase == 1 || (kPhase == 0 && ps.phase == kPhasePrimary)) {
        if (aov) aov_of(s, vw, *aov);
        if (!s.hit) {
            ps.rad = s.color;
            ps.phase = kPhaseDone;
            ps.rng = rng.state;
            ps.dim = dim;
            return false;
        }
        const V3 P = s.pos, N = s.N, alb = s.albedo, em = s.color;
        const float rough = s.rough, metal = s.metal;
        const V3 F0 = vmix(v3s(0.04f), alb, metal);
        if (length(em) > 0.001f) ps.rad = ps.rad + em;
        if (light_choices<kMis>(sc) > 0)
            nee_light<kTex, kMis>(sc, pp, rng, dim, P, N, ps.rd, alb, rough, metal, F0, nullptr, qL);
        if (sc.has_cdf) nee_env(sc, pp, rng, dim, P, N, ps.rd, alb, rough, metal, F0, nullptr, qE);
        // stage B init (505-543)
        const V3 inDir = ps.rd;
        V3 sd;
        if (pp.flags & kFlagVndf) {
            // VNDF mode (pt_raygen_realtime.rgen:723-800)
            const V3 V = normalize(-inDir);
            const float NdotV = gmaxf(dot(N, V), 1e-4f);
            const float alpha = rough * rough;
            if (rough < 0.02f) {
                sd = reflect(inDir, N);
                ps.thr = F0 + (1.0f - F0) * pow5f(1.0f - NdotV);
                ps.last_pdf = 1.0f;
                ps.delta = true;
            } else {
                const V3 up = fabsf(N.y) < 0.999f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
                const V3 T = normalize(cross(up, N));
                const V3 B = cross(N, T);
                const V3 Vloc = v3(dot(V, T), dot(V, B), dot(V, N));
                const float u0 = rng.s1(dim), u1 = rng.s1(dim + 1);
                dim += 2;
                const V3 Hloc = sample_vndf(Vloc, alpha, alpha, u0, u1);
                V3 H = normalize(T * Hloc.x + B * Hloc.y + N * Hloc.z);
                V3 refl = reflect(-V, H);
                if (dot(refl, N) <= 0.0f) {
                    refl = reflect(inDir, N);
                    H = N;
                }
                refl = normalize(refl);
                sd = refl;
                const float NdotL = gmaxf(dot(N, refl), 1e-4f);
                const float NdotH = gmaxf(dot(N, H), 1e-4f);
                const float VdotH = gmaxf(dot(V, H), 1e-4f);
                const V3 F = F0 + (1.0f - F0) * pow5f(1.0f - VdotH);
                ps.thr = F * smith_g2_over_g1(NdotV, NdotL, alpha);
                const float D = ggx_d_iso(NdotH, alpha);
                const float G1V = smith_g1(NdotV, alpha);
                ps.last_pdf = G1V * D / (4.0f * NdotV) + 1e-6f;
                ps.delta = false;
            }
        } else {
            sd = spec_dir(rng, dim, inDir, N, rough);
            ps.thr = vmix(v3s(1.0f), alb, metal);
            if (rough < 0.05f) {
                ps.last_pdf = 1.0f;
                ps.delta = true;
            } else {
                const V3 Hs = normalize(-inDir + sd);
                const float NdotHs = gmaxf(dot(N, Hs), 0.001f);
                const float VdotHs = gmaxf(dot(-inDir, Hs), 0.001f);
                const float Ds = ggxD(pp, N, Hs, NdotHs, rough);
                ps.last_pdf = Ds * NdotHs / (4.0f * VdotHs + 1e-4f);
                ps.delta = false;
            }
        }
        ps.fhP = P;
        ps.fhN = N;
        ps.fhAlb = alb;
        ps.ro = P + N * 0.01f;
        ps.rd = sd;
        ps.phase = kPhaseSpec;
        ps.bounce = 1;
        if (pp.max_bounces == 0) start_diffuse_chain(pp, rng, dim, ps);
        ps.rng = rng.state;
        ps.dim = dim;
        return ps.phase != kPhaseDone;
    }

    // chain bounce (stage B or C body)
    const bool specChain = (ps.phase == kPhaseSpec);
    bool end_chain = false;
    const float nsel = static_cast<float>(light_choices<kMis>(sc));
    if (kMis && sc.emitter_mis)
        ps.rad = ps.rad + ps.thr * light_hits(sc, ps.ro, ps.rd, s.hit ? h.t : 10000.0f, ps.delta, ps.last_pdf, nsel);
    if (!s.hit) {
        float w = 1.0f;
        if (s.env_pdf > 0.0f && sc.has_cdf && !ps.delta) w = mis_balance(ps.last_pdf, s.env_pdf);
        ps.rad = ps.rad + ps.thr * s.color * w;
        end_chain = true;
    } else {
        const V3 bP = s.pos, bN = s.N, bAlb = s.albedo, bE = s.color;
        if (length(bE) > 0.001f) {
            float w = 1.0f;
            if (kMis && sc.nemis != 0u && !ps.delta) {
                const float pdf = emis_pdf_at(sc, h.inst, s.gtri, ps.rd, h.t, nsel);
                if (pdf > 0.0f) w = mis_balance(ps.last_pdf, pdf);
            }
            if (kMis) ps.rad = ps.rad + ps.thr * bE * w;
            else ps.rad = ps.rad + ps.thr * bE;
        }
        const float bR = s.rough, bM = s.metal;
        const V3 bF0 = vmix(v3s(0.04f), bAlb, bM);
        if (light_choices<kMis>(sc) > 0)
            nee_light<kTex, kMis>(sc, pp, rng, dim, bP, bN, ps.rd, bAlb, bR, bM, bF0, &ps.thr, qL);
        if (sc.has_cdf) nee_env(sc, pp, rng, dim, bP, bN, ps.rd, bAlb, bR, bM, bF0, &ps.thr, qE);
        bool killed = false;
        if (ps.bounce > 1) {   // Russian roulette (766-771)
            const float p = maxc(ps.thr);
            const float rr = rng.s1(dim);
            dim += 1;
            if (p < 0.01f || rr > p) killed = true;
            else ps.thr = ps.thr / p;
        }
        if (killed) {
            end_chain = true;
        } else {
            const float cosI = fabsf(dot(normalize(ps.rd), bN));
            const V3 fres = bF0 + (1.0f - bF0) * pow5f(1.0f - cosI);
            float sp = maxc(fres);
            sp = sp * (1.0f - bR * 0.9f);
            sp = gmixf(sp, 1.0f, bM);
            const float choice = rng.s1(dim);
            dim += 1;
            if (choice < sp || bR < 0.05f) {
                const V3 inDir = ps.rd;
                ps.rd = spec_dir(rng, dim, ps.rd, bN, bR);
                ps.ro = bP + bN * 0.01f;
                if (specChain) ps.thr = ps.thr * vmix(v3s(1.0f), bAlb, bM);
                else ps.thr = ps.thr * (bAlb * (1.0f - bM));
                ps.thr = ps.thr / gmaxf(sp, 0.01f);
                if (bR < 0.05f) {
                    ps.last_pdf = 1.0f;
                    ps.delta = true;
                } else {
                    const V3 Hs = normalize(-inDir + ps.rd);
                    const float NdotHs = gmaxf(dot(bN, Hs), 0.001f);
                    const float VdotHs = gmaxf(dot(-inDir, Hs), 0.001f);
                    const float as = bR * bR, as2 = as * as;
                    const float dg = NdotHs * NdotHs * (as2 - 1.0f) + 1.0f;
                    const float Ds = as2 / (kPI * dg * dg + 1e-4f);
                    const float pdfS = Ds * NdotHs / (4.0f * VdotHs + 1e-4f);
                    ps.last_pdf = sp * pdfS;
                    ps.delta = false;
                }
            } else {
                const float d0 = rng.s1(dim), d1 = rng.s1(dim + 1);
                dim += 2;
                ps.rd = cos_hemi(bN, d0, d1);
                ps.ro = bP + bN * 0.01f;
                ps.thr = ps.thr * bAlb;
                ps.thr = ps.thr / gmaxf(1.0f - sp, 0.01f);
                ps.last_pdf = (1.0f - sp) * gmaxf(dot(ps.rd, bN), 0.0f) / kPI;
                ps.delta = false;
            }
            if (ps.bounce >= pp.max_bounces) end_chain = true;
            else ps.bounce += 1;
        }
    }
    if (end_chain) {
        if (specChain) start_diffuse_chain(pp, rng, dim, ps);
        else ps.phase = kPhaseDone;
    }
    ps.rng = rng.state;
    ps.dim = dim;
    return ps.phase != kPhaseDone;
}

}  // namespace ohao
