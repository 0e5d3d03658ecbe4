// oracle_pt.hpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// Host restatement of OHAO's path-tracing shaders, instantiated for float
// (bit-parity reference for the CUDA kernels) and double (converged FP64
// render for RMSE). Each function cites the GLSL it restates:
//   shaders/rt/pt_raygen.rgen            main() stages A/B/C (126-1186)
//   shaders/rt/pt_closesthit.rchit       closest-hit shading (37-162)
//   shaders/rt/pt_miss.rmiss             env lookup + pdf (52-81)
//   shaders/includes/rt/env_sampling.glsl (16-94)
//   shaders/includes/rt/mis.glsl          (7-9)
//   shaders/includes/rt/sampler_pcg.glsl  (9-29), sampler_sobol.glsl (13-82)
//   shaders/includes/material/ggx_aniso.glsl (12-55)
//   shaders/rt/includes/pbr_unpack.glsl   (8-20)
// Deliberate, documented deviations from the reference shader:
//   * accumulation is own-pixel progressive (the offline raygen's forced
//     behaviour, pt_raygen_offline.rgen:1239-1246), never reprojected;
//   * emissive radiance of a material is read from matColors[3*id+2].yzw
//     (unused in the reference) instead of an emissive texture;
//   * diffuse texture slot 0 selects the linear 64x64-style tile albedo map
//     (bilinear, diff_map.hpp:40-67 sampling) instead of a bindless sRGB
//     texture; other texture indices are rejected by the host API;
//   * texture filtering is restated in float (the reference uses the
//     hardware sampler, LINEAR/REPEAT, LOD 0).
// Traversal is float in both instantiations; the integrator arithmetic runs
// in Real. The float instantiation is checked bit for bit against the
// reference's own shader files compiled as C++ (glsl_pin.py), on scenes
// outside the deviations above.
#pragma once
#include "oracle_bvh.hpp"
#include <vector>
#include <cstdint>

namespace orc {

constexpr uint32_t kFlagFireflyClamp = 1u << 2;   // pt_raygen.rgen:58
constexpr uint32_t kFlagEnvFixedV = 1u << 8;      // "fixed" env lookup mode (not reference)
constexpr uint32_t kFlagVndf = 1u << 9;           // VNDF stage-B sampling (pt_raygen_realtime.rgen:723-800)
constexpr uint32_t kFlagAlphaTest = 1u << 10;     // rays without gl_RayFlagsOpaqueEXT (pt_anyhit.rahit runs)
constexpr uint32_t kFlagEmitterMis = 1u << 13;    // emitter MIS (not reference)
constexpr uint32_t kSamplerPCG = 0, kSamplerSobol = 1;
constexpr uint32_t kNoTex = 0xFFFFFFFFu;

struct Light {   // GPULight, gpu_light.hpp:10-16 (80 bytes)
    float pos_type[4], col_int[4], dir_param[4], extra[4], extra2[4];
};

struct Instance {
    uint32_t blas;
    float xform[12];      // object-to-world, row-major 3x4
    uint32_t custom;
    uint32_t mask;
    float w2o[12];        // world-to-object, row-major 3x4
    float nrm[9];         // transpose(inverse(mat3(xform))), row-major
};

struct Blas {
    uint32_t first_index = 0, index_count = 0;
    bool no_opaque = false;   // OHAO_BLAS_FLAG_NO_OPAQUE: takes the alpha test
    WideBVH bvh;
    std::vector<TriRec> tris;
    Box box = box_empty();
};

struct Settings {
    uint32_t max_bounces = 4;
    uint32_t sampler = kSamplerPCG;
    uint32_t flags = 0;
    float clamp_lum = 0.0f;
    float aniso = 0.0f, aniso_rot = 0.0f;
    float pix_jitter[2] = {0.0f, 0.0f};
};

struct View {
    float inv_view[16];   // column-major (glm)
    float inv_proj[16];
    uint32_t width, height;
};

inline void affine_xform_point(const float m[12], const float p[3], float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = ((m[r * 4 + 0] * p[0] + m[r * 4 + 1] * p[1]) + m[r * 4 + 2] * p[2]) + m[r * 4 + 3];
}
inline void affine_xform_dir(const float m[12], const float d[3], float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = (m[r * 4 + 0] * d[0] + m[r * 4 + 1] * d[1]) + m[r * 4 + 2] * d[2];
}

// An instance transform is usable when it is finite and its 3x3 part has a
// non-zero, finite determinant (double); the build treats any other instance
// as masked out (ohao_pt_build does the same).
inline bool instance_invertible(const float x[12]) {
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(x[k])) return false;
    const double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
    const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    return det != 0.0 && std::isfinite(det);
}

// Inverse of a row-major 3x4 affine transform and the normal matrix
// transpose(inverse(M3)), computed in double by cofactors, rounded to float.
inline void instance_matrices(const float x[12], float w2o[12], float nrm[9]) {
    double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    double det = a * A + b * B + c * C;
    double inv[9] = {A / det, D / det, G / det, B / det, E / det, H / det, C / det, F / det, I / det};
    double t[3] = {x[3], x[7], x[11]};
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) w2o[r * 4 + k] = static_cast<float>(inv[r * 3 + k]);
        w2o[r * 4 + 3] = static_cast<float>(-(inv[r * 3 + 0] * t[0] + inv[r * 3 + 1] * t[1] + inv[r * 3 + 2] * t[2]));
    }
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) nrm[r * 3 + k] = static_cast<float>(inv[k * 3 + r]);
}

struct Scene {
    // global geometry (rt_build.cpp:27-186 layout)
    std::vector<float> pos;       // 3 per vertex
    std::vector<float> normals;   // 4 per vertex
    std::vector<float> uvs;       // 2 per vertex
    std::vector<uint32_t> indices;
    std::vector<uint32_t> mat_ids;  // per global triangle
    std::vector<float> mats;        // 12 per material (3 x vec4)
    std::vector<Light> lights;
    // environment (light_upload.cpp:428-462)
    bool has_env = false, has_cdf = false;
    std::vector<float> env;         // RGBA32F W*H*4
    uint32_t env_w = 0, env_h = 0;
    std::vector<float> marg, cond;
    float env_integral = 0.0f, env_intensity = 1.0f;
    // tile albedo map (texture slot 0)
    std::vector<float> albedo_map;  // w*h*3
    uint32_t map_w = 0, map_h = 0;
    // bindless textures: RGBA8 UNORM texels back to back, per texture (first texel, w, h)
    std::vector<uint8_t> tex_texels;
    struct TexInfo { size_t off; int w, h; };
    std::vector<TexInfo> tex_info;

    // Texel c read as c / 255, sampled LINEAR / REPEAT at LOD 0 with texel
    // centres at (i + 0.5) / size; the four channels in float.
    void tex_sample(uint32_t idx, float u, float v, float out[4]) const {
        const TexInfo& ti = tex_info[idx];
        const int W = ti.w, H = ti.h;
        const float x = u * float(W) - 0.5f;
        const float y = v * float(H) - 0.5f;
        const float fx0 = std::floor(x), fy0 = std::floor(y);
        const float fx = x - fx0, fy = y - fy0;
        auto wrap = [](long long i, int n) { long long m = i % n; return static_cast<int>(m < 0 ? m + n : m); };
        const long long ix = static_cast<long long>(fx0), iy = static_cast<long long>(fy0);
        const int x0 = wrap(ix, W), x1 = wrap(ix + 1, W), y0 = wrap(iy, H), y1 = wrap(iy + 1, H);
        auto tx = [&](int xx, int yy, int c) {
            return float(tex_texels[ti.off * 4 + (static_cast<size_t>(yy) * W + xx) * 4 + c]) / 255.0f;
        };
        for (int c = 0; c < 4; ++c) {
            const float top = tx(x0, y0, c) * (1.0f - fx) + tx(x1, y0, c) * fx;
            const float bot = tx(x0, y1, c) * (1.0f - fx) + tx(x1, y1, c) * fx;
            out[c] = top * (1.0f - fy) + bot * fy;
        }
    }

    // pt_anyhit.rahit:17-50 for a candidate hit of a non-opaque ray: false
    // (ignore) when the instance's BLAS is non-opaque and the material's
    // diffuse texture has alpha < 0.5 at the hit's UV.
    bool alpha_accept(uint32_t inst, uint32_t prim, float u, float v) const {
        const Instance& in = instances[inst];
        if (!blases[in.blas].no_opaque) return true;
        const uint32_t gtri = (in.custom & 0xFFFFFFu) + prim;
        const uint32_t mid = mat_ids[gtri];
        const uint32_t dtex = f2u(mats[static_cast<size_t>(mid) * 12 + 3]);
        if (dtex == kNoTex || (dtex == 0u && map_w > 0)) return true;
        const uint32_t i0 = indices[gtri * 3 + 0], i1 = indices[gtri * 3 + 1], i2 = indices[gtri * 3 + 2];
        const float w = 1.0f - u - v;
        const float tu = w * uvs[2 * i0] + u * uvs[2 * i1] + v * uvs[2 * i2];
        const float tv = w * uvs[2 * i0 + 1] + u * uvs[2 * i1 + 1] + v * uvs[2 * i2 + 1];
        float c[4];
        tex_sample(dtex, tu, tv, c);
        return !(c[3] < 0.5f);
    }
    static bool alpha_accept_cb(const void* self, uint32_t inst, uint32_t prim, float u, float v) {
        return static_cast<const Scene*>(self)->alpha_accept(inst, prim, u, v);
    }
    HitFilter alpha_filter() const { return HitFilter{this, &Scene::alpha_accept_cb}; }
    // Emitter MIS (not the reference's): the emissive triangles as one more
    // choice of the light NEE. Entries run over the instances in order
    // (visible, invertible instances of opaque BLASes) and each one's
    // emissive triangles in order; pdf_area = (CDF step) / area, the CDF over
    // area x emission_weight accumulated in double and rounded to float.
    struct EmisTri { float p0[3], e1[3], e2[3], pdf_area; uint32_t inst, prim; };
    std::vector<EmisTri> emis;
    std::vector<float> emis_cdf;
    std::vector<uint32_t> emis_rank;   // per global triangle: bit 31 emissive, low bits its rank
    std::vector<uint32_t> emis_first;  // per instance: first entry (0xFFFFFFFF: none), rank of its first triangle

    // luminance of the slot-2 emission (negative channels as 0), + 1 with an
    // emissive texture
    static float emission_weight(const float* m) {
        float l = 0.2126f * std::max(m[9], 0.0f) + 0.7152f * std::max(m[10], 0.0f) + 0.0722f * std::max(m[11], 0.0f);
        if (f2u(m[7]) != kNoTex) l = l + 1.0f;
        return l;
    }
    void build_emitters() {
        emis.clear();
        emis_cdf.clear();
        emis_rank.assign(mat_ids.size(), 0u);
        emis_first.assign(instances.size() * 2, 0u);
        const size_t nt = mat_ids.size();
        uint32_t cnt = 0;
        for (size_t g = 0; g < nt; ++g) {
            const uint32_t mid = mat_ids[g];
            const bool em = static_cast<size_t>(mid) * 12 + 12 <= mats.size() && emission_weight(&mats[mid * 12]) > 0.0f;
            emis_rank[g] = cnt | (em ? 0x80000000u : 0u);
            if (em) ++cnt;
        }
        std::vector<double> acc;
        std::vector<float> area;
        double total = 0.0;
        for (uint32_t ii = 0; ii < instances.size(); ++ii) {
            const Instance& in = instances[ii];
            const Blas& bl = blases[in.blas];
            const uint32_t first = in.custom & 0xFFFFFFu, count = bl.index_count / 3;
            emis_first[2 * ii] = 0xFFFFFFFFu;
            if (!(in.mask & 0xFFu) || !instance_invertible(in.xform) || bl.no_opaque ||
                static_cast<uint64_t>(first) + count > nt)
                continue;
            emis_first[2 * ii] = static_cast<uint32_t>(emis.size());
            emis_first[2 * ii + 1] = count ? (emis_rank[first] & 0x7FFFFFFFu) : 0u;
            for (uint32_t p = 0; p < count; ++p) {
                if (!(emis_rank[first + p] & 0x80000000u)) continue;
                float v[3][3], w[3][3];
                fetch_tri(bl.first_index, p, v);
                for (int k = 0; k < 3; ++k) affine_xform_point(in.xform, v[k], w[k]);
                EmisTri E;
                for (int a = 0; a < 3; ++a) {
                    E.p0[a] = w[0][a];
                    E.e1[a] = w[1][a] - w[0][a];
                    E.e2[a] = w[2][a] - w[0][a];
                }
                const float cx = E.e1[1] * E.e2[2] - E.e1[2] * E.e2[1];
                const float cy = E.e1[2] * E.e2[0] - E.e1[0] * E.e2[2];
                const float cz = E.e1[0] * E.e2[1] - E.e1[1] * E.e2[0];
                const float a = 0.5f * std::sqrt((cx * cx + cy * cy) + cz * cz);
                total += static_cast<double>(a * emission_weight(&mats[mat_ids[first + p] * 12]));
                acc.push_back(total);
                area.push_back(a);
                E.inst = ii;
                E.prim = p;
                E.pdf_area = 0.0f;
                emis.push_back(E);
            }
        }
        if (emis.empty() || !(total > 0.0)) {
            emis.clear();
            return;
        }
        emis_cdf.resize(emis.size());
        for (size_t i = 0; i < emis.size(); ++i) emis_cdf[i] = static_cast<float>(acc[i] / total);
        emis_cdf.back() = 1.0f;
        for (size_t i = 0; i < emis.size(); ++i) {
            const float pmf = emis_cdf[i] - (i ? emis_cdf[i - 1] : 0.0f);
            emis[i].pdf_area = area[i] > 0.0f ? pmf / area[i] : 0.0f;
        }
    }
    // first entry whose CDF value is above u (the last when none is)
    uint32_t emis_search(float u) const {
        uint32_t lo = 0, hi = static_cast<uint32_t>(emis.size()) - 1u;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (emis_cdf[mid] <= u) lo = mid + 1u;
            else hi = mid;
        }
        return lo;
    }
    // the entry of a hit on global triangle gtri of instance inst, or -1
    int64_t emis_entry(uint32_t inst, uint32_t gtri) const {
        if (emis.empty() || !(emis_rank[gtri] & 0x80000000u) || emis_first[2 * inst] == 0xFFFFFFFFu) return -1;
        return static_cast<int64_t>(emis_first[2 * inst] + (emis_rank[gtri] & 0x7FFFFFFFu) - emis_first[2 * inst + 1]);
    }

    // acceleration structure
    std::vector<Instance> instances;
    std::vector<Blas> blases;
    bool two_level = false;
    WideBVH flat;
    std::vector<TriRec> flat_tris;
    WideBVH tlas;
    std::vector<uint32_t> tlas_inst;

    void fetch_tri(uint32_t first_index, uint32_t p, float v[3][3]) const {
        for (int k = 0; k < 3; ++k) {
            uint32_t vi = indices[first_index + 3 * p + k];
            for (int a = 0; a < 3; ++a) v[k][a] = pos[3 * vi + a];
        }
    }

    static Box tri_box(const float v[3][3]) {
        Box b;
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = std::min(std::min(v[0][a], v[1][a]), v[2][a]);
            b.hi[a] = std::max(std::max(v[0][a], v[1][a]), v[2][a]);
        }
        return b;
    }

    // ohao_pt_build: flat BVH over world-space triangles when the instanced
    // triangle count is <= flatten_limit, two-level TLAS/BLAS otherwise.
    void build(uint64_t flatten_limit, int force_mode) {
        for (auto& in : instances) {
            if (!instance_invertible(in.xform)) in.mask = 0;
            instance_matrices(in.xform, in.w2o, in.nrm);
        }
        uint64_t total = 0;
        for (auto& in : instances)
            if (in.mask & 0xFFu) total += blases[in.blas].index_count / 3;
        two_level = (force_mode == 2) || (force_mode == 0 && total > flatten_limit);
        if (!two_level) {
            std::vector<Box> boxes;
            std::vector<TriRec> recs;
            boxes.reserve(total);
            recs.reserve(total);
            for (uint32_t ii = 0; ii < instances.size(); ++ii) {
                const Instance& in = instances[ii];
                if (!(in.mask & 0xFFu)) continue;
                const Blas& bl = blases[in.blas];
                for (uint32_t p = 0; p < bl.index_count / 3; ++p) {
                    float v[3][3], w[3][3];
                    fetch_tri(bl.first_index, p, v);
                    for (int k = 0; k < 3; ++k) affine_xform_point(in.xform, v[k], w[k]);
                    TriRec r;
                    for (int a = 0; a < 3; ++a) { r.v0[a] = w[0][a]; r.v1[a] = w[1][a]; r.v2[a] = w[2][a]; }
                    r.prim = p; r.inst = ii; r.ref = static_cast<uint32_t>(recs.size());
                    recs.push_back(r);
                    boxes.push_back(tri_box(w));
                }
            }
            flat = WideBuilder(boxes).build();
            flat_tris.resize(recs.size());
            for (size_t j = 0; j < recs.size(); ++j) flat_tris[j] = recs[flat.prim_order[j]];
        } else {
            for (auto& bl : blases) {
                std::vector<Box> boxes;
                std::vector<TriRec> recs;
                for (uint32_t p = 0; p < bl.index_count / 3; ++p) {
                    float v[3][3];
                    fetch_tri(bl.first_index, p, v);
                    TriRec r;
                    for (int a = 0; a < 3; ++a) { r.v0[a] = v[0][a]; r.v1[a] = v[1][a]; r.v2[a] = v[2][a]; }
                    r.prim = p; r.inst = 0xFFFFFFFFu; r.ref = p;
                    recs.push_back(r);
                    Box b = tri_box(v);
                    boxes.push_back(b);
                    bl.box = box_union(bl.box, b);
                }
                bl.bvh = WideBuilder(boxes).build();
                bl.tris.resize(recs.size());
                for (size_t j = 0; j < recs.size(); ++j) bl.tris[j] = recs[bl.bvh.prim_order[j]];
            }
            std::vector<Box> iboxes;
            std::vector<uint32_t> ids;
            for (uint32_t ii = 0; ii < instances.size(); ++ii) {
                const Instance& in = instances[ii];
                if (!(in.mask & 0xFFu) || blases[in.blas].tris.empty()) continue;
                iboxes.push_back(instance_world_box(in, blases[in.blas].tris));
                ids.push_back(ii);
            }
            tlas = WideBuilder(iboxes).build();
            tlas_inst.resize(ids.size());
            for (size_t j = 0; j < ids.size(); ++j) tlas_inst[j] = ids[tlas.prim_order[j]];
        }
        build_emitters();
    }

    // World box of an instance: min/max of its transform applied to every
    // vertex of its BLAS's triangle records, padded by 2^-20 of the
    // coordinate magnitude so that rounding in the transform cannot exclude
    // geometry.
    static Box instance_world_box(const Instance& in, const std::vector<TriRec>& tris) {
        Box wb = box_empty();
        if (tris.empty()) return wb;
        for (const TriRec& r : tris) {
            const float* vs[3] = {r.v0, r.v1, r.v2};
            for (int k = 0; k < 3; ++k) {
                float w[3];
                affine_xform_point(in.xform, vs[k], w);
                for (int a = 0; a < 3; ++a) { wb.lo[a] = std::min(wb.lo[a], w[a]); wb.hi[a] = std::max(wb.hi[a], w[a]); }
            }
        }
        for (int a = 0; a < 3; ++a) {
            float pad = (std::fabs(wb.lo[a]) + std::fabs(wb.hi[a])) * 0x1p-20f;
            wb.lo[a] = wb.lo[a] - pad;
            wb.hi[a] = wb.hi[a] + pad;
        }
        return wb;
    }

    // traceRayEXT(gl_RayFlagsOpaqueEXT) closest hit.
    // alpha: a ray without gl_RayFlagsOpaqueEXT (the alpha test applies).
    HitRec closest(const float o[3], const float d[3], float tmin, float tmax, TravStats* st = nullptr,
                   bool alpha = false) const {
        HitRec best;
        if (!(tmax > tmin)) return best;
        const HitFilter af = alpha_filter();
        const HitFilter* filter = alpha ? &af : nullptr;
        if (!two_level) {
            RayPre r = ray_pre(o, d);
            BvhView v{flat.nodes.data(), flat_tris.data(), static_cast<uint32_t>(flat.nodes.size())};
            bvh_closest(v, r, tmin, tmax, best, 0xFFFFFFFFu, st, filter);
            return best;
        }
        RayPre r = ray_pre(o, d);
        std::vector<std::pair<uint32_t, float>> stack;
        if (tlas.nodes.empty()) return best;
        stack.push_back({0u, -INFINITY});
        while (!stack.empty()) {
            auto [ni, tn0] = stack.back();
            stack.pop_back();
            if (tn0 > cull_limit(best, tmax)) continue;
            const WideNode& n = tlas.nodes[ni];
            if (st) st->nodes++;
            NodeHits h = node_test(n, r, tmin, best.hit() ? best.t : tmax);
            for (int i = 0; i < 8; ++i) {
                if (!(h.mask & (1u << i)) || (n.imask & (1u << i))) continue;
                uint32_t cnt = n.meta[i] >> 5, off = n.meta[i] & 31u;
                for (uint32_t q = 0; q < cnt; ++q) {
                    uint32_t ii = tlas_inst[n.tri_base + off + q];
                    const Instance& in = instances[ii];
                    const Blas& bl = blases[in.blas];
                    if (st) st->insts++;
                    float oo[3], od[3];
                    affine_xform_point(in.w2o, o, oo);
                    affine_xform_dir(in.w2o, d, od);
                    RayPre ro = ray_pre(oo, od);
                    BvhView v{bl.bvh.nodes.data(), bl.tris.data(), static_cast<uint32_t>(bl.bvh.nodes.size())};
                    bvh_closest(v, ro, tmin, tmax, best, ii, st, filter);
                }
            }
            uint32_t ids[8]; float tns[8]; int cnt = 0;
            for (int i = 0; i < 8; ++i) {
                if (!(h.mask & (1u << i)) || !(n.imask & (1u << i))) continue;
                ids[cnt] = n.child_base + (n.meta[i] & 7u);
                tns[cnt] = h.tnear[i];
                cnt++;
            }
            for (int i = 1; i < cnt; ++i)
                for (int j = i; j > 0 && tns[j] > tns[j - 1]; --j) { std::swap(tns[j], tns[j - 1]); std::swap(ids[j], ids[j - 1]); }
            for (int i = 0; i < cnt; ++i) stack.push_back({ids[i], tns[i]});
        }
        return best;
    }

    // traceRayEXT(TerminateOnFirstHit|Opaque|SkipClosestHit): occluded?
    bool occluded(const float o[3], const float d[3], float tmin, float tmax, TravStats* st = nullptr,
                  bool alpha = false) const {
        if (!(tmax > tmin)) return false;
        RayPre r = ray_pre(o, d);
        const HitFilter af = alpha_filter();
        const HitFilter* filter = alpha ? &af : nullptr;
        if (!two_level) {
            BvhView v{flat.nodes.data(), flat_tris.data(), static_cast<uint32_t>(flat.nodes.size())};
            return bvh_any(v, r, tmin, tmax, st, filter);
        }
        if (tlas.nodes.empty()) return false;
        std::vector<uint32_t> stack{0u};
        while (!stack.empty()) {
            uint32_t ni = stack.back();
            stack.pop_back();
            const WideNode& n = tlas.nodes[ni];
            if (st) st->nodes++;
            NodeHits h = node_test(n, r, tmin, tmax);
            for (int i = 0; i < 8; ++i) {
                if (!(h.mask & (1u << i))) continue;
                if (n.imask & (1u << i)) { stack.push_back(n.child_base + (n.meta[i] & 7u)); continue; }
                uint32_t cnt = n.meta[i] >> 5, off = n.meta[i] & 31u;
                for (uint32_t q = 0; q < cnt; ++q) {
                    uint32_t ii = tlas_inst[n.tri_base + off + q];
                    const Instance& in = instances[ii];
                    const Blas& bl = blases[in.blas];
                    if (st) st->insts++;
                    float oo[3], od[3];
                    affine_xform_point(in.w2o, o, oo);
                    affine_xform_dir(in.w2o, d, od);
                    RayPre ro = ray_pre(oo, od);
                    BvhView v{bl.bvh.nodes.data(), bl.tris.data(), static_cast<uint32_t>(bl.bvh.nodes.size())};
                    if (bvh_any(v, ro, tmin, tmax, st, filter, ii)) return true;
                }
            }
        }
        return false;
    }

    // Brute-force ground truth over every visible instance triangle.
    HitRec closest_brute(const float o[3], const float d[3], float tmin, float tmax, bool alpha = false) const {
        HitRec best;
        if (!(tmax > tmin)) return best;
        for (uint32_t ii = 0; ii < instances.size(); ++ii) {
            const Instance& in = instances[ii];
            if (!(in.mask & 0xFFu)) continue;
            const Blas& bl = blases[in.blas];
            RayPre r;
            bool obj = two_level;
            if (obj) {
                float oo[3], od[3];
                affine_xform_point(in.w2o, o, oo);
                affine_xform_dir(in.w2o, d, od);
                r = ray_pre(oo, od);
            } else {
                r = ray_pre(o, d);
            }
            for (uint32_t p = 0; p < bl.index_count / 3; ++p) {
                float v[3][3], w[3][3];
                fetch_tri(bl.first_index, p, v);
                if (!obj) for (int k = 0; k < 3; ++k) affine_xform_point(in.xform, v[k], w[k]);
                float t, u, vv;
                bool h = obj ? tri_intersect(r, v[0], v[1], v[2], tmin, tmax, t, u, vv)
                             : tri_intersect(r, w[0], w[1], w[2], tmin, tmax, t, u, vv);
                if (!h) continue;
                if (alpha && !alpha_accept(ii, p, u, vv)) continue;
                if (!best.hit() || t < best.t || (t == best.t && key_less(ii, p, best.inst, best.prim))) {
                    best.t = t; best.u = u; best.v = vv; best.inst = ii; best.prim = p;
                }
            }
        }
        return best;
    }
};

// ---------------------------------------------------------------------------
// Samplers (sampler_pcg.glsl:9-29, sampler_sobol.glsl:13-82)
// ---------------------------------------------------------------------------
extern const uint32_t kSobolDirs[128];

inline uint32_t owen_scramble(uint32_t v, uint32_t seed) {
    v = (v << 16) | (v >> 16);
    v = ((v & 0x00FF00FFu) << 8) | ((v & 0xFF00FF00u) >> 8);
    v = ((v & 0x0F0F0F0Fu) << 4) | ((v & 0xF0F0F0F0u) >> 4);
    v = ((v & 0x33333333u) << 2) | ((v & 0xCCCCCCCCu) >> 2);
    v = ((v & 0x55555555u) << 1) | ((v & 0xAAAAAAAAu) >> 1);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    v = ((v & 0x55555555u) << 1) | ((v & 0xAAAAAAAAu) >> 1);
    v = ((v & 0x33333333u) << 2) | ((v & 0xCCCCCCCCu) >> 2);
    v = ((v & 0x0F0F0F0Fu) << 4) | ((v & 0xF0F0F0F0u) >> 4);
    v = ((v & 0x00FF00FFu) << 8) | ((v & 0xFF00FF00u) >> 8);
    v = (v << 16) | (v >> 16);
    return v;
}
inline uint32_t sobol_int(uint32_t index, uint32_t dim) {
    uint32_t r = 0;
    for (uint32_t bit = 0; index != 0; bit++, index >>= 1)
        if (index & 1u) r ^= kSobolDirs[dim * 32 + bit];
    return r;
}
inline uint32_t sobol_hash_pixel(uint32_t px, uint32_t py) {
    uint32_t h = (px * 0x1b873593u) ^ (py * 0xcc9e2d51u);
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}
inline float sobol_sample(uint32_t index, uint32_t seed, uint32_t dim) {
    uint32_t pad = dim >> 2, local = dim & 3u;
    uint32_t s = seed ^ (pad * 0x9e3779b9u);
    uint32_t v = owen_scramble(sobol_int(index, local), s);
    return static_cast<float>(v >> 8) * (1.0f / 16777216.0f);
}
inline uint32_t pcg_next(uint32_t& st) {
    st = st * 747796405u + 2891336453u;
    uint32_t w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (w >> 22u) ^ w;
}

struct Sampler {
    uint32_t type, state, index, seed;
    void init(uint32_t t, uint32_t px, uint32_t py, uint32_t sampleIdx) {
        type = t;
        state = px * 1973u + py * 9277u + sampleIdx * 26699u + 1u;
        index = sampleIdx;
        seed = sobol_hash_pixel(px, py);
    }
    float s1(uint32_t dim) {
        if (type == kSamplerPCG) return static_cast<float>(pcg_next(state)) / 4294967296.0f;
        return sobol_sample(index, seed, dim);
    }
};

// ---------------------------------------------------------------------------
// Integrator
// ---------------------------------------------------------------------------
template <class R>
struct Surf {                 // RayPayload after closest hit / miss
    bool hit = false;
    V3<R> color, hitPos, N, albedo;
    R rough = 0, metal = 0;
    R dist = -1;
    R envPdf = 0;
    // provenance for the adjoint and emitter MIS
    uint32_t gtri = 0, matid = 0, inst = 0;
    float uv[2] = {0, 0};
};

template <class R>
struct PathTracer {
    const Scene& sc;
    const Settings& st;
    PathTracer(const Scene& s, const Settings& t) : sc(s), st(t) {}

    // parameter overrides used by the adjoint checks (sampling vs evaluation)
    const float* albedo_map_override = nullptr;

    static constexpr R PI = R(3.14159265358979f);     // OHAO_PI
    static constexpr R TWOPI = R(6.28318530717959f);  // OHAO_TWOPI

    // env_sampling.glsl:16-37
    int search_marg(R u) const {
        int lo = 0, hi = static_cast<int>(sc.env_h) - 1;
        while (lo < hi) { int mid = (lo + hi) / 2; if (R(sc.marg[mid]) < u) lo = mid + 1; else hi = mid; }
        return lo;
    }
    int search_cond(uint32_t base, R u) const {
        int lo = 0, hi = static_cast<int>(sc.env_w) - 1;
        while (lo < hi) { int mid = (lo + hi) / 2; if (R(sc.cond[base + mid]) < u) lo = mid + 1; else hi = mid; }
        return lo;
    }
    // env_sampling.glsl:52-74
    void sample_env(R u1, R u2, V3<R>& dir, R& pdf) const {
        const uint32_t W = sc.env_w, H = sc.env_h;
        int y = search_marg(u1);
        uint32_t base = static_cast<uint32_t>(y) * W;
        int x = search_cond(base, u2);
        R u = (R(float(x)) + R(0.5f)) / R(float(W));
        R v = (R(float(y)) + R(0.5f)) / R(float(H));
        R phi = (u - R(0.5f)) * TWOPI;
        R theta = v * PI;
        R sinT = m_sin(theta);
        dir = V3<R>(sinT * m_cos(phi), m_cos(theta), sinT * m_sin(phi));
        R theta2 = (R(float(y)) + R(0.5f)) / R(float(H)) * PI;
        R sinT2 = gmax(m_sin(theta2), R(1e-4f));
        R condDiff = R(sc.cond[base + x]) - (x > 0 ? R(sc.cond[base + x - 1]) : R(0));
        R margDiff = R(sc.marg[y]) - (y > 0 ? R(sc.marg[y - 1]) : R(0));
        R pdfUV = condDiff * margDiff * R(float(W)) * R(float(H));
        pdf = pdfUV / (TWOPI * PI * sinT2);
        pdf = gmax(pdf, R(0));
    }
    // env_sampling.glsl:77-94
    R pdf_env(V3<R> dir) const {
        const uint32_t W = sc.env_w, H = sc.env_h;
        R theta = m_acos(gclamp(dir.y, R(-1), R(1)));
        R phi = m_atan2(dir.z, dir.x);
        R u = phi / TWOPI + R(0.5f);
        R v = theta / PI;
        int x = std::clamp(static_cast<int>(u * R(float(W))), 0, static_cast<int>(W) - 1);
        int y = std::clamp(static_cast<int>(v * R(float(H))), 0, static_cast<int>(H) - 1);
        uint32_t base = static_cast<uint32_t>(y) * W;
        R condDiff = R(sc.cond[base + x]) - (x > 0 ? R(sc.cond[base + x - 1]) : R(0));
        R margDiff = R(sc.marg[y]) - (y > 0 ? R(sc.marg[y - 1]) : R(0));
        R pdfUV = condDiff * margDiff * R(float(W)) * R(float(H));
        R sinT = gmax(m_sin(theta), R(1e-4f));
        return gmax(pdfUV / (TWOPI * PI * sinT), R(0));
    }
    // Hardware-sampler stand-in: bilinear, REPEAT, texel centres at (i+0.5)/N.
    V3<R> env_texture(R u, R v) const {
        const int W = static_cast<int>(sc.env_w), H = static_cast<int>(sc.env_h);
        R x = u * R(float(W)) - R(0.5f);
        R y = v * R(float(H)) - R(0.5f);
        R fx0 = std::floor(x), fy0 = std::floor(y);
        R fx = x - fx0, fy = y - fy0;
        auto wrap = [](long long i, int n) { long long m = i % n; return static_cast<int>(m < 0 ? m + n : m); };
        long long ix = static_cast<long long>(fx0), iy = static_cast<long long>(fy0);
        int x0 = wrap(ix, W), x1 = wrap(ix + 1, W), y0 = wrap(iy, H), y1 = wrap(iy + 1, H);
        auto tex = [&](int xx, int yy) {
            const float* p = &sc.env[(static_cast<size_t>(yy) * W + xx) * 4];
            return V3<R>(R(p[0]), R(p[1]), R(p[2]));
        };
        V3<R> top = tex(x0, y0) * (R(1) - fx) + tex(x1, y0) * fx;
        V3<R> bot = tex(x0, y1) * (R(1) - fx) + tex(x1, y1) * fx;
        return top * (R(1) - fy) + bot * fy;
    }
    // pt_miss.rmiss:52-81
    void miss(V3<R> rd, Surf<R>& s) const {
        s.hit = false;
        s.dist = R(-1);
        if (sc.has_env) {
            V3<R> dir = normalize(rd);
            R phi = m_atan2(dir.z, dir.x);
            R u = phi / R(6.2831853f) + R(0.5f);
            R v;
            if (st.flags & kFlagEnvFixedV) v = m_acos(gclamp(dir.y, R(-1), R(1))) / R(3.1415926f);
            else v = m_asin(gclamp(dir.y, R(-1), R(1))) / R(3.1415926f) + R(0.5f);
            R envS = (sc.env_intensity > 0.0f) ? R(sc.env_intensity) : R(1);
            s.color = env_texture(u, v) * envS;
        } else {
            s.color = V3<R>(R(0));
        }
        if (sc.has_env && sc.has_cdf) s.envPdf = pdf_env(normalize(rd));
        else s.envPdf = R(0);
    }
    // diff_map.hpp:40-67 bilinear sample of the tile albedo map
    V3<R> albedo_map_sample(R u, R v) const {
        const float* map = albedo_map_override ? albedo_map_override : sc.albedo_map.data();
        const int w = static_cast<int>(sc.map_w), h = static_cast<int>(sc.map_h);
        u = gclamp(u, R(0), R(1));
        v = gclamp(v, R(0), R(1));
        R x = u * R(float(w - 1));
        R y = v * R(float(h - 1));
        int x0 = static_cast<int>(x), y0 = static_cast<int>(y);
        int x1 = std::min(x0 + 1, w - 1), y1 = std::min(y0 + 1, h - 1);
        R tx = x - R(float(x0)), ty = y - R(float(y0));
        R out[3];
        for (int c = 0; c < 3; ++c) {
            auto at = [&](int ix, int iy) { return R(map[(static_cast<size_t>(iy) * w + ix) * 3 + c]); };
            R a = at(x0, y0) * (R(1) - tx) + at(x1, y0) * tx;
            R b = at(x0, y1) * (R(1) - tx) + at(x1, y1) * tx;
            out[c] = a * (R(1) - ty) + b * ty;
        }
        return V3<R>(out[0], out[1], out[2]);
    }
    // pt_closesthit.rchit:37-162
    void closest_hit(const float o[3], const float d[3], const HitRec& h, Surf<R>& s) const {
        s.hit = true;
        R t = R(h.t);
        V3<R> ro{R(o[0]), R(o[1]), R(o[2])}, rd{R(d[0]), R(d[1]), R(d[2])};
        s.hitPos = ro + rd * t;
        s.dist = t;
        const Instance& in = sc.instances[h.inst];
        R u = R(h.u), v = R(h.v);
        R w = R(1) - u - v;
        uint32_t gtri = (in.custom & 0xFFFFFFu) + h.prim;
        s.gtri = gtri;
        s.inst = h.inst;
        uint32_t i0 = sc.indices[gtri * 3 + 0], i1 = sc.indices[gtri * 3 + 1], i2 = sc.indices[gtri * 3 + 2];
        R tu = w * R(sc.uvs[2 * i0]) + u * R(sc.uvs[2 * i1]) + v * R(sc.uvs[2 * i2]);
        R tv = w * R(sc.uvs[2 * i0 + 1]) + u * R(sc.uvs[2 * i1 + 1]) + v * R(sc.uvs[2 * i2 + 1]);
        s.uv[0] = static_cast<float>(tu);
        s.uv[1] = static_cast<float>(tv);
        auto nv = [&](uint32_t i) { return V3<R>(R(sc.normals[4 * i]), R(sc.normals[4 * i + 1]), R(sc.normals[4 * i + 2])); };
        V3<R> n0 = nv(i0), n1 = nv(i1), n2 = nv(i2);
        V3<R> interp = n0 * w + n1 * u + n2 * v;
        auto nmul = [&](V3<R> x) {
            const float* m = in.nrm;
            return V3<R>(R(m[0]) * x.x + R(m[1]) * x.y + R(m[2]) * x.z,
                         R(m[3]) * x.x + R(m[4]) * x.y + R(m[5]) * x.z,
                         R(m[6]) * x.x + R(m[7]) * x.y + R(m[8]) * x.z);
        };
        V3<R> wn;
        bool thin = !(dot(interp, interp) > R(0.0001f));
        if (!thin) {
            wn = normalize(nmul(normalize(interp)));
        } else {
            float oo[3], od[3];
            affine_xform_point(in.w2o, o, oo);
            affine_xform_dir(in.w2o, d, od);
            V3<R> hl = V3<R>(R(oo[0]), R(oo[1]), R(oo[2])) + V3<R>(R(od[0]), R(od[1]), R(od[2])) * t;
            V3<R> al(std::fabs(hl.x), std::fabs(hl.y), std::fabs(hl.z));
            auto sgn = [](R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); };
            V3<R> ln;
            if (al.x >= al.y && al.x >= al.z) ln = V3<R>(sgn(hl.x), R(0), R(0));
            else if (al.y >= al.z) ln = V3<R>(R(0), sgn(hl.y), R(0));
            else ln = V3<R>(R(0), R(0), sgn(hl.z));
            wn = normalize(nmul(ln));
            if (dot(wn, rd) > R(0)) wn = -wn;
        }
        uint32_t mid = sc.mat_ids[gtri];
        s.matid = mid;
        const float* m = &sc.mats[static_cast<size_t>(mid) * 12];
        const uint32_t diffTex = f2u(m[3]), normTex = f2u(m[6]), emisTex = f2u(m[7]), rmTex = f2u(m[8]);
        // bindless texture sample at the hit's UV (texture coordinates in float)
        auto tex = [&](uint32_t idx, R out[4]) {
            float c[4];
            sc.tex_sample(idx, static_cast<float>(tu), static_cast<float>(tv), c);
            for (int k = 0; k < 4; ++k) out[k] = R(c[k]);
        };
        // albedo x sRGB-decoded diffuse texture (pt_closesthit.rchit:108-113);
        // diffuse index 0 = the tile albedo map when one is set
        V3<R> alb{R(m[0]), R(m[1]), R(m[2])};
        if (diffTex != kNoTex) {
            if (diffTex == 0u && sc.map_w > 0) {
                alb = alb * albedo_map_sample(tu, tv);
            } else {
                R c[4];
                tex(diffTex, c);
                alb = alb * V3<R>(m_pow(c[0], R(2.2f)), m_pow(c[1], R(2.2f)), m_pow(c[2], R(2.2f)));
            }
        }
        // normal map in the Frisvad basis (pt_closesthit.rchit:116-133)
        if (normTex != kNoTex) {
            R c[4];
            tex(normTex, c);
            V3<R> mapN = normalize(V3<R>(c[0] * R(2) - R(1), c[1] * R(2) - R(1), c[2] * R(2) - R(1)));
            V3<R> T, B;
            if (wn.z < R(-0.9999f)) {
                T = V3<R>(R(0), R(-1), R(0));
                B = V3<R>(R(-1), R(0), R(0));
            } else {
                R a = R(1) / (R(1) + wn.z);
                R dd = -wn.x * wn.y * a;
                T = V3<R>(R(1) - wn.x * wn.x * a, dd, -wn.x);
                B = V3<R>(dd, R(1) - wn.y * wn.y * a, -wn.y);
            }
            wn = normalize(T * mapN.x + B * mapN.y + wn * mapN.z);
        }
        s.N = wn;
        s.albedo = alb;
        // roughness / metallic x ORM texture G / B (pt_closesthit.rchit:139-148)
        R rough = R(m[4]), metal = R(m[5]);
        if (rmTex != kNoTex) {
            R c[4];
            tex(rmTex, c);
            rough = rough * c[1];
            metal = metal * c[2];
        }
        rough = gmax(rough, R(0.04f));
        // sRGB-decoded emissive texture (pt_closesthit.rchit:150-156) plus the
        // slot-2 emission of this ABI
        V3<R> emis(R(0));
        if (emisTex != kNoTex) {
            R c[4];
            tex(emisTex, c);
            emis = V3<R>(m_pow(c[0], R(2.2f)), m_pow(c[1], R(2.2f)), m_pow(c[2], R(2.2f)));
        }
        s.color = emis + V3<R>(R(m[9]), R(m[10]), R(m[11]));
        // payload.attenuation = (roughness, clamp(metallic,0,1), curv) then
        // unpackHitPbr
        R rr, mm;
        unpack_hit_pbr(V3<R>(rough, gclamp(metal, R(0), R(1)), R(0)), rr, mm);
        s.rough = rr;
        s.metal = mm;
    }
    // unpackHitPbr (pbr_unpack.glsl:8-20)
    static void unpack_hit_pbr(V3<R> att, R& rr, R& mm) {
        if (att.x < R(0) && att.y < R(1e-4f)) {
            rr = -att.x; if (rr >= R(10)) rr = rr - R(10); rr = gmax(rr, R(0.01f)); mm = R(1);
        } else {
            rr = std::fabs(att.x); if (rr >= R(10)) rr = rr - R(10); rr = gmax(rr, R(0.01f)); mm = gclamp(att.y, R(0), R(1));
        }
    }

    void trace(V3<R> o, V3<R> d, Surf<R>& s, TravStats* ts) const {
        float of[3] = {float(o.x), float(o.y), float(o.z)}, df[3] = {float(d.x), float(d.y), float(d.z)};
        HitRec h = sc.closest(of, df, 0.001f, 10000.0f, ts, (st.flags & kFlagAlphaTest) != 0u);
        if (h.hit()) closest_hit(of, df, h, s);
        else miss(d, s);
    }
    // Shadow query; on a miss the miss shader runs (payload.color = env).
    bool shadow(V3<R> o, V3<R> d, R tmax, Surf<R>& s, TravStats* ts) const {
        float of[3] = {float(o.x), float(o.y), float(o.z)}, df[3] = {float(d.x), float(d.y), float(d.z)};
        bool occ = sc.occluded(of, df, 0.001f, float(tmax), ts, (st.flags & kFlagAlphaTest) != 0u);
        if (!occ) miss(d, s);
        return !occ;
    }

    // pt_raygen.rgen:90-97
    V3<R> cos_hemi(V3<R> N, R u0, R u1) const {
        V3<R> up = std::fabs(N.y) < R(0.999f) ? V3<R>(R(0), R(1), R(0)) : V3<R>(R(1), R(0), R(0));
        V3<R> T = normalize(cross(up, N));
        V3<R> B = cross(N, T);
        R r = m_sqrt(u0);
        R phi = R(6.2831853f) * u1;
        return normalize(T * r * m_cos(phi) + B * r * m_sin(phi) + N * m_sqrt(gmax(R(0), R(1) - r * r)));
    }
    // ggx_aniso.glsl:12-55
    R ggxD(V3<R> N, V3<R> H, R NdotH, R rough) const {
        R an = R(st.aniso);
        if (an < R(0.001f)) {
            R a = rough * rough, a2 = a * a;
            R denom = NdotH * NdotH * (a2 - R(1)) + R(1);
            return a2 / (R(3.14159265f) * denom * denom + R(0.0001f));
        }
        V3<R> up(R(0), R(1), R(0));
        V3<R> ref = std::fabs(dot(up, N)) > R(0.97f) ? V3<R>(R(1), R(0), R(0)) : up;
        V3<R> T = normalize(ref - N * dot(ref, N));
        V3<R> B = cross(N, T);
        R c = m_cos(R(st.aniso_rot)), s = m_sin(R(st.aniso_rot));
        V3<R> Tr = T * c + B * s;
        V3<R> Br = B * c - T * s;
        R r2 = rough * rough;
        R aspect = m_sqrt(R(1) - an * R(0.9f));
        R rT = gmax(r2 / aspect, R(0.001f));
        R rB = gmax(r2 * aspect, R(0.001f));
        R TdotH = dot(Tr, H), BdotH = dot(Br, H);
        R dd = (TdotH * TdotH / rT) + (BdotH * BdotH / rB) + NdotH * NdotH;
        return R(1) / (R(3.14159265f) * rT * rB * dd * dd + R(0.0001f));
    }
    static R mis(R a, R b) { return a / gmax(a + b, R(1e-6f)); }   // mis.glsl:7-9

    V3<R> clampc(V3<R> c) const {
        if ((st.flags & kFlagFireflyClamp) && st.clamp_lum > 0.0f) {
            R l = lum(c);
            if (l > R(st.clamp_lum)) c = c * (R(st.clamp_lum) / l);
        }
        return c;
    }

    // Light choice and sample point of a light NEE (the draws and geometry of
    // pt_raygen.rgen:305-383); valid = NdotL > 0 && weight > 0. mis_pdf: the
    // solid-angle pdf of an emitter-MIS sample (emissive triangle, sphere or
    // area light), else 0.
    struct LightSmp {
        bool valid = false;
        V3<R> L, Le;
        R weight = 0, shadowDist = 0, NdotL = 0, n = 0, mis_pdf = 0;
    };
    bool emitter_mis() const { return (st.flags & kFlagEmitterMis) != 0u; }
    // choices of the light NEE: the lights, + the emissive triangles as one
    uint32_t light_choices() const {
        return static_cast<uint32_t>(sc.lights.size()) + ((emitter_mis() && !sc.emis.empty()) ? 1u : 0u);
    }
    // emission of triangle prim of instance inst at barycentrics (u, v), as
    // closest_hit evaluates it
    V3<R> emission_at(uint32_t inst, uint32_t prim, R u, R v) const {
        const Instance& in = sc.instances[inst];
        const uint32_t gtri = (in.custom & 0xFFFFFFu) + prim;
        const float* m = &sc.mats[static_cast<size_t>(sc.mat_ids[gtri]) * 12];
        const uint32_t emisTex = f2u(m[7]);
        V3<R> emis(R(0));
        if (emisTex != kNoTex) {
            const R w = R(1) - u - v;
            const uint32_t i0 = sc.indices[gtri * 3 + 0], i1 = sc.indices[gtri * 3 + 1], i2 = sc.indices[gtri * 3 + 2];
            const R tu = w * R(sc.uvs[2 * i0]) + u * R(sc.uvs[2 * i1]) + v * R(sc.uvs[2 * i2]);
            const R tv = w * R(sc.uvs[2 * i0 + 1]) + u * R(sc.uvs[2 * i1 + 1]) + v * R(sc.uvs[2 * i2 + 1]);
            float c[4];
            sc.tex_sample(emisTex, static_cast<float>(tu), static_cast<float>(tv), c);
            emis = V3<R>(m_pow(R(c[0]), R(2.2f)), m_pow(R(c[1]), R(2.2f)), m_pow(R(c[2]), R(2.2f)));
        }
        return emis + V3<R>(R(m[9]), R(m[10]), R(m[11]));
    }
    LightSmp sample_light(Sampler& smp, uint32_t& dim, V3<R> P, V3<R> N) const {
        LightSmp out;
        const uint32_t n = light_choices();
        const uint32_t nl = static_cast<uint32_t>(sc.lights.size());
        const float usel = smp.s1(dim);
        uint32_t li = static_cast<uint32_t>(usel * float(n));
        dim += 1;
        li = std::min(li, n - 1u);
        if (emitter_mis() && li == nl) {
            // an emissive triangle by power (the rest of the choice's draw),
            // a uniform point on it; both faces emit
            const auto& E = sc.emis[sc.emis_search(usel * float(n) - float(nl))];
            R a0 = R(smp.s1(dim)), a1 = R(smp.s1(dim + 1)); dim += 2;
            R su = m_sqrt(a0);
            R b1 = su * (R(1) - a1), b2 = su * a1;
            V3<R> e1(R(E.e1[0]), R(E.e1[1]), R(E.e1[2])), e2(R(E.e2[0]), R(E.e2[1]), R(E.e2[2]));
            V3<R> lp = V3<R>(R(E.p0[0]), R(E.p0[1]), R(E.p0[2])) + e1 * b1 + e2 * b2;
            V3<R> ng = normalize(cross(e1, e2));
            V3<R> tl = lp - P;
            R ld = length(tl);
            V3<R> L = tl / ld;
            R lcos = std::fabs(dot(L, ng));
            R weight = lcos / (R(E.pdf_area) * (ld * ld));
            out.mis_pdf = R(E.pdf_area) * (ld * ld) / (lcos * R(float(n)));
            out.NdotL = gmax(dot(N, L), R(0));
            out.valid = out.NdotL > R(0) && weight > R(0);
            out.L = L;
            out.Le = emission_at(E.inst, E.prim, b1, b2);
            out.weight = weight;
            out.shadowDist = ld - R(0.02f);
            out.n = R(float(n));
            return out;
        }
        const Light& L0 = sc.lights[li];
        R ltype = R(L0.pos_type[3]);
        V3<R> lc(R(L0.pos_type[0]), R(L0.pos_type[1]), R(L0.pos_type[2]));
        V3<R> lcol(R(L0.col_int[0]), R(L0.col_int[1]), R(L0.col_int[2]));
        R lint = R(L0.col_int[3]);
        R lrad = R(L0.dir_param[3]);
        V3<R> ldir = normalize(V3<R>(R(L0.dir_param[0]), R(L0.dir_param[1]), R(L0.dir_param[2])));
        R outerAngle = R(L0.extra[3]);
        R r = gmax(lrad, R(0.01f));
        R area = R(4) * R(3.14159f) * r * r;
        V3<R> Le = lcol * lint / gmax(area, R(0.01f));
        V3<R> L;
        R shadowDist, weight;
        if (ltype < R(0.5f)) {
            R u1 = R(smp.s1(dim)), u2 = R(smp.s1(dim + 1)); dim += 2;
            R cosT = R(1) - R(2) * u1;
            R sinT = m_sqrt(gmax(R(0), R(1) - cosT * cosT));
            R phi = R(6.2831853f) * u2;
            V3<R> off = V3<R>(sinT * m_cos(phi), sinT * m_sin(phi), cosT) * r;
            V3<R> lp = lc + off;
            V3<R> ln = normalize(off);
            V3<R> tl = lp - P;
            R ld = length(tl);
            L = tl / ld;
            R lcos = gmax(dot(-L, ln), R(0));
            R la = R(4) * R(3.14159f) * r * r;
            weight = lcos * la / (ld * ld);
            shadowDist = ld - R(0.02f);
            if (emitter_mis()) out.mis_pdf = (ld * ld) / (lcos * la * R(float(n)));
        } else if (ltype < R(1.5f)) {
            L = -ldir;
            weight = R(1);
            shadowDist = R(10000);
        } else if (ltype < R(2.5f)) {
            R u1 = R(smp.s1(dim)), u2 = R(smp.s1(dim + 1)); dim += 2;
            R cosT = R(1) - R(2) * u1;
            R sinT = m_sqrt(gmax(R(0), R(1) - cosT * cosT));
            R phi = R(6.2831853f) * u2;
            V3<R> off = V3<R>(sinT * m_cos(phi), sinT * m_sin(phi), cosT) * r;
            V3<R> lp = lc + off;
            V3<R> tl = lp - P;
            R ld = length(tl);
            L = tl / ld;
            shadowDist = ld - R(0.02f);
            R cosA = dot(-L, ldir);
            // radians(x) = x * (pi/180)
            R innerCos = m_cos(R(L0.dir_param[3]) * R(0.017453292f));
            R outerCos = m_cos(outerAngle * R(0.017453292f));
            R spot = gclamp((cosA - outerCos) / (innerCos - outerCos + R(0.001f)), R(0), R(1));
            spot = spot * spot;
            R la = R(4) * R(3.14159f) * r * r;
            weight = la / (ld * ld) * spot;
        } else {
            V3<R> e1(R(L0.extra[0]), R(L0.extra[1]), R(L0.extra[2]));
            V3<R> e2(R(L0.extra2[0]), R(L0.extra2[1]), R(L0.extra2[2]));
            R ar = R(L0.extra2[3]);
            R a0 = R(smp.s1(dim)), a1 = R(smp.s1(dim + 1)); dim += 2;
            V3<R> lp = lc + e1 * a0 + e2 * a1;
            V3<R> ln = normalize(cross(e1, e2));
            V3<R> tl = lp - P;
            R ld = length(tl);
            L = tl / ld;
            R lcos = gmax(dot(-L, ln), R(0));
            weight = lcos * ar / (ld * ld);
            shadowDist = ld - R(0.02f);
            if (emitter_mis()) out.mis_pdf = (ld * ld) / (lcos * ar * R(float(n)));
        }
        out.NdotL = gmax(dot(N, L), R(0));
        out.valid = out.NdotL > R(0) && weight > R(0);
        out.L = L;
        out.Le = Le;
        out.weight = weight;
        out.shadowDist = shadowDist;
        out.n = R(float(n));
        return out;
    }

    // Analytic light NEE (pt_raygen.rgen:305-434 for bounce 0 with ggxD,
    // 585-705 / 893-1013 for chain bounces with the inline D). Returns the
    // unclamped contribution without throughput; `visible` reports the test.
    struct NeeOut { bool valid = false; V3<R> contrib; };
    NeeOut nee_light(Sampler& smp, uint32_t& dim, V3<R> P, V3<R> N, V3<R> inDir, V3<R> albedo, R rough, R metal,
                     V3<R> F0, const V3<R>* thr, TravStats* ts) const {
        const bool bounce0 = (thr == nullptr);
        NeeOut out;
        const LightSmp ls = sample_light(smp, dim, P, N);
        const V3<R> L = ls.L, Le = ls.Le;
        const R NdotL = ls.NdotL, weight = ls.weight;
        const R n = ls.n;
        if (ls.valid) {
            Surf<R> sh;
            if (shadow(P + N * R(0.01f), L, ls.shadowDist, sh, ts)) {
                V3<R> V = normalize(-inDir);
                V3<R> H = normalize(L + V);
                R NdotH = gmax(dot(N, H), R(0.001f));
                R NdotV = gmax(dot(N, V), R(0.001f));
                R VdotH = gmax(dot(V, H), R(0.001f));
                R D;
                if (bounce0) {
                    D = ggxD(N, H, NdotH, rough);
                } else {
                    R a = rough * rough, a2 = a * a;
                    R denom = NdotH * NdotH * (a2 - R(1)) + R(1);
                    D = a2 / (R(3.14159f) * denom * denom + R(0.0001f));
                }
                V3<R> F = F0 + (R(1) - F0) * pow5(R(1) - VdotH);
                R k = (rough + R(1)) * (rough + R(1)) / R(8);
                R G = (NdotL / (NdotL * (R(1) - k) + k)) * (NdotV / (NdotV * (R(1) - k) + k));
                V3<R> spec = D * F * G / (R(4) * NdotV * NdotL + R(0.001f));
                V3<R> kD = (R(1) - F) * (R(1) - metal);
                V3<R> diff = kD * albedo / R(3.14159f);
                out.valid = true;
                if (bounce0) out.contrib = Le * (diff + spec) * NdotL * weight * n;
                else out.contrib = *thr * Le * (diff + spec) * NdotL * weight * n;
                if (ls.mis_pdf > R(0))
                    out.contrib = out.contrib * mis(ls.mis_pdf, bsdf_pdf(inDir, N, F0, rough, metal, NdotL, NdotH, VdotH, D));
            }
        }
        return out;
    }

    // The BSDF pdf of the estimator's env MIS (pt_raygen.rgen:466-479).
    static R bsdf_pdf(V3<R> inDir, V3<R> N, V3<R> F0, R rough, R metal, R NdotL, R NdotH, R VdotH, R D) {
        R cosI = std::fabs(dot(normalize(inDir), N));
        V3<R> fres = F0 + (R(1) - F0) * pow5(R(1) - cosI);
        R sp = maxc(fres) * (R(1) - rough * R(0.9f));
        sp = gmix(sp, R(1), metal);
        R pdfD = NdotL / PI;
        R pdfS = D * NdotH / (R(4) * VdotH + R(1e-4f));
        return gmix(pdfD, pdfS, sp);
    }

    // Emitter MIS, BSDF side: the sphere and area lights the ray crosses
    // before tmax (lights stay transparent), each from its emitting side,
    // weighted against its light-NEE pdf (1 after a delta bounce).
    V3<R> light_hits(V3<R> ro, V3<R> rd, R tmax, bool delta, R lastPdf, R n) const {
        V3<R> sum(R(0));
        for (const Light& Lt : sc.lights) {
            const R ltype = R(Lt.pos_type[3]);
            if (ltype >= R(0.5f) && ltype < R(2.5f)) continue;
            V3<R> lc(R(Lt.pos_type[0]), R(Lt.pos_type[1]), R(Lt.pos_type[2]));
            R r = gmax(R(Lt.dir_param[3]), R(0.01f));
            R area = R(4) * R(3.14159f) * r * r;
            V3<R> Le = V3<R>(R(Lt.col_int[0]), R(Lt.col_int[1]), R(Lt.col_int[2])) * R(Lt.col_int[3]) / gmax(area, R(0.01f));
            R t, lcos, la;
            if (ltype < R(0.5f)) {
                V3<R> oc = ro - lc;
                R b = dot(oc, rd);
                R c = dot(oc, oc) - r * r;
                R disc = b * b - c;
                if (!(disc >= R(0))) continue;
                t = -b - m_sqrt(disc);
                if (!(t > R(0.001f) && t < tmax)) continue;
                V3<R> ln = normalize(ro + rd * t - lc);
                lcos = dot(-rd, ln);
                la = R(4) * R(3.14159f) * r * r;
            } else {
                V3<R> e1(R(Lt.extra[0]), R(Lt.extra[1]), R(Lt.extra[2]));
                V3<R> e2(R(Lt.extra2[0]), R(Lt.extra2[1]), R(Lt.extra2[2]));
                V3<R> nn = cross(e1, e2);
                V3<R> ln = normalize(nn);
                lcos = dot(-rd, ln);
                if (!(lcos > R(0))) continue;
                t = dot(lc - ro, ln) / -lcos;
                if (!(t > R(0.001f) && t < tmax)) continue;
                V3<R> rel = ro + rd * t - lc;
                R inv = R(1) / dot(nn, nn);
                R a = dot(cross(rel, e2), nn) * inv;
                R bb = dot(cross(e1, rel), nn) * inv;
                if (!(a >= R(0) && a <= R(1) && bb >= R(0) && bb <= R(1))) continue;
                la = R(Lt.extra2[3]);
            }
            if (!(lcos > R(0))) continue;
            R w = R(1);
            if (!delta) w = mis(lastPdf, (t * t) / (lcos * la * n));
            sum = sum + Le * w;
        }
        return sum;
    }

    // Emitter MIS, BSDF side: the light-NEE pdf of a hit on an emissive-table
    // triangle (0 for any other).
    R emis_pdf_at(uint32_t inst, uint32_t gtri, V3<R> rd, R t, R n) const {
        const int64_t e = sc.emis_entry(inst, gtri);
        if (e < 0) return R(0);
        const auto& E = sc.emis[static_cast<size_t>(e)];
        if (!(E.pdf_area > 0.0f)) return R(0);
        V3<R> ng = normalize(cross(V3<R>(R(E.e1[0]), R(E.e1[1]), R(E.e1[2])), V3<R>(R(E.e2[0]), R(E.e2[1]), R(E.e2[2]))));
        R lcos = std::fabs(dot(rd, ng));
        return R(E.pdf_area) * (t * t) / (lcos * n);
    }

    // Env NEE with balance MIS (pt_raygen.rgen:438-500, 708-763, 1016-1071).
    NeeOut nee_env(Sampler& smp, uint32_t& dim, V3<R> P, V3<R> N, V3<R> inDir, V3<R> albedo, R rough, R metal,
                   V3<R> F0, const V3<R>* thr, TravStats* ts) const {
        const bool bounce0 = (thr == nullptr);
        NeeOut out;
        R u1 = R(smp.s1(dim)), u2 = R(smp.s1(dim + 1)); dim += 2;
        V3<R> envDir; R envPdf;
        sample_env(u1, u2, envDir, envPdf);
        R NdotL = gmax(dot(N, envDir), R(0));
        if (NdotL > R(0) && envPdf > R(0)) {
            Surf<R> sh;
            if (shadow(P + N * R(0.01f), envDir, R(10000), sh, ts)) {
                V3<R> envRad = sh.color;
                V3<R> V = normalize(-inDir);
                V3<R> H = normalize(envDir + V);
                R NdotH = gmax(dot(N, H), R(0.001f));
                R NdotV = gmax(dot(N, V), R(0.001f));
                R VdotH = gmax(dot(V, H), R(0.001f));
                R D;
                if (bounce0) {
                    D = ggxD(N, H, NdotH, rough);
                } else {
                    R a = rough * rough, a2 = a * a;
                    R denom = NdotH * NdotH * (a2 - R(1)) + R(1);
                    D = a2 / (PI * denom * denom + R(0.0001f));
                }
                V3<R> F = F0 + (R(1) - F0) * pow5(R(1) - VdotH);
                R k = (rough + R(1)) * (rough + R(1)) / R(8);
                R G = (NdotL / (NdotL * (R(1) - k) + k)) * (NdotV / (NdotV * (R(1) - k) + k));
                V3<R> spec = D * F * G / (R(4) * NdotV * NdotL + R(0.001f));
                V3<R> kD = (R(1) - F) * (R(1) - metal);
                V3<R> diff = kD * albedo / PI;
                V3<R> brdf = diff + spec;
                R cosI = std::fabs(dot(normalize(inDir), N));
                V3<R> fres = F0 + (R(1) - F0) * pow5(R(1) - cosI);
                R sp = maxc(fres) * (R(1) - rough * R(0.9f));
                sp = gmix(sp, R(1), metal);
                R pdfD = NdotL / PI;
                R pdfS = D * NdotH / (R(4) * VdotH + R(1e-4f));
                R bsdfPdf = gmix(pdfD, pdfS, sp);
                R w = mis(envPdf, bsdfPdf);
                out.valid = true;
                if (bounce0) out.contrib = envRad * brdf * NdotL * w / envPdf;
                else out.contrib = *thr * envRad * brdf * NdotL * w / envPdf;
            }
        }
        return out;
    }

    // GGX visible-normal sampling and its Smith terms (ggx_aniso.glsl:56-133,
    // Heitz 2018), alpha = roughness^2; inversesqrt as 1 / sqrt.
    static R ggx_d_iso(R NdotH, R alpha) {
        R a2 = alpha * alpha;
        R denom = NdotH * NdotH * (a2 - R(1)) + R(1);
        return a2 / (R(3.14159265f) * denom * denom + R(1e-8f));
    }
    static R smith_lambda(R c, R alpha) {
        R c2 = c * c;
        R tan2 = gmax(R(0), R(1) - c2) / gmax(c2, R(1e-8f));
        return R(0.5f) * (R(-1) + m_sqrt(R(1) + alpha * alpha * tan2));
    }
    static R smith_g1(R c, R alpha) { return R(1) / (R(1) + smith_lambda(c, alpha)); }
    static R smith_g2_over_g1(R NdotV, R NdotL, R alpha) {
        R lv = smith_lambda(NdotV, alpha), ll = smith_lambda(NdotL, alpha);
        return (R(1) + lv) / (R(1) + lv + ll + R(1e-8f));
    }
    static V3<R> sample_vndf(V3<R> Ve, R ax, R ay, R u0, R u1) {
        V3<R> Vh = normalize(V3<R>(ax * Ve.x, ay * Ve.y, Ve.z));
        R lensq = Vh.x * Vh.x + Vh.y * Vh.y;
        V3<R> T1 = lensq > R(0) ? V3<R>(-Vh.y, Vh.x, R(0)) * (R(1) / m_sqrt(lensq)) : V3<R>(R(1), R(0), R(0));
        V3<R> T2 = cross(Vh, T1);
        R r = m_sqrt(u0);
        R phi = R(2.0f) * R(3.14159265f) * u1;
        R t1 = r * m_cos(phi);
        R t2 = r * m_sin(phi);
        R s = R(0.5f) * (R(1) + Vh.z);
        t2 = (R(1) - s) * m_sqrt(gmax(R(0), R(1) - t1 * t1)) + s * t2;
        V3<R> Nh = T1 * t1 + T2 * t2 + Vh * m_sqrt(gmax(R(0), R(1) - t1 * t1 - t2 * t2));
        return normalize(V3<R>(ax * Nh.x, ay * Nh.y, gmax(R(0), Nh.z)));
    }

    // Specular-lobe "jitter" sample (pt_raygen.rgen:516-525, 784-793).
    V3<R> spec_dir(Sampler& smp, uint32_t& dim, V3<R> inDir, V3<R> N, R rough) const {
        V3<R> refl = reflect(inDir, N);
        if (rough > R(0.01f)) {
            R j0 = R(smp.s1(dim)), j1 = R(smp.s1(dim + 1)); dim += 2;
            V3<R> jit = cos_hemi(refl, j0, j1) * rough;
            refl = normalize(refl + jit);
            if (dot(refl, N) < R(0)) {
                R f0 = R(smp.s1(dim)), f1 = R(smp.s1(dim + 1)); dim += 2;
                refl = cos_hemi(N, f0, f1);
            }
        }
        return refl;
    }

    // One chain (stage B when spec, stage C otherwise), bounces 1..maxBounces.
    void chain(Sampler& smp, uint32_t& dim, bool specChain, V3<R> ro, V3<R> rd, V3<R> thr, R lastPdf, bool lastDelta,
               V3<R>& radiance, TravStats* ts) const {
        const bool useEnvMis = sc.has_cdf;   // pc.control.w > 0 && pc.tuning.y > 0
        const uint32_t nsel = light_choices();
        for (uint32_t bounce = 1; bounce <= st.max_bounces; ++bounce) {
            Surf<R> s;
            trace(ro, rd, s, ts);
            if (emitter_mis())
                radiance = radiance + thr * light_hits(ro, rd, s.hit ? s.dist : R(10000), lastDelta, lastPdf, R(float(nsel)));
            if (!s.hit) {
                R w = R(1);
                if (s.envPdf > R(0) && useEnvMis && !lastDelta) w = mis(lastPdf, s.envPdf);
                radiance = radiance + thr * s.color * w;
                break;
            }
            V3<R> bP = s.hitPos, bN = s.N, bAlb = s.albedo, bE = s.color;
            if (length(bE) > R(0.001f)) {
                if (emitter_mis()) {
                    R w = R(1);
                    if (!sc.emis.empty() && !lastDelta) {
                        const R pdf = emis_pdf_at(s.inst, s.gtri, rd, s.dist, R(float(nsel)));
                        if (pdf > R(0)) w = mis(lastPdf, pdf);
                    }
                    radiance = radiance + thr * bE * w;
                } else {
                    radiance = radiance + thr * bE;
                }
            }
            R bR = s.rough, bM = s.metal;
            V3<R> bF0 = vmix(V3<R>(R(0.04f)), bAlb, bM);
            if (nsel > 0) {
                NeeOut o = nee_light(smp, dim, bP, bN, rd, bAlb, bR, bM, bF0, &thr, ts);
                if (o.valid) radiance = radiance + clampc(o.contrib);
            }
            if (useEnvMis) {
                NeeOut o = nee_env(smp, dim, bP, bN, rd, bAlb, bR, bM, bF0, &thr, ts);
                if (o.valid) radiance = radiance + clampc(o.contrib);
            }
            if (bounce > 1) {   // Russian roulette (766-771)
                R p = maxc(thr);
                R rr = R(smp.s1(dim)); dim += 1;
                if (p < R(0.01f) || rr > p) break;
                thr = thr / p;
            }
            R cosI = std::fabs(dot(normalize(rd), bN));
            V3<R> fres = bF0 + (R(1) - bF0) * pow5(R(1) - cosI);
            R sp = maxc(fres);
            sp = sp * (R(1) - bR * R(0.9f));
            sp = gmix(sp, R(1), bM);
            R choice = R(smp.s1(dim)); dim += 1;
            if (choice < sp || bR < R(0.05f)) {
                V3<R> inDir = rd;
                rd = spec_dir(smp, dim, rd, bN, bR);
                ro = bP + bN * R(0.01f);
                if (specChain) thr = thr * vmix(V3<R>(R(1)), bAlb, bM);
                else thr = thr * (bAlb * (R(1) - bM));
                thr = thr / gmax(sp, R(0.01f));
                if (bR < R(0.05f)) {
                    lastPdf = R(1); lastDelta = true;
                } else {
                    V3<R> Hs = normalize(-inDir + rd);
                    R NdotHs = gmax(dot(bN, Hs), R(0.001f));
                    R VdotHs = gmax(dot(-inDir, Hs), R(0.001f));
                    R as = bR * bR, as2 = as * as;
                    R dg = NdotHs * NdotHs * (as2 - R(1)) + R(1);
                    R Ds = as2 / (PI * dg * dg + R(1e-4f));
                    R pdfS = Ds * NdotHs / (R(4) * VdotHs + R(1e-4f));
                    lastPdf = sp * pdfS;
                    lastDelta = false;
                }
            } else {
                R d0 = R(smp.s1(dim)), d1 = R(smp.s1(dim + 1)); dim += 2;
                rd = cos_hemi(bN, d0, d1);
                ro = bP + bN * R(0.01f);
                thr = thr * bAlb;
                thr = thr / gmax(R(1) - sp, R(0.01f));
                lastPdf = (R(1) - sp) * gmax(dot(rd, bN), R(0)) / PI;
                lastDelta = false;
            }
        }
    }

    // Jittered camera ray direction (pt_raygen.rgen:138-163); origin = camera.
    V3<R> camera_dir(const View& vw, uint32_t px, uint32_t py, Sampler& smp, uint32_t& dim) const {
        R jx = R(smp.s1(dim)) - R(0.5f), jy = R(smp.s1(dim + 1)) - R(0.5f);
        dim += 2;
        R uvx = (R(float(px)) + R(0.5f) + jx + R(st.pix_jitter[0])) / R(float(vw.width));
        R uvy = (R(float(py)) + R(0.5f) + jy + R(st.pix_jitter[1])) / R(float(vw.height));
        R ndcx = uvx * R(2) - R(1), ndcy = uvy * R(2) - R(1);
        const float* iv = vw.inv_view;
        V3<R> fwd = -V3<R>(R(iv[8]), R(iv[9]), R(iv[10]));
        V3<R> right{R(iv[0]), R(iv[1]), R(iv[2])};
        V3<R> up{R(iv[4]), R(iv[5]), R(iv[6])};
        R aspect = R(float(vw.width)) / R(float(vw.height));
        R tanY = std::fabs(R(vw.inv_proj[5]));
        R tanX = tanY * aspect;
        return normalize(fwd + right * ndcx * tanX - up * ndcy * tanY);
    }

    // pt_raygen.rgen main(): one path sample; returns the clamped radiance.
    V3<R> path(const View& vw, uint32_t px, uint32_t py, uint32_t sampleIdx, TravStats* ts = nullptr,
               Surf<R>* first = nullptr) const {
        Sampler smp;
        smp.init(st.sampler, px, py, sampleIdx);
        uint32_t dim = 0;
        R jx = R(smp.s1(dim)) - R(0.5f), jy = R(smp.s1(dim + 1)) - R(0.5f);
        dim += 2;
        R uvx = (R(float(px)) + R(0.5f) + jx + R(st.pix_jitter[0])) / R(float(vw.width));
        R uvy = (R(float(py)) + R(0.5f) + jy + R(st.pix_jitter[1])) / R(float(vw.height));
        R ndcx = uvx * R(2) - R(1), ndcy = uvy * R(2) - R(1);
        const float* iv = vw.inv_view;
        V3<R> camPos{R(iv[12]), R(iv[13]), R(iv[14])};
        V3<R> fwd = -V3<R>(R(iv[8]), R(iv[9]), R(iv[10]));
        V3<R> right{R(iv[0]), R(iv[1]), R(iv[2])};
        V3<R> up{R(iv[4]), R(iv[5]), R(iv[6])};
        R aspect = R(float(vw.width)) / R(float(vw.height));
        R tanY = std::fabs(R(vw.inv_proj[5]));
        R tanX = tanY * aspect;
        V3<R> rayDir = normalize(fwd + right * ndcx * tanX - up * ndcy * tanY);
        V3<R> rayOrg = camPos;
        V3<R> radiance(R(0));
        Surf<R> s;
        trace(rayOrg, rayDir, s, ts);
        if (first) *first = s;
        if (!s.hit) {
            radiance = s.color;
        } else {
            V3<R> P = s.hitPos, N = s.N, alb = s.albedo, em = s.color;
            R rough = s.rough, metal = s.metal;
            V3<R> F0 = vmix(V3<R>(R(0.04f)), alb, metal);
            if (length(em) > R(0.001f)) radiance = radiance + em;
            if (light_choices() > 0) {
                NeeOut o = nee_light(smp, dim, P, N, rayDir, alb, rough, metal, F0, nullptr, ts);
                if (o.valid) radiance = radiance + clampc(o.contrib);
            }
            if (sc.has_cdf) {
                NeeOut o = nee_env(smp, dim, P, N, rayDir, alb, rough, metal, F0, nullptr, ts);
                if (o.valid) radiance = radiance + clampc(o.contrib);
            }
            // Stage B init (505-543)
            V3<R> specDir, specThr;
            R specPdf;
            bool specDelta;
            {
                R cosI = std::fabs(dot(normalize(rayDir), N));
                V3<R> fres = F0 + (R(1) - F0) * pow5(R(1) - cosI);
                R sp = maxc(fres) * (R(1) - rough * R(0.9f));
                sp = gmix(sp, R(1), metal);
                (void)sp;
                V3<R> inDir = rayDir;
                if (st.flags & kFlagVndf) {
                    // VNDF mode (pt_raygen_realtime.rgen:723-800)
                    V3<R> V = normalize(-inDir);
                    R NdotV = gmax(dot(N, V), R(1e-4f));
                    R alpha = rough * rough;
                    if (rough < R(0.02f)) {
                        specDir = reflect(inDir, N);
                        specThr = F0 + (R(1) - F0) * pow5(R(1) - NdotV);
                        specPdf = R(1); specDelta = true;
                    } else {
                        V3<R> up = std::fabs(N.y) < R(0.999f) ? V3<R>(R(0), R(1), R(0)) : V3<R>(R(1), R(0), R(0));
                        V3<R> T = normalize(cross(up, N));
                        V3<R> B = cross(N, T);
                        V3<R> Vloc(dot(V, T), dot(V, B), dot(V, N));
                        R u0 = R(smp.s1(dim)), u1 = R(smp.s1(dim + 1)); dim += 2;
                        V3<R> Hloc = sample_vndf(Vloc, alpha, alpha, u0, u1);
                        V3<R> H = normalize(T * Hloc.x + B * Hloc.y + N * Hloc.z);
                        V3<R> refl = reflect(-V, H);
                        if (dot(refl, N) <= R(0)) { refl = reflect(inDir, N); H = N; }
                        refl = normalize(refl);
                        specDir = refl;
                        R NdotL = gmax(dot(N, refl), R(1e-4f));
                        R NdotH = gmax(dot(N, H), R(1e-4f));
                        R VdotH = gmax(dot(V, H), R(1e-4f));
                        V3<R> F = F0 + (R(1) - F0) * pow5(R(1) - VdotH);
                        specThr = F * smith_g2_over_g1(NdotV, NdotL, alpha);
                        R D = ggx_d_iso(NdotH, alpha);
                        R G1V = smith_g1(NdotV, alpha);
                        specPdf = G1V * D / (R(4) * NdotV) + R(1e-6f);
                        specDelta = false;
                    }
                } else {
                    specDir = spec_dir(smp, dim, rayDir, N, rough);
                    specThr = vmix(V3<R>(R(1)), alb, metal);
                    if (rough < R(0.05f)) {
                        specPdf = R(1); specDelta = true;
                    } else {
                        V3<R> Hs = normalize(-inDir + specDir);
                        R NdotHs = gmax(dot(N, Hs), R(0.001f));
                        R VdotHs = gmax(dot(-inDir, Hs), R(0.001f));
                        R Ds = ggxD(N, Hs, NdotHs, rough);
                        specPdf = Ds * NdotHs / (R(4) * VdotHs + R(1e-4f));
                        specDelta = false;
                    }
                }
            }
            chain(smp, dim, true, P + N * R(0.01f), specDir, specThr, specPdf, specDelta, radiance, ts);
            // Stage C init (836-850)
            R d0 = R(smp.s1(dim)), d1 = R(smp.s1(dim + 1)); dim += 2;
            V3<R> diffDir = cos_hemi(N, d0, d1);
            V3<R> diffThr = alb;
            R diffPdf = gmax(dot(diffDir, N), R(0)) / PI;
            chain(smp, dim, false, P + N * R(0.01f), diffDir, diffThr, diffPdf, false, radiance, ts);
        }
        return clampc(radiance);   // firefly clamp on the total (1138-1141)
    }
};

}  // namespace orc
