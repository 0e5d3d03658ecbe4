// oracle_capi.cpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// extern "C" surface of the host oracle, loaded by tests/ (ctypes), by the
// smoke check and by bench.py's CPU-baseline leg. Never linked into the
// product library.
#include "oracle_pt.hpp"
#include "oracle_adjoint.hpp"
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {
// Sobol direction numbers for dimensions 0-3 (32 per dimension), the table
// the reference ships in shaders/includes/rt/sampler_sobol_tables.glsl:10-47
// and ohao/render/rt/sobol_generator.cpp (kDirectionNumbers). Dimension 2 is
// not the textbook Joe-Kuo dimension, so the values are data, not derived.
const uint32_t kSobolDirs[128] = {
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
}  // namespace orc

using namespace orc;

struct AbiInstance {   // ohao_pt_instance (include/ohao_pt.h)
    uint32_t blas;
    float xform[12];
    uint32_t custom_index;
    uint32_t mask;
    uint32_t sbt_offset;
};
static_assert(sizeof(AbiInstance) == 64, "instance record is 64 bytes");

extern "C" {

Scene* orc_scene_create() { return new Scene(); }
void orc_scene_destroy(Scene* s) { delete s; }

void orc_scene_set_geometry(Scene* s, const float* pos, uint32_t pos_stride_bytes, uint32_t nverts, const float* normal4,
                            const float* uv2, const uint32_t* idx, uint32_t ntris, const uint32_t* matid) {
    s->pos.resize(static_cast<size_t>(nverts) * 3);
    const uint8_t* pb = reinterpret_cast<const uint8_t*>(pos);
    for (uint32_t i = 0; i < nverts; ++i) std::memcpy(&s->pos[3 * i], pb + static_cast<size_t>(i) * pos_stride_bytes, 12);
    s->normals.assign(normal4, normal4 + static_cast<size_t>(nverts) * 4);
    if (uv2) s->uvs.assign(uv2, uv2 + static_cast<size_t>(nverts) * 2);
    else s->uvs.assign(static_cast<size_t>(nverts) * 2, 0.0f);
    s->indices.assign(idx, idx + static_cast<size_t>(ntris) * 3);
    s->mat_ids.assign(matid, matid + ntris);
}
void orc_scene_set_materials(Scene* s, const float* m, uint32_t n) {
    s->mats.assign(m, m + static_cast<size_t>(n) * 12);
    if (!s->instances.empty()) s->build_emitters();
}
void orc_scene_set_lights(Scene* s, const float* l, uint32_t n) {
    s->lights.resize(n);
    if (n) std::memcpy(s->lights.data(), l, static_cast<size_t>(n) * 80);
}
void orc_scene_set_env(Scene* s, const float* rgba, uint32_t w, uint32_t h, const float* marg, const float* cond,
                       float integral, float intensity) {
    s->has_env = rgba != nullptr && w > 0 && h > 0;
    s->has_cdf = s->has_env && marg != nullptr && cond != nullptr;
    s->env_w = w; s->env_h = h;
    if (s->has_env) s->env.assign(rgba, rgba + static_cast<size_t>(w) * h * 4);
    if (s->has_cdf) {
        s->marg.assign(marg, marg + h);
        s->cond.assign(cond, cond + static_cast<size_t>(w) * h);
    }
    s->env_integral = integral;
    s->env_intensity = intensity;
}
void orc_scene_set_albedo_map(Scene* s, const float* map, uint32_t w, uint32_t h) {
    s->map_w = w; s->map_h = h;
    s->albedo_map.assign(map, map + static_cast<size_t>(w) * h * 3);
}
// n RGBA8 textures: texels back to back, sizes as (width, height) pairs
void orc_scene_set_textures(Scene* s, const uint8_t* texels, const uint32_t* sizes, uint32_t n) {
    s->tex_info.clear();
    size_t off = 0;
    for (uint32_t i = 0; i < n; ++i) {
        s->tex_info.push_back({off, static_cast<int>(sizes[2 * i]), static_cast<int>(sizes[2 * i + 1])});
        off += static_cast<size_t>(sizes[2 * i]) * sizes[2 * i + 1];
    }
    s->tex_texels.assign(texels, texels + off * 4);
}
// pt_anyhit.rahit's alpha test on n candidate hits (instance, primitive, u, v)
void orc_alpha_accept(const Scene* s, const uint32_t* inst, const uint32_t* prim, const float* uv, uint32_t n,
                      uint32_t* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = s->alpha_accept(inst[i], prim[i], uv[2 * i], uv[2 * i + 1]) ? 1u : 0u;
}
void orc_scene_set_blas_flags(Scene* s, uint32_t blas, uint32_t flags) { s->blases[blas].no_opaque = (flags & 1u) != 0; }
uint32_t orc_scene_add_blas(Scene* s, uint32_t first_index, uint32_t index_count) {
    Blas b;
    b.first_index = first_index;
    b.index_count = index_count;
    s->blases.push_back(std::move(b));
    return static_cast<uint32_t>(s->blases.size() - 1);
}
void orc_scene_set_instances(Scene* s, const AbiInstance* in, uint32_t n) {
    s->instances.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        Instance& d = s->instances[i];
        d.blas = in[i].blas;
        std::memcpy(d.xform, in[i].xform, sizeof(d.xform));
        d.custom = in[i].custom_index;
        d.mask = in[i].mask;
    }
}
// force_mode: 0 auto, 1 flat, 2 two-level
void orc_scene_build(Scene* s, uint64_t flatten_limit, int force_mode) { s->build(flatten_limit, force_mode); }
int orc_scene_two_level(const Scene* s) { return s->two_level ? 1 : 0; }

// which = -1: flat BVH (or TLAS when two-level); which = k: BLAS k.
void orc_bvh_sizes(const Scene* s, int which, uint32_t* nnodes, uint32_t* nprims, uint32_t* height) {
    const WideBVH* b;
    size_t np;
    if (which < 0) {
        b = s->two_level ? &s->tlas : &s->flat;
        np = s->two_level ? s->tlas_inst.size() : s->flat_tris.size();
    } else {
        b = &s->blases[which].bvh;
        np = s->blases[which].tris.size();
    }
    *nnodes = static_cast<uint32_t>(b->nodes.size());
    *nprims = static_cast<uint32_t>(np);
    *height = b->height;
}
void orc_bvh_copy(const Scene* s, int which, void* nodes, void* prims) {
    if (which < 0) {
        const WideBVH& b = s->two_level ? s->tlas : s->flat;
        std::memcpy(nodes, b.nodes.data(), b.nodes.size() * sizeof(WideNode));
        if (s->two_level) std::memcpy(prims, s->tlas_inst.data(), s->tlas_inst.size() * 4);
        else std::memcpy(prims, s->flat_tris.data(), s->flat_tris.size() * sizeof(TriRec));
    } else {
        const Blas& bl = s->blases[which];
        std::memcpy(nodes, bl.bvh.nodes.data(), bl.bvh.nodes.size() * sizeof(WideNode));
        std::memcpy(prims, bl.tris.data(), bl.tris.size() * sizeof(TriRec));
    }
}

// rays: n x 8 floats (o.xyz, tmin, d.xyz, tmax). hits: n x 5 u32
// (t bits, u bits, v bits, instance, primitive) -- any-hit mode writes
// hits[5i] = 1 when occluded. mode: 0 closest (BVH), 1 any (BVH),
// 2 closest (brute force). stats (optional): per-ray nodes, tris.
void orc_trace(const Scene* s, const float* rays, uint32_t n, uint32_t* hits, int mode, uint32_t* stats, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
        const float* r = rays + i * 8;
        TravStats st;
        uint32_t* h = hits + i * 5;
        const bool alpha = (mode & 4) != 0;   // non-opaque rays (alpha test)
        const int kind = mode & 3;
        if (kind == 1) {
            bool occ = s->occluded(r, r + 4, r[3], r[7], &st, alpha);
            h[0] = occ ? 1u : 0u; h[1] = h[2] = 0; h[3] = h[4] = 0xFFFFFFFFu;
        } else {
            HitRec hr = (kind == 2) ? s->closest_brute(r, r + 4, r[3], r[7], alpha)
                                    : s->closest(r, r + 4, r[3], r[7], &st, alpha);
            h[0] = f2u(hr.t); h[1] = f2u(hr.u); h[2] = f2u(hr.v); h[3] = hr.inst; h[4] = hr.prim;
            if (!hr.hit()) { h[0] = h[1] = h[2] = 0; h[3] = h[4] = 0xFFFFFFFFu; }
        }
        if (stats) { stats[2 * i] = static_cast<uint32_t>(st.nodes); stats[2 * i + 1] = static_cast<uint32_t>(st.tris); }
    }
}

struct AbiSettings {   // subset of ohao_pt_settings used by the oracle
    uint32_t max_bounces, sampler, flags;
    float clamp_lum, aniso, aniso_rot;
};

static Settings to_settings(const AbiSettings* a) {
    Settings s;
    s.max_bounces = a->max_bounces;
    s.sampler = a->sampler;
    s.flags = a->flags;
    s.clamp_lum = a->clamp_lum;
    s.aniso = a->aniso;
    s.aniso_rot = a->aniso_rot;
    return s;
}

// Per-path radiance for `npix` pixels (pixel ids y*W+x, or all pixels when
// pix == NULL) x `spp` samples (sample index = sample_base + k). out is
// [spp][npix][3] in Real (float when fp64 == 0, double otherwise).
// stats (optional, u64 x 3): nodes, triangles, instances visited.
void orc_render_paths(const Scene* s, const float* inv_view, const float* inv_proj, uint32_t width, uint32_t height,
                      const AbiSettings* as, uint32_t sample_base, uint32_t spp, const uint32_t* pix, uint32_t npix,
                      void* out, int fp64, int nthreads, uint64_t* stats) {
    View vw;
    std::memcpy(vw.inv_view, inv_view, 64);
    std::memcpy(vw.inv_proj, inv_proj, 64);
    vw.width = width; vw.height = height;
    Settings st = to_settings(as);
    const uint32_t np = pix ? npix : width * height;
    const int64_t total = static_cast<int64_t>(np) * spp;
    uint64_t tn = 0, tt = 0, ti = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : tn, tt, ti)
#endif
    for (int64_t k = 0; k < total; ++k) {
        uint32_t smp = static_cast<uint32_t>(k / np), pi = static_cast<uint32_t>(k % np);
        uint32_t p = pix ? pix[pi] : pi;
        uint32_t px = p % width, py = p / width;
        TravStats ts;
        if (fp64) {
            PathTracer<double> pt(*s, st);
            V3<double> r = pt.path(vw, px, py, sample_base + smp, stats ? &ts : nullptr);
            double* o = static_cast<double*>(out) + k * 3;
            o[0] = r.x; o[1] = r.y; o[2] = r.z;
        } else {
            PathTracer<float> pt(*s, st);
            V3<float> r = pt.path(vw, px, py, sample_base + smp, stats ? &ts : nullptr);
            float* o = static_cast<float*>(out) + k * 3;
            o[0] = r.x; o[1] = r.y; o[2] = r.z;
        }
        tn += ts.nodes; tt += ts.tris; ti += ts.insts;
    }
    if (stats) { stats[0] = tn; stats[1] = tt; stats[2] = ti; }
}

// Detached-sampling FP64 radiance (oracle_adjoint.hpp) for `npix` pixels x
// `spp` samples: decisions with the scene's parameters, values with mats_e
// (12 floats per material) and map_e (the tile albedo map, or NULL).
// out is [spp][npix][3] double.
void orc_detached_paths(const Scene* s, const float* inv_view, const float* inv_proj, uint32_t width, uint32_t height,
                        const AbiSettings* as, uint32_t sample_base, uint32_t spp, const uint32_t* pix, uint32_t npix,
                        const float* mats_e, const float* map_e, double* out, int nthreads) {
    View vw;
    std::memcpy(vw.inv_view, inv_view, 64);
    std::memcpy(vw.inv_proj, inv_proj, 64);
    vw.width = width; vw.height = height;
    Settings st = to_settings(as);
    const uint32_t np = pix ? npix : width * height;
    const int64_t total = static_cast<int64_t>(np) * spp;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t k = 0; k < total; ++k) {
        uint32_t smp = static_cast<uint32_t>(k / np), pi = static_cast<uint32_t>(k % np);
        uint32_t p = pix ? pix[pi] : pi;
        DetachedPath dp(*s, st, mats_e, map_e);
        V3<double> r = dp.path(vw, p % width, p / width, sample_base + smp);
        out[k * 3 + 0] = r.x; out[k * 3 + 1] = r.y; out[k * 3 + 2] = r.z;
    }
}

// Analytic FP64 gradient of the detached estimator (DetachedPathT<Dd>) for
// up to kGradSlots selected parameters: grad[j] = sum over pixels p and
// channels c of dLdI[p*3+c] * d(mean of the p's spp paths)_c / d theta_j,
// theta = roughness of materials rough_ids[0..n_rough) then map entries
// (texel*3 + channel) map_ids[0..n_map). Sampling with the scene's
// parameters; values too (theta_e == theta_s). with_score adds the score
// terms of the sampling decisions (the derivative of the expectation);
// without them it is the derivative of the function that the finite
// differences of orc_detached_paths see.
int orc_detached_grad(const Scene* s, const float* inv_view, const float* inv_proj, uint32_t width, uint32_t height,
                      const AbiSettings* as, uint32_t sample_base, uint32_t spp, const double* dLdI,
                      const int32_t* rough_ids, uint32_t n_rough, const int32_t* map_ids, uint32_t n_map,
                      int with_score, double* grad_out, int nthreads) {
    if (n_rough + n_map > static_cast<uint32_t>(kGradSlots)) return -1;
    View vw;
    std::memcpy(vw.inv_view, inv_view, 64);
    std::memcpy(vw.inv_proj, inv_proj, 64);
    vw.width = width; vw.height = height;
    Settings st = to_settings(as);
    const size_t nmat = s->mats.size() / 12;
    std::vector<int32_t> rslot(nmat, -1), mslot(s->albedo_map.size(), -1);
    for (uint32_t j = 0; j < n_rough; ++j) rslot[static_cast<size_t>(rough_ids[j])] = static_cast<int32_t>(j);
    for (uint32_t j = 0; j < n_map; ++j) mslot[static_cast<size_t>(map_ids[j])] = static_cast<int32_t>(n_rough + j);
    const uint32_t np = width * height;
    const int64_t total = static_cast<int64_t>(np) * spp;
    const uint32_t nparam = n_rough + n_map;
    std::vector<double> acc(nparam, 0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        std::vector<double> loc(nparam, 0.0);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t k = 0; k < total; ++k) {
            const uint32_t smp = static_cast<uint32_t>(k / np), p = static_cast<uint32_t>(k % np);
            DetachedPathT<Dd> dp(*s, st, s->mats.data(), s->albedo_map.empty() ? nullptr : s->albedo_map.data());
            dp.rough_slot = rslot.data();
            dp.map_slot = mslot.empty() ? nullptr : mslot.data();
            dp.with_score = with_score != 0;
            const V3<Dd> r = dp.path(vw, p % width, p / width, sample_base + smp);
            const double* g = dLdI + static_cast<size_t>(p) * 3;
            for (uint32_t j = 0; j < nparam; ++j) loc[j] += (g[0] * r.x.d[j] + g[1] * r.y.d[j] + g[2] * r.z.d[j]) / spp;
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        for (uint32_t j = 0; j < nparam; ++j) acc[j] += loc[j];
    }
    for (uint32_t j = 0; j < nparam; ++j) grad_out[j] = acc[j];
    return 0;
}

// Progressive own-pixel accumulation of per-path radiance in sample order
// (pt_raygen.rgen:1144-1186 with reprojection off): accum is RGBA32F
// (mean, count) per pixel, updated in place; history = frames already in it.
void orc_accumulate(const float* paths, uint32_t npix, uint32_t spp, float* accum, uint32_t history) {
    for (uint32_t p = 0; p < npix; ++p) {
        float* a = accum + 4 * static_cast<size_t>(p);
        for (uint32_t k = 0; k < spp; ++k) {
            const float* L = paths + (static_cast<size_t>(k) * npix + p) * 3;
            if (history + k == 0) {
                a[0] = L[0]; a[1] = L[1]; a[2] = L[2]; a[3] = 1.0f;
            } else {
                float cnt = a[3] + 1.0f;
                a[0] = (a[0] * a[3] + L[0]) / cnt;
                a[1] = (a[1] * a[3] + L[1]) / cnt;
                a[2] = (a[2] * a[3] + L[2]) / cnt;
                a[3] = cnt;
            }
        }
    }
}

// EnvCDF::build restated (env_cdf.cpp:13-61): serial float sums.
void orc_env_cdf_build(const float* px, int w, int h, float* marg, float* cond, float* integral) {
    std::vector<float> rowSum(h, 0.0f);
    const float kPi = 3.14159265358979323846f;
    for (int y = 0; y < h; ++y) {
        float theta = kPi * (float(y) + 0.5f) / float(h);
        float sinT = std::sin(theta);
        float acc = 0.0f;
        for (int x = 0; x < w; ++x) {
            const float* p = px + (static_cast<size_t>(y) * w + x) * 4;
            float lw = (0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2]) * sinT;
            acc += lw;
            cond[static_cast<size_t>(y) * w + x] = acc;
        }
        if (acc > 0.0f) {
            for (int x = 0; x < w; ++x) cond[static_cast<size_t>(y) * w + x] /= acc;
        } else {
            for (int x = 0; x < w; ++x) cond[static_cast<size_t>(y) * w + x] = float(x + 1) / float(w);
        }
        rowSum[y] = acc;
    }
    float total = 0.0f;
    for (int y = 0; y < h; ++y) { total += rowSum[y]; marg[y] = total; }
    *integral = total;
    if (total > 0.0f) for (int y = 0; y < h; ++y) marg[y] /= total;
    else for (int y = 0; y < h; ++y) marg[y] = float(y + 1) / float(h);
}

float orc_sobol_sample1d(uint32_t index, uint32_t dim) {   // SobolGenerator::sample1D
    return static_cast<float>(sobol_int(index, dim) >> 8) * (1.0f / 16777216.0f);
}
uint32_t orc_owen_scramble(uint32_t v, uint32_t seed) { return owen_scramble(v, seed); }
// getSample1D for pixel/sample, dims 0..n-1 (sampler 0 = PCG, 1 = Sobol)
void orc_sampler_stream(uint32_t type, uint32_t px, uint32_t py, uint32_t sample, uint32_t n, float* out) {
    Sampler s;
    s.init(type, px, py, sample);
    for (uint32_t d = 0; d < n; ++d) out[d] = s.s1(d);
}
// op: 0 sin, 1 cos, 2 atan2(y=in[2i], x=in[2i+1]), 3 asin, 4 acos
void orc_math(int op, const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        switch (op) {
            case 0: out[i] = sin_f(in[i]); break;
            case 1: out[i] = cos_f(in[i]); break;
            case 2: out[i] = atan2_f(in[2 * i], in[2 * i + 1]); break;
            case 3: out[i] = asin_f(in[i]); break;
            default: out[i] = acos_f(in[i]); break;
        }
    }
}
// The oracle's restatement of the reference's GLSL helpers, record for
// record as gref_helper / gref_env in glsl_ref_api.inc (same function ids
// and layouts), for the pin tests.
int orc_glsl_helper(int fn, const float* in, uint32_t n, float* out) {
    static constexpr int kIn[9] = {3, 2, 10, 2, 2, 2, 3, 7, 3};
    static constexpr int kOut[9] = {10, 1, 1, 1, 1, 1, 1, 3, 2};
    using PT = PathTracer<float>;
    using V = V3<float>;
    if (fn < 0 || fn > 8) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + static_cast<size_t>(i) * kIn[fn];
        float* o = out + static_cast<size_t>(i) * kOut[fn];
        switch (fn) {
            case 0: {
                Sampler s;
                s.init(kSamplerPCG, uint32_t(a[0]), uint32_t(a[1]), uint32_t(a[2]));
                for (uint32_t d = 0; d < 10; ++d) o[d] = s.s1(d);
                break;
            }
            case 1: o[0] = PT::mis(a[0], a[1]); break;
            case 2: {
                Scene sc;
                Settings st;
                st.aniso = a[8];
                st.aniso_rot = a[9];
                PT pt(sc, st);
                o[0] = pt.ggxD(V(a[0], a[1], a[2]), V(a[3], a[4], a[5]), a[6], a[7]);
                break;
            }
            case 3: o[0] = PT::ggx_d_iso(a[0], a[1]); break;
            case 4: o[0] = PT::smith_lambda(a[0], a[1]); break;
            case 5: o[0] = PT::smith_g1(a[0], a[1]); break;
            case 6: o[0] = PT::smith_g2_over_g1(a[0], a[1], a[2]); break;
            case 7: {
                const V h = PT::sample_vndf(V(a[0], a[1], a[2]), a[3], a[4], a[5], a[6]);
                o[0] = h.x;
                o[1] = h.y;
                o[2] = h.z;
                break;
            }
            default: PT::unpack_hit_pbr(V(a[0], a[1], a[2]), o[0], o[1]); break;
        }
    }
    return 0;
}
int orc_glsl_env(int fn, const float* marg, const float* cond, uint32_t w, uint32_t h, const float* in, uint32_t n,
                 float* out) {
    static constexpr int kIn[4] = {1, 2, 2, 3};
    static constexpr int kOut[4] = {1, 1, 4, 1};
    if (fn < 0 || fn > 3 || !marg || !cond || w == 0 || h == 0) return -1;
    Scene sc;
    sc.env_w = w;
    sc.env_h = h;
    sc.marg.assign(marg, marg + h);
    sc.cond.assign(cond, cond + static_cast<size_t>(w) * h);
    sc.has_env = sc.has_cdf = true;
    Settings st;
    PathTracer<float> pt(sc, st);
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + static_cast<size_t>(i) * kIn[fn];
        float* o = out + static_cast<size_t>(i) * kOut[fn];
        switch (fn) {
            case 0: o[0] = float(pt.search_marg(a[0])); break;
            case 1: o[0] = float(pt.search_cond(uint32_t(a[0]) * w, a[1])); break;
            case 2: {
                V3<float> dir;
                float pdf;
                pt.sample_env(a[0], a[1], dir, pdf);
                o[0] = dir.x;
                o[1] = dir.y;
                o[2] = dir.z;
                o[3] = pdf;
                break;
            }
            default: o[0] = pt.pdf_env(V3<float>(a[0], a[1], a[2])); break;
        }
    }
    return 0;
}
// The reference's display transform to RGBA8 (pt_raygen.rgen:99-102,
// 1262-1269): per channel pow(ACES(x * 0.5), 1/2.2) stored to UNORM8 with
// round to nearest, alpha 255. The byte is the number of thresholds
// ((k + 0.5) / 255)^2.2 (k = 0..254, double pow rounded to float) that
// ACES(x * 0.5) reaches, which is that rounding without a float pow.
void orc_display_rgba8(const float* rgba, uint64_t npix, uint8_t* out) {
    float thr[255];
    for (int k = 0; k < 255; ++k) thr[k] = static_cast<float>(std::pow((k + 0.5) / 255.0, 2.2));
    for (uint64_t i = 0; i < npix; ++i) {
        for (int c = 0; c < 3; ++c) {
            const float x = rgba[4 * i + c] * 0.5f;
            const float y = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
            const float cl = std::min(std::max(y, 0.0f), 1.0f);
            const float v = (y != y) ? 0.0f : cl;   // NaN -> 0
            int b = 0;
            while (b < 255 && v >= thr[b]) ++b;
            out[4 * i + c] = static_cast<uint8_t>(b);
        }
        out[4 * i + 3] = 255;
    }
}

void orc_pow_def(const float* x, uint64_t n, float y, float* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = pow_def(x[i], y);
}

// Emitter-MIS table: returns the entry count; when tri / cdf are non-null
// writes 12 floats per entry (p0, pdf_area, p1 - p0, instance bits,
// p2 - p0, prim bits) and the CDF.
uint32_t orc_emitter_table(const Scene* s, float* tri, float* cdf) {
    const size_t n = s->emis.size();
    for (size_t i = 0; tri && i < n; ++i) {
        const auto& E = s->emis[i];
        float* o = tri + 12 * i;
        for (int a = 0; a < 3; ++a) { o[a] = E.p0[a]; o[4 + a] = E.e1[a]; o[8 + a] = E.e2[a]; }
        o[3] = E.pdf_area;
        std::memcpy(o + 7, &E.inst, 4);
        std::memcpy(o + 11, &E.prim, 4);
    }
    if (cdf && n) std::memcpy(cdf, s->emis_cdf.data(), n * 4);
    return static_cast<uint32_t>(n);
}

// n light-NEE draws at P (shading normal N) under settings flags, draw k
// from the PCG stream of pixel (k, 0), sample `seed`. Per draw 15 floats:
// L (3), Le (3), weight, choices, mis_pdf, valid, then the BSDF side of
// emitter MIS for a ray from P along L: the emissive-table pdf at its
// closest hit (0 when it hits no table triangle), and the weighted radiance
// of the sphere / area lights it crosses with a BSDF pdf of 1 (3), and
// the distance of that closest hit (-1: none).
void orc_light_samples(const Scene* s, uint32_t flags, const float* P, const float* N, uint32_t n, uint32_t seed,
                       float* out) {
    Settings st;
    st.flags = flags;
    PathTracer<float> pt(*s, st);
    const V3<float> p(P[0], P[1], P[2]), nn(N[0], N[1], N[2]);
    const float nsel = float(pt.light_choices());
    for (uint32_t k = 0; k < n; ++k) {
        Sampler smp;
        smp.init(kSamplerPCG, k, 0, seed);
        uint32_t dim = 0;
        const auto ls = pt.sample_light(smp, dim, p, nn);
        float* o = out + static_cast<size_t>(k) * 15;
        o[0] = ls.L.x; o[1] = ls.L.y; o[2] = ls.L.z;
        o[3] = ls.Le.x; o[4] = ls.Le.y; o[5] = ls.Le.z;
        o[6] = ls.weight; o[7] = ls.n; o[8] = ls.mis_pdf; o[9] = ls.valid ? 1.0f : 0.0f;
        o[10] = 0.0f;
        const float of[3] = {P[0], P[1], P[2]}, df[3] = {ls.L.x, ls.L.y, ls.L.z};
        const HitRec h = s->closest(of, df, 0.001f, 10000.0f);
        if (h.hit()) {
            const uint32_t gtri = (s->instances[h.inst].custom & 0xFFFFFFu) + h.prim;
            o[10] = pt.emis_pdf_at(h.inst, gtri, ls.L, h.t, nsel);
        }
        const V3<float> lh = pt.light_hits(p, ls.L, h.hit() ? h.t : 10000.0f, false, 1.0f, nsel);
        o[11] = lh.x; o[12] = lh.y; o[13] = lh.z;
        o[14] = h.hit() ? h.t : -1.0f;
    }
}

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
