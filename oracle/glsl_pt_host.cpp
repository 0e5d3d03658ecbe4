// glsl_pt_host.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Host side of the shader pin library: runs the reference's path-tracing
// shaders (compiled as C++, glsl_pt_api.inc) over an oracle scene, tracing
// through the oracle's BVH, and returns per-path radiance in the layout of
// the oracle's own orc_render_paths so the two compare record for record.
#include <cstring>

#include "glsl_pt_iface.h"
#include "oracle_pt.hpp"

using namespace orc;

namespace {

void trace_cb(const void* ctx, const float o[3], const float d[3], float tmin, float tmax, int32_t any_hit,
              GptHit* out) {
    const Scene& sc = *static_cast<const Scene*>(ctx);
    std::memset(out, 0, sizeof *out);
    if (any_hit) {
        out->hit = sc.occluded(o, d, tmin, tmax) ? 1 : 0;
        return;
    }
    const HitRec h = sc.closest(o, d, tmin, tmax);
    if (!h.hit()) return;
    const Instance& in = sc.instances[h.inst];
    out->hit = 1;
    out->t = h.t;
    out->u = h.u;
    out->v = h.v;
    out->custom_index = static_cast<int32_t>(in.custom & 0xFFFFFFu);
    out->primitive = static_cast<int32_t>(h.prim);
    std::memcpy(out->object_to_world, in.xform, sizeof in.xform);
    affine_xform_point(in.w2o, o, out->object_origin);
    affine_xform_dir(in.w2o, d, out->object_direction);
}

// The shader pin's view of an oracle scene: arrays, environment, traversal
// and the bindless textures as RGBA32F texels (c / 255).
struct PinScene {
    GptScene gs;
    std::vector<std::vector<float>> tex;
    std::vector<const float*> tex_ptr;
    std::vector<uint32_t> tex_sizes;
    explicit PinScene(const Scene* s) {
        std::memset(&gs, 0, sizeof gs);
        gs.normals = s->normals.data();
        gs.indices = s->indices.data();
        gs.uvs = s->uvs.data();
        gs.mat_ids = s->mat_ids.data();
        gs.mats = s->mats.data();
        gs.lights = s->lights.empty() ? nullptr : &s->lights[0].pos_type[0];
        gs.nlights = static_cast<uint32_t>(s->lights.size());
        gs.env = s->has_env ? s->env.data() : nullptr;
        gs.env_w = s->env_w;
        gs.env_h = s->env_h;
        gs.marg = s->has_cdf ? s->marg.data() : nullptr;
        gs.cond = s->has_cdf ? s->cond.data() : nullptr;
        gs.env_integral = s->env_integral;
        gs.env_intensity = s->env_intensity;
        gs.has_cdf = s->has_env && s->has_cdf ? 1 : 0;
        gs.trace_ctx = s;
        gs.trace = trace_cb;
        for (const auto& ti : s->tex_info) {
            std::vector<float> t(static_cast<size_t>(ti.w) * ti.h * 4);
            for (size_t i = 0; i < t.size(); ++i) t[i] = float(s->tex_texels[ti.off * 4 + i]) / 255.0f;
            tex.push_back(std::move(t));
            tex_sizes.push_back(static_cast<uint32_t>(ti.w));
            tex_sizes.push_back(static_cast<uint32_t>(ti.h));
        }
        for (const auto& t : tex) tex_ptr.push_back(t.data());
        gs.tex_rgba = tex_ptr.data();
        gs.tex_sizes = tex_sizes.data();
        gs.ntex = static_cast<uint32_t>(tex.size());
    }
};

}  // namespace

// The any-hit shader on n candidate hits (instance index, primitive index,
// u, v as floats bits): out[i] = 1 accepted, 0 ignored.
extern "C" void gpt_anyhit(const Scene* s, const uint32_t* inst, const uint32_t* prim, const float* uv, uint32_t n,
                           uint32_t* out) {
    PinScene ps(s);
    for (uint32_t i = 0; i < n; ++i)
        out[i] = static_cast<uint32_t>(gpt_anyhit_accept(&ps.gs, static_cast<int32_t>(s->instances[inst[i]].custom & 0xFFFFFFu),
                                                         static_cast<int32_t>(prim[i]), uv[2 * i], uv[2 * i + 1]));
}

// settings: max_bounces, sampler, flags, clamp_lum, aniso, aniso_rot (the
// oracle's AbiSettings). out: [spp][npix][3] float radiance.
extern "C" void gpt_render_paths(const Scene* s, const float* inv_view, const float* inv_proj, uint32_t width,
                                 uint32_t height, const uint32_t* settings_u32, uint32_t sample_base, uint32_t spp,
                                 const uint32_t* pix, uint32_t npix, float* out) {
    PinScene ps(s);
    const GptScene& gs = ps.gs;
    GptCamera cam;
    std::memcpy(cam.inv_view, inv_view, 64);
    std::memcpy(cam.inv_proj, inv_proj, 64);
    cam.width = width;
    cam.height = height;
    GptSettings st;
    st.max_bounces = settings_u32[0];
    st.sampler = settings_u32[1];
    st.flags = settings_u32[2];
    std::memcpy(&st.clamp_luminance, &settings_u32[3], 4);
    std::memcpy(&st.aniso_strength, &settings_u32[4], 4);
    std::memcpy(&st.aniso_rotation, &settings_u32[5], 4);
    const uint32_t np = pix ? npix : width * height;
    for (uint32_t k = 0; k < spp; ++k)
        for (uint32_t i = 0; i < np; ++i) {
            const uint32_t p = pix ? pix[i] : i;
            float rgba[4];
            gpt_shade_pixel(&gs, &cam, &st, p % width, p / width, sample_base + k, rgba);
            float* o = out + (static_cast<size_t>(k) * np + i) * 3;
            o[0] = rgba[0];
            o[1] = rgba[1];
            o[2] = rgba[2];
        }
}
