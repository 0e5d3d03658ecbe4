// pt_types.hpp -- plain-old-data shared by the host context and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/ohao_pt.h"

namespace ohao {

constexpr uint32_t kInstNoOpaque = 1u << 8;   // DInst::mask: the BLAS takes the alpha test

struct DInst {          // per instance, 96 bytes
    float w2o[12];      // world-to-object 3x4, row-major
    float nrm[9];       // transpose(inverse(mat3(object-to-world))), row-major
    uint32_t custom;
    uint32_t blas;
    uint32_t mask;
};
static_assert(sizeof(DInst) == 96, "DInst layout");

struct DBlas {
    uint32_t node_off, tri_off, nnodes, ntris;
};

struct DScene {
    // flat BVH, or the TLAS when two_level
    const uint4* nodes;
    const float4* tris;
    const uint32_t* tlas_inst;
    uint32_t nnodes;
    int two_level;
    const DBlas* blas;
    const uint4* blas_nodes;
    const float4* blas_tris;
    const DInst* inst;
    // shading data
    const uint32_t* indices;
    const float4* normals;
    const float2* uvs;
    const uint32_t* mat_ids;
    const float4* mats;
    const float4* lights;
    uint32_t nlights;
    const float4* env;
    uint32_t env_w, env_h;
    const float* marg;
    const float* cond;
    // guide tables of the inverse-CDF searches (env_guide.hpp), or null:
    // guide_mm + 1 entries for the marginal, guide_mc + 1 per row
    const uint16_t* guide_marg;
    const uint16_t* guide_cond;
    uint32_t guide_mm, guide_mc;
    float env_intensity;
    int has_env, has_cdf;
    const float* albedo_map;
    uint32_t map_w, map_h;
    uint32_t stack_limit;   // traversal stack entries per ray, in [1, 64]
    // bindless textures (RGBA8 UNORM) and their (first texel, width, height, 0)
    const uchar4* tex;
    const uint4* tex_info;
    uint32_t ntex;
    uint32_t alpha_test;    // non-opaque rays: alpha-test kInstNoOpaque instances
    float box_lo[3];        // the scene's bounding box: low corner and 4 / extent per axis
    float box_inv[3];
    // emitter MIS (OHAO_PT_FLAG_EMITTER_MIS; all zero / null otherwise):
    // the emissive triangles are one more choice of the light NEE, sampled
    // by power, and sphere / area lights are found by BSDF rays; both sides
    // weighted by the balance heuristic
    uint32_t emitter_mis;   // the flag is set on this render
    uint32_t nemis;         // emissive-triangle entries (0: none)
    const float4* emis_tri; // 3 per entry: (p0, pdf per area), (p1 - p0, instance bits), (p2 - p0, prim bits)
    const float* emis_cdf;  // nemis entries, non-decreasing, the last 1
    const uint32_t* emis_rank;  // per global triangle: bit 31 emissive, low bits its rank among the emissive ones
    const uint2* emis_inst;     // per instance: (first entry or 0xFFFFFFFF, rank of its first triangle)
};

struct PathParams {
    uint32_t max_bounces;
    uint32_t sampler;
    uint32_t flags;
    float clamp_lum;
    float aniso, aniso_rot;
    uint32_t sample_base;
    uint32_t refill;        // per-view wavefront traversal: 0 one ray per thread, 1..32 persistent warps
};

struct ViewParams {
    float inv_view[16];
    float inv_proj[16];
    uint32_t width, height;
    uint32_t pix_base;   // per-view wavefront: first pixel rank of the range a wave lane renders (0: the view)
    uint32_t pad;
};

struct RenderView {
    ViewParams vp;
    float* accum;        // device RGBA32F
    uint32_t history;
    float* path_out;     // device [spp][npix][4] or null
    float* aov;          // device [npix][OHAO_PT_AOV_FLOATS] or null
    // recorded when `accum` holds its history (an upload still in flight on
    // another stream): the render waits for it before it first reads the
    // accumulator; null = already there
    cudaEvent_t accum_ready;
};

struct ProfileAcc {
    float extend_ms = 0, shadow_ms = 0, shade_ms = 0, other_ms = 0, total_ms = 0;
    uint32_t extend_launches = 0, shadow_launches = 0, shade_launches = 0, other_launches = 0;
    uint64_t rays_closest = 0, rays_shadow = 0;
    uint64_t nodes_closest = 0, tris_closest = 0, nodes_shadow = 0, tris_shadow = 0;
    uint32_t lanes = 1;     // pixel lanes the unprofiled render would run
};

// display.cu: RGBA8 display image of npix RGBA32F texels
cudaError_t launch_display(const float* accum, uint32_t npix, uint8_t* rgba8, cudaStream_t st);

// wavefront.cu
size_t wavefront_scratch_bytes(uint32_t capacity);
uint32_t wavefront_default_capacity();
// Pixel lanes of the per-view wavefront, and its streams besides the
// caller's: lane l renders a slice of the view's pixels on main[l] (lane 0 on
// the caller's stream; main[0] unused), each with capacity / kWaveLanes paths
// of the scratch, and runs each step's shadow rays on aux[l] beside its next
// step's closest-hit rays. Null members: that part runs serially.
constexpr int kWaveLanes = 4;
struct WaveStreams {
    cudaStream_t main[kWaveLanes];
    cudaStream_t aux[kWaveLanes];
};
size_t wavefront_lanes_scratch_bytes(uint32_t capacity);   // kWaveLanes lanes of capacity / kWaveLanes paths
ohao_status wavefront_render(const DScene& sc, const RenderView& view, const PathParams& pp, uint32_t spp,
                             void* scratch, size_t scratch_bytes, uint32_t capacity, cudaStream_t st, bool profile,
                             ProfileAcc* prof, int* d_err, std::string& err, const WaveStreams* ws = nullptr);
ohao_status trace_rays(const DScene& sc, const float* rays, uint32_t n, uint32_t* hits, int any_hit, uint32_t* stats,
                       cudaStream_t st, int* d_err, std::string& err);

// persistent.cu
struct PersistentState;
PersistentState* persistent_create();
void persistent_destroy(PersistentState* s);
uint32_t persistent_max_views();
const char* persistent_variant_name(const PersistentState* s);
const char* persistent_variant_at(uint32_t i);                        // nullptr past the last
bool persistent_select(PersistentState* s, const char* name);         // false: unknown name
// scene_box: 6 floats (lo.xyz, hi.xyz) bounding the scene, for ray reordering
ohao_status persistent_render(PersistentState* s, const DScene& sc, const RenderView* views, uint32_t n,
                              const PathParams& pp, uint32_t spp, const float* scene_box, cudaStream_t st, int* d_err,
                              bool profile, ProfileAcc* prof, std::string& err);
ohao_status persistent_autotune(PersistentState* s, const DScene& sc, const RenderView* views, uint32_t n,
                                const PathParams& pp, uint32_t spp, const float* scene_box, cudaStream_t st, int* d_err,
                                float* best_ms, std::string& err);

// adjoint.cu
uint32_t adjoint_max_bounces();
size_t adjoint_scratch_bytes(uint32_t nviews);
// Mean over views of the per-view RGB MSE between views[v].accum and
// targets[v] (with ldr: between the display transform of views[v].accum and
// display-space targets); writes d loss / d pixel into grads_out[v] (device
// RGBA32F).
ohao_status adjoint_mse(const RenderView* views, const float* const* targets, uint32_t nviews, bool ldr, void* scratch,
                        size_t scratch_bytes, float* const* grads_out, float* loss_out, cudaStream_t st,
                        std::string& err);
// Path-replay gradient: grads[v] = d loss / d pixel of views[v]'s image (the
// mean of spp paths from sample pp.sample_base); overwrites grad_map
// (map_h*map_w*3) and grad_rough (nmats), either may be null.
ohao_status adjoint_backward(const DScene& sc, const RenderView* views, const float* const* grads, uint32_t nviews,
                             const PathParams& pp, uint32_t spp, uint32_t nmats, void* scratch, size_t scratch_bytes,
                             float* grad_map, float* grad_rough, cudaStream_t st, int* d_err, std::string& err);

}  // namespace ohao
