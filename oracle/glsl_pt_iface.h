// glsl_pt_iface.h -- TEST INFRASTRUCTURE ONLY.
//
// Plain-C interface between the two translation units of the shader pin
// library: the reference's path-tracing shaders compiled as C++ (GLSL float
// semantics) and the host side that owns the oracle's scene and traversal
// (ordinary C++ semantics). The hardware traversal behind traceRayEXT is
// closed, so the shaders trace through the oracle's BVH via `trace`.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GptHit {
    int32_t hit;
    float t, u, v;               // hit distance and barycentrics
    int32_t custom_index;        // instance custom index (24 bits)
    int32_t primitive;           // primitive index within the instance's BLAS
    float object_to_world[12];   // row-major 3x4
    float object_origin[3], object_direction[3];
} GptHit;

// any_hit != 0: terminate on the first hit, report only whether one exists
typedef void (*GptTraceFn)(const void* ctx, const float o[3], const float d[3], float tmin, float tmax,
                           int32_t any_hit, GptHit* out);

typedef struct GptScene {
    const float* normals;    // 4 per vertex
    const uint32_t* indices;
    const float* uvs;        // 2 per vertex
    const uint32_t* mat_ids;
    const float* mats;       // 12 per material
    const float* lights;     // 20 floats (80 bytes) per light
    uint32_t nlights;
    const float* env;        // RGBA32F env_w * env_h, or NULL
    uint32_t env_w, env_h;
    const float* marg;
    const float* cond;
    float env_integral, env_intensity;
    int32_t has_cdf;
    const void* trace_ctx;
    GptTraceFn trace;
    // bindless textures as RGBA32F texels (the UNORM8 texels c / 255)
    const float* const* tex_rgba;
    const uint32_t* tex_sizes;   // (width, height) per texture
    uint32_t ntex;
} GptScene;

typedef struct GptCamera {
    float inv_view[16], inv_proj[16];   // column-major
    uint32_t width, height;
} GptCamera;

typedef struct GptSettings {
    uint32_t sampler, max_bounces, flags;
    float clamp_luminance, aniso_strength, aniso_rotation;
} GptSettings;

// One launch of the raygen shader for pixel (px, py) and sample index
// `sample` with no history; rgba = the accumulation image's texel (the
// path's radiance, count 1).
void gpt_shade_pixel(const GptScene* scene, const GptCamera* cam, const GptSettings* st, uint32_t px, uint32_t py,
                     uint32_t sample, float rgba[4]);

// The any-hit shader on one candidate hit (instance custom index, primitive
// index, barycentrics): 1 when it accepts the hit, 0 when it executes
// ignoreIntersectionEXT.
int32_t gpt_anyhit_accept(const GptScene* scene, int32_t custom_index, int32_t primitive, float u, float v);

#ifdef __cplusplus
}
#endif
