/*
 * ohao_pt.h -- C ABI of the GB300 path-tracing hot path.
 *
 * Drop-in for the Vulkan path-tracing pass of OHAO (Qervas/ohao_engine): the
 * calls below take the same scene, material, light, environment and TLAS/BLAS
 * data the reference binds to its RT pipeline, and replace
 *   - the driver BLAS/TLAS build behind RTAccelerationStructure
 *     (ohao/render/rt/rt_acceleration_structure.hpp:73-107),
 *   - the inputs PathTracer binds (ohao/render/rt/path_tracer.hpp:124-194),
 *   - PathTracer::render -> vkCmdTraceRaysKHR
 *     (ohao/render/rt/path_tracer_render.cpp:687-731) and the GLSL programs
 *     shaders/rt/pt_raygen.rgen, pt_closesthit.rchit, pt_miss.rmiss.
 * Plain C: pointers, sizes and status codes; no exception crosses the ABI.
 * A context is externally synchronised (one thread at a time), like the
 * reference's single command buffer. Unless a parameter says "device", every
 * pointer is host memory and is copied before the call returns.
 */
#ifndef OHAO_PT_H
#define OHAO_PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t ohao_status;
#define OHAO_OK 0
#define OHAO_ERR_INVALID_ARG (-1)
#define OHAO_ERR_OOM (-2)
#define OHAO_ERR_CUDA (-3)
#define OHAO_ERR_TIMEOUT (-4)      /* a bounded device-side wait gave up */
#define OHAO_ERR_NOT_BUILT (-5)    /* render/trace before ohao_pt_build */
#define OHAO_ERR_UNSUPPORTED (-6)
#define OHAO_ERR_DEVICE_CHECK (-7) /* a device-side bounds/stack check fired */
#define OHAO_ERR_TOO_LARGE (-8)    /* input beyond the fixed capacity of ohao_bvh_build_noalloc */

/* Same object as cudaStream_t (struct CUstream_st*); NULL = legacy stream. */
typedef struct CUstream_st* ohao_stream;

typedef struct ohao_pt_ctx ohao_pt_ctx;

typedef struct ohao_pt_desc {
    int32_t device;          /* CUDA device ordinal */
    uint32_t flags;          /* reserved, 0 */
    uint64_t flatten_limit;  /* instanced triangles up to which one flat BVH is
                                built over world-space triangles; above it a
                                two-level TLAS/BLAS is built. 0 = 2^25 */
} ohao_pt_desc;

/* GPULight, ohao/render/rt/gpu_light.hpp:10-16 (80 bytes, std430). */
typedef struct ohao_gpu_light {
    float position_type[4];    /* xyz position, w type (0 sphere,1 dir,2 spot,3 area) */
    float color_intensity[4];
    float dir_param[4];        /* xyz direction, w radius / inner angle */
    float extra[4];            /* spot: w outer angle; area: xyz edge1 */
    float extra2[4];           /* area: xyz edge2, w area */
} ohao_gpu_light;

/* RTInstance, rt_acceleration_structure.hpp:41-47; transform is the row-major
 * 3x4 VkTransformMatrixKHR of buildTLAS (rt_acceleration_structure.cpp:437-445).
 * custom_index is gl_InstanceCustomIndexEXT (24 bits): OHAO sets it to the
 * global triangle offset, so globalTriID = custom_index + primitiveID. */
typedef struct ohao_pt_instance {
    uint32_t blas;
    float transform[12];
    uint32_t custom_index;
    uint32_t mask;             /* instance skipped when (mask & 0xFF) == 0 */
    uint32_t sbt_offset;       /* unused (one hit group) */
} ohao_pt_instance;

#define OHAO_PT_AOV_FLOATS 12

/* One camera view. Matrices are column-major (glm) like the reference push
 * constants (pt_raygen.rgen:41-49). accum is a device RGBA32F image of
 * width*height texels holding (mean radiance, sample count); history is the
 * number of frames already in it (0 overwrites), the reference's
 * historyFrameCount. path_radiance (device, optional) receives every path's
 * radiance as [spp][height*width][4] floats. aov (device, optional) receives
 * the last sample's first-hit record as [height*width][OHAO_PT_AOV_FLOATS]
 * floats: albedo.rgb, normal*0.5+0.5, view depth, hit flag, roughness,
 * metallic, 0, 0 (background pixels: environment colour, 0, 1e30, 0, 0, 0). */
typedef struct ohao_pt_view {
    float inv_view[16];
    float inv_proj[16];
    uint32_t width;
    uint32_t height;
    uint32_t history;
    uint32_t reserved;
    float* accum;
    float* path_radiance;
    float* aov;
    /* Optional display image, RGBA8 width*height*4 bytes: the reference's
     * outputImage (pt_raygen.rgen:1262-1269), pow(ACES(accum * 0.5), 1/2.2)
     * per channel rounded to nearest, alpha 255, written from the
     * accumulator after the call's samples. Device memory for
     * ohao_pt_render; host memory for ohao_pt_render_host (the readback of
     * VulkanRenderer::getPixels, render_dispatch.cpp:170-186). */
    uint8_t* display;
} ohao_pt_view;

#define OHAO_SAMPLER_PCG 0u
#define OHAO_SAMPLER_SOBOL 1u

/* flag bits keep the reference's PT_FLAG values (pt_raygen.rgen:56-60) */
#define OHAO_PT_FLAG_FIREFLY_CLAMP (1u << 2)
#define OHAO_PT_FLAG_ENV_FIXED_V (1u << 8)   /* not reference: un-mirrored env lookup */
/* Rays without gl_RayFlagsOpaqueEXT: triangles of OHAO_BLAS_FLAG_NO_OPAQUE
 * BLASes take the alpha test of pt_anyhit.rahit:17-50 (closest-hit and
 * shadow rays alike). Off by default, as in the reference. */
#define OHAO_PT_FLAG_ALPHA_TEST (1u << 10)
/* Shade each bounce's ray queue in material order (binned on the device by
 * a key of hit/miss, path phase, metallic, roughness, textured) instead of
 * queue order; the image is the same. Not the reference's (its shading
 * order is the hardware's). */
#define OHAO_PT_FLAG_SORT_MATERIAL (1u << 11)
/* Trace each bounce's rays grouped by direction octant and origin (a
 * device-side binning of the ray queue) instead of queue order; the image
 * is the same. Per-view wavefront only: the persistent pool's launch
 * configuration sets its own ray order. Not the reference's. */
#define OHAO_PT_FLAG_SORT_RAYS (1u << 12)
/* Not the offline reference estimator: the first specular bounce (stage B)
 * draws the half-vector from the GGX distribution of visible normals with
 * weight F * G2/G1 (pt_raygen_realtime.rgen:723-800, ggx_aniso.glsl:56-133)
 * instead of the roughness-scaled cosine jitter; not differentiated by
 * ohao_pt_backward / ohao_pt_adjoint. */
#define OHAO_PT_FLAG_GGX_VNDF (1u << 9)
/* Emitter MIS, not the reference's (which adds emission only where a BSDF
 * ray hits it and never lets a BSDF ray find a GPULight):
 *  - the emissive triangles (material slot-2 emission or an emissive
 *    texture; of visible instances of opaque BLASes) become one more choice
 *    of the light NEE (lights + 1 choices), a triangle chosen by power
 *    (area x luminance of the slot-2 emission, + area with an emissive
 *    texture) and a uniform point on it, both faces emitting;
 *  - BSDF rays of the chains find sphere and area GPULights (each light
 *    crossed, from its emitting side; the lights stay transparent);
 *  - both sides of these emitters are weighted by the balance heuristic
 *    between the light-NEE pdf and the BSDF pdf the estimator's env MIS
 *    uses (pt_raygen.rgen:466-479 and 557-562), weight 1 on the BSDF side
 *    after a delta bounce, as for the environment.
 * Camera rays see no GPULight, as in the reference. Not differentiated by
 * ohao_pt_backward / ohao_pt_adjoint. The emissive table is built on the
 * first render that sets the flag after a build or material change. */
#define OHAO_PT_FLAG_EMITTER_MIS (1u << 13)
#define OHAO_PT_FLAG_PROFILE (1u << 16)      /* record per-kernel CUDA-event times */
/* ohao_pt_adjoint: replay the gradient with fresh samples (sample indices
 * from sample_index_base + spp) instead of the rendered ones, so that it
 * estimates the gradient of the loss of the expected image; with the same
 * samples it would also differentiate the image's noise. */
#define OHAO_PT_FLAG_ADJOINT_DECORRELATE (1u << 17)
/* ohao_pt_adjoint: the loss of the reference's inverse lab, mseRGB on
 * display images (ohao/inverse/image_loss.hpp:59-80): d_targets hold display
 * values in [0, 1] (an RGBA8 capture / 255) and the render passes through
 * the display transform pow(ACES(x / 2), 1/2.2) in float -- before the 8-bit
 * rounding, whose derivative is zero almost everywhere. */
#define OHAO_PT_FLAG_ADJOINT_LDR_LOSS (1u << 18)

#define OHAO_PT_MODE_AUTO 0u
#define OHAO_PT_MODE_WAVEFRONT 1u
#define OHAO_PT_MODE_PERSISTENT 2u

/* Per-call parameters: the reference's push constants and RTRenderSettings
 * (path_tracer_render.cpp:687-719, rt_settings.hpp:17-35). Sample k of a
 * pixel uses sample index sample_index_base + k (PathTracer::m_sampleIndex). */
typedef struct ohao_pt_settings {
    uint32_t spp;
    uint32_t max_bounces;
    uint32_t sample_index_base;
    uint32_t sampler;          /* OHAO_SAMPLER_* */
    uint32_t flags;            /* OHAO_PT_FLAG_* */
    float clamp_luminance;     /* tuning.x */
    float aniso_strength;      /* jitter.z */
    float aniso_rotation;      /* jitter.w */
    uint32_t mode;             /* OHAO_PT_MODE_* */
    /* Traversal stack entries per ray (0 = all 64). A smaller limit makes
     * deep traversals stop with OHAO_ERR_DEVICE_CHECK instead of finishing;
     * it exists to exercise that check. Not the reference's. */
    uint32_t trace_stack_limit;
    /* Traversal shape of the per-view wavefront: 0 = the library's default
     * (one ray per thread on a flat BVH, persistent warps refilled at 8 idle
     * lanes on a two-level one); 1..32 = persistent warps over the ray
     * queue, a warp claiming new rays once at least this many of its lanes
     * are idle; 33 = one ray per thread over a grid-stride loop. Every shape
     * gives the same image. */
    uint32_t wavefront_refill;
    uint32_t reserved[5];
} ohao_pt_settings;

/* Per-kernel timings of the last profiled render/trace (CUDA events on the
 * launching stream): total milliseconds and launch counts. */
typedef struct ohao_pt_profile {
    float extend_ms, shadow_ms, shade_ms, other_ms, total_ms;
    uint32_t extend_launches, shadow_launches, shade_launches, other_launches;
    uint64_t rays_closest, rays_shadow;
    uint64_t nodes_closest, tris_closest;   /* BVH nodes / triangles visited by closest-hit rays */
    uint64_t nodes_shadow, tris_shadow;     /* ... by shadow (any-hit) rays */
    uint32_t lanes;            /* pixel lanes the same call runs unprofiled (per-view wavefront: 1, or 4
                                  with one ray per thread in traversal; each lane runs this profile's
                                  kernel sequence over its slice of the pixels); profiled calls run one */
    uint32_t reserved;
} ohao_pt_profile;

/* ---- lifecycle (PathTracer::init / destroy) ---- */
ohao_status ohao_pt_create(const ohao_pt_desc* desc, ohao_pt_ctx** out);
void ohao_pt_destroy(ohao_pt_ctx* ctx);
const char* ohao_pt_last_error(const ohao_pt_ctx* ctx);
const char* ohao_pt_version(void);

/* ---- scene inputs ----
 * Global geometry as OHAO's RT scene packer uploads it (rt_build.cpp:27-186):
 * positions at pos_stride_bytes (12 packed, 100 for OHAO's Vertex), float4
 * normals, float2 UVs (may be NULL), global pre-offset uint32 indices, one
 * material id per global triangle (PathTracer::setNormalBuffer/setUVBuffer/
 * setMaterialBuffers, path_tracer.hpp:124-133). */
ohao_status ohao_pt_set_geometry(ohao_pt_ctx* ctx, const float* pos, uint32_t pos_stride_bytes, uint32_t nverts,
                                 const float* normal4, const float* uv2, const uint32_t* indices, uint32_t ntris,
                                 const uint32_t* mat_ids);
/* The same upload from device memory, ordered on `stream` (the device
 * buffers the reference's RT scene packer fills, rt_build.cpp:27-186, bound
 * without a host round trip). uv2 may be NULL. The index and material-id
 * checks run on the device; the call returns when the copies and checks on
 * `stream` have finished, so the caller may reuse its buffers afterwards. */
ohao_status ohao_pt_set_geometry_device(ohao_pt_ctx* ctx, const float* d_pos, uint32_t pos_stride_bytes,
                                        uint32_t nverts, const float* d_normal4, const float* d_uv2,
                                        const uint32_t* d_indices, uint32_t ntris, const uint32_t* d_mat_ids,
                                        ohao_stream stream);
/* RTAccelerationStructure::createBLAS (rt_acceleration_structure.cpp:205-300):
 * one triangle geometry over indices [first_index, first_index+index_count). */
ohao_status ohao_pt_create_blas(ohao_pt_ctx* ctx, uint32_t first_index, uint32_t index_count, uint32_t* out_blas);
/* Geometry flags of a BLAS. The reference builds every BLAS with
 * VK_GEOMETRY_OPAQUE_BIT_KHR (rt_acceleration_structure.cpp:227,342) and
 * traces every ray with gl_RayFlagsOpaqueEXT, so its any-hit shader never
 * runs; OHAO_BLAS_FLAG_NO_OPAQUE marks a BLAS whose triangles take the
 * alpha test of pt_anyhit.rahit:17-50 (a hit whose diffuse texture alpha at
 * the hit's UV is below 0.5 is ignored) for rays traced with
 * OHAO_PT_FLAG_ALPHA_TEST. Applies from the next ohao_pt_build. */
#define OHAO_BLAS_FLAG_NO_OPAQUE 1u
ohao_status ohao_pt_set_blas_flags(ohao_pt_ctx* ctx, uint32_t blas, uint32_t flags);
/* clearInstances + addInstance (rt_acceleration_structure.hpp:90-97). */
ohao_status ohao_pt_set_instances(ohao_pt_ctx* ctx, const ohao_pt_instance* inst, uint32_t n);
/* buildTLAS + the BLAS builds (rt_acceleration_structure.cpp:419-530): LBVH
 * on the device; synchronous with respect to `stream`. */
ohao_status ohao_pt_build(ohao_pt_ctx* ctx, ohao_stream stream);
int32_t ohao_pt_is_two_level(const ohao_pt_ctx* ctx);
/* Material table, 3 x vec4 per material (layout_meta.hpp:20-58): diffuse,
 * normal, emissive and roughness-metal texture indices into the bindless
 * texture array of ohao_pt_set_textures (0xFFFFFFFF = none), sampled as
 * pt_closesthit.rchit:108-157 does (sRGB decode pow(c, 2.2) of diffuse and
 * emissive, tangent-space normal map in the Frisvad basis, G = roughness and
 * B = metallic factors). Diffuse index 0 reads the tile albedo map instead
 * when one is set (ohao_pt_set_albedo_map; linear RGB, no alpha). Slot 2
 * .yzw (unused by the reference) carries emissive RGB added to the texture's.
 * Every index a render needs must name a texture by then
 * (OHAO_ERR_INVALID_ARG otherwise). */
ohao_status ohao_pt_set_materials(ohao_pt_ctx* ctx, const float* vec4x3, uint32_t n);
/* The bindless texture array (BindlessTextureManager's sampler2D
 * textures[], pt_closesthit.rchit:35): RGBA8 UNORM images sampled LINEAR /
 * REPEAT at LOD 0 with texel centres at (i + 0.5) / size, restated in float.
 * Replaces the whole array; at most 65536 textures. */
typedef struct ohao_pt_texture {
    const uint8_t* rgba8;      /* host, width*height*4 bytes, row 0 at v = 0 */
    uint32_t width;
    uint32_t height;
} ohao_pt_texture;
ohao_status ohao_pt_set_textures(ohao_pt_ctx* ctx, const ohao_pt_texture* textures, uint32_t n);
/* updateRTMaterialParams (rt_build.cpp:313-389): rewrite records in place. */
ohao_status ohao_pt_update_materials(ohao_pt_ctx* ctx, const float* vec4x3, uint32_t first, uint32_t n);
/* Light SSBO (light_upload.cpp:153-300), at most 64 lights. */
ohao_status ohao_pt_set_lights(ohao_pt_ctx* ctx, const ohao_gpu_light* lights, uint32_t n);
/* HDR environment (RGBA32F w*h, row 0 = +Y in the CDF convention) with its
 * marginal (h) / conditional (w*h) CDFs and integral (setEnvCDFBuffers,
 * path_tracer.hpp:170-177); marg/cond NULL disables env importance sampling;
 * rgba NULL removes the environment. intensity <= 0 means 1 (pt_miss.rmiss:65). */
ohao_status ohao_pt_set_env(ohao_pt_ctx* ctx, const float* rgba, uint32_t w, uint32_t h, const float* marg,
                            const float* cond, float integral, float intensity);
/* Linear RGB tile albedo map (w*h*3 floats) read by materials whose diffuse
 * texture index is 0, sampled bilinearly as ohao/render/diff/diff_map.hpp:40-67. */
ohao_status ohao_pt_set_albedo_map(ohao_pt_ctx* ctx, const float* rgb, uint32_t w, uint32_t h);
/* EnvCDF::build (ohao/render/rt/env_cdf.cpp:13-61), bit-identical. */
ohao_status ohao_env_cdf_build(const float* rgba, int32_t w, int32_t h, float* marg, float* cond, float* integral);

/* ---- render (PathTracer::render) ----
 * Renders settings->spp samples per pixel into each view's device accum
 * buffer on `stream`. n_views > 1 with mode AUTO uses the persistent
 * multi-view kernel. */
ohao_status ohao_pt_render(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                           const ohao_pt_settings* settings, ohao_stream stream);
/* Host-buffer variant (VulkanRenderer::getPixels analogue): views' device
 * pointers are ignored; accumulation runs in library-owned device images
 * seeded from and copied back to host_accum[i] (RGBA32F width*height). */
ohao_status ohao_pt_render_host(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                const ohao_pt_settings* settings, float* const* host_accum, ohao_stream stream);
ohao_status ohao_pt_get_profile(const ohao_pt_ctx* ctx, ohao_pt_profile* out);
/* The display transform alone (the tonemap + gamma tail of
 * pt_raygen.rgen:1262-1269) over npix device RGBA32F texels into device
 * RGBA8: for an accumulator written elsewhere, or a denoised image. */
ohao_status ohao_pt_display(const float* d_rgba32f, uint32_t npix, uint8_t* d_rgba8, ohao_stream stream);

/* First-hit features (the record of ohao_pt_view.aov) averaged over st->spp
 * camera samples per pixel, sample indices st->sample_index_base + k, into
 * d_aov ([height*width][OHAO_PT_AOV_FLOATS] floats, device): albedo,
 * encoded normal, roughness and metallic averaged over the samples, the hit
 * flag as the fraction of samples that hit, the view depth averaged over
 * the samples that hit (1e30 if none). One sample gives the record a render
 * writes for that sample, bit for bit. Costs one closest-hit traversal and
 * one surface evaluation per sample: auxiliary inputs for a denoiser of a
 * low-sample radiance image. Not the reference's. */
ohao_status ohao_pt_aov(ohao_pt_ctx* ctx, const ohao_pt_view* view, const ohao_pt_settings* st, float* d_aov,
                        ohao_stream stream);
/* Times the compiled launch shapes of the persistent multi-view kernel
 * (block size, blocks per SM, pixels per work-queue claim) on these views
 * and keeps the fastest for later renders of this context. The views'
 * accumulators are overwritten. No counterpart in the reference. */
ohao_status ohao_pt_autotune(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                             const ohao_pt_settings* settings, float* best_ms, ohao_stream stream);
/* Name of the persistent launch shape in use ("default" before autotune). */
const char* ohao_pt_launch_config(const ohao_pt_ctx* ctx);
/* Name of compiled launch shape `index` (NULL past the last), and selection
 * of one by name for later renders of this context (OHAO_ERR_INVALID_ARG for
 * an unknown name). All shapes give bit-identical images. No counterpart in
 * the reference. */
const char* ohao_pt_launch_config_at(uint32_t index);
ohao_status ohao_pt_set_launch_config(ohao_pt_ctx* ctx, const char* name);

/* ---- Gradients (path replay) ----
 * Replace the inverse lab's coordinate finite differences over the tile
 * albedo map and material parameters (ohao/inverse/diff_fit.hpp:177-200,
 * ohao/inverse/staged_fit.hpp:316-332; the map is ohao/render/diff/
 * diff_map.hpp). Parameters: the linear albedo map of ohao_pt_set_albedo_map
 * (read by materials whose diffuse texture index is 0) and every material's
 * roughness. Sampling is detached: each path of the image is replayed from
 * its own seed with its primal decisions, and BRDF values, albedo factors and
 * MIS weights are differentiated. Not supported with the firefly clamp or
 * max_bounces above 16. No counterpart call in the reference.
 *
 * ohao_pt_backward: d_grad_image[v] (device RGBA32F, A ignored) is dLoss/dI
 * for the image that ohao_pt_render produced with the same views, settings
 * and history 0. Overwrites d_grad_albedo_map (device, map_h*map_w*3 floats)
 * and d_grad_roughness (device, one float per material); either may be NULL. */
ohao_status ohao_pt_backward(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                             const ohao_pt_settings* settings, const float* const* d_grad_image,
                             float* d_grad_albedo_map, float* d_grad_roughness, ohao_stream stream);
/* lossMulti (ohao/render/diff/diff_vk_forward.hpp:80-93) on linear radiance:
 * renders every view into views[v].accum with history 0, loss = mean over
 * views of the RGB mean squared error against d_targets[v] (device RGBA32F),
 * written to *loss (host), and its gradients as for ohao_pt_backward. */
ohao_status ohao_pt_adjoint(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                  const ohao_pt_settings* settings, const float* const* d_targets,
                                  float* d_grad_albedo_map, float* d_grad_roughness, float* loss,
                                  ohao_stream stream);

/* Host-buffer variant (the inverse lab keeps its images and parameters in
 * host memory): views' device pointers are ignored; host_targets[v] (RGBA32F
 * width*height, display values in [0, 1] with OHAO_PT_FLAG_ADJOINT_LDR_LOSS)
 * are uploaded, the renders accumulate in library-owned device images, and
 * the gradients land in host_grad_albedo_map (map_h*map_w*3 floats) and
 * host_grad_roughness (one float per material); either may be NULL. Returns
 * when the host buffers hold the results. */
ohao_status ohao_pt_adjoint_host(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                 const ohao_pt_settings* settings, const float* const* host_targets,
                                 float* host_grad_albedo_map, float* host_grad_roughness, float* loss,
                                 ohao_stream stream);

/* ---- traceRayEXT as a batch call ----
 * rays: device, n x 8 floats (origin.xyz, tmin, dir.xyz, tmax).
 * hits: device, n x 5 uint32 (t bits, u bits, v bits, instance, primitive);
 * a miss has instance = primitive = 0xFFFFFFFF. any_hit bit 0 set writes 1/0
 * in hits[5i] (occluded); bit 1 set traces non-opaque rays (the alpha test
 * of OHAO_PT_FLAG_ALPHA_TEST). stats (device, optional): n x 2 uint32
 * nodes/triangles visited. */
ohao_status ohao_pt_trace(ohao_pt_ctx* ctx, const float* rays, uint32_t n, uint32_t* hits, int32_t any_hit,
                          uint32_t* stats, ohao_stream stream);

/* ---- BVH inspection (tests / tools) ----
 * which = -1: the flat BVH (or the TLAS when two-level); which = k: BLAS k.
 * Nodes are ohao_bvh8_node; primitives are ohao_bvh_tri (uint32 instance ids
 * for the TLAS). Host destination buffers. */
typedef struct ohao_bvh8_node {
    float origin[3];
    int8_t exps[3];            /* per-axis power-of-two grid exponent */
    uint8_t imask;             /* bit i: slot i is an internal child */
    uint32_t child_base;       /* first internal child node */
    uint32_t tri_base;         /* first primitive of this node's leaves */
    uint8_t meta[8];           /* 0 empty; 0x80|rank internal; (count<<5)|offset leaf */
    uint8_t qlo[3][8];         /* child box per axis on the grid, rounded outward; */
    uint8_t qhi[3][8];         /* an empty slot holds qlo 255, qhi 0 (no ray enters it) */
} ohao_bvh8_node;               /* 80 bytes */
typedef struct ohao_bvh_tri {
    float v0[3]; uint32_t prim;
    float v1[3]; uint32_t inst;
    float v2[3]; uint32_t ref;
} ohao_bvh_tri;                 /* 48 bytes */
ohao_status ohao_pt_bvh_info(const ohao_pt_ctx* ctx, int32_t which, uint32_t* n_nodes, uint32_t* n_prims,
                             uint32_t* height);
ohao_status ohao_pt_bvh_download(ohao_pt_ctx* ctx, int32_t which, void* nodes, void* prims);

/* ---- BVH build that allocates nothing ----
 * No counterpart in the reference (its BVH builds happen inside the Vulkan
 * driver). For callers that cannot call cudaMalloc: a host application that
 * gives the renderer a fixed memory budget and owns the rest of the GPU, or a
 * per-frame rebuild of a small animated mesh where an allocation would
 * synchronise the device and stall the engine's other streams. Builds the
 * same 8-wide BVH as ohao_pt_build over n primitive boxes (device, 6 floats
 * lo.xyz hi.xyz each), n <= 65536: d_nodes (device) receives up to n
 * ohao_bvh8_node records, d_prim_order (device, n uint32) the box index of
 * each leaf slot, d_root_box (device) 6 floats; *out_nnodes / *out_height
 * are written on the host. Larger n returns OHAO_ERR_TOO_LARGE before the
 * device is touched. The build scratch is one fixed array in device memory
 * (about 9.2 MB per GPU that loads the library, held until exit) shared by
 * every call: calls that overlap on the GPU (other threads or streams) race
 * on it and must be serialised by the caller. The first call on a device
 * resolves the array's device address (cached per device ordinal; a
 * cudaDeviceReset of that device invalidates it, so the library is not used
 * on a device after a reset). Every call blocks the host until its build on
 * `stream` has finished. */
#define OHAO_BVH_NOALLOC_MAX_PRIMS 65536u
ohao_status ohao_bvh_build_noalloc(const float* d_boxes, uint32_t n, void* d_nodes, uint32_t* d_prim_order,
                                   float* d_root_box, uint32_t* out_nnodes, uint32_t* out_height, ohao_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* OHAO_PT_H */
