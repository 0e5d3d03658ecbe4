/*
 * ohao_dn.h -- C ABI of the GB300 learned denoiser.
 *
 * The reference denoises with Intel Open Image Denoise on the CPU
 * (ohao/render/rt/oidn_denoise.cpp:10-29: color + albedo + normal in,
 * denoised color out, falling back to the noisy image when OIDN is absent).
 * This library replaces it with a small convolutional U-Net (5 levels,
 * 32/48/64/96/128 channels, 3x3 convolutions, ReLU, 2x2 max-pool, nearest
 * upsampling, skip concatenation) whose convolutions run as BF16 implicit
 * GEMMs on tcgen05 tensor cores with FP32 accumulation, and which is trained
 * on the GPU by the same library from pairs the path tracer renders.
 *
 * Inputs per image: the path tracer's accumulator (device RGBA32F, the
 * ohao_pt_view.accum layout) and its AOV image (device
 * [h*w][OHAO_PT_AOV_FLOATS] floats, the ohao_pt_view.aov layout). Network
 * input channels: log(1 + radiance / m).rgb with m = albedo + 0.04 on hits
 * and 1 elsewhere (albedo demodulation), albedo.rgb, encoded normal,
 * 1 / (1 + depth) on hits, roughness, metallic. Output: log(1 + radiance / m),
 * returned remodulated as linear RGBA32F. Loss: L1 in that log space plus
 * L1 after the reference's display transform.
 *
 * Status codes and ohao_stream are those of ohao_pt.h. A context is
 * externally synchronised. No counterpart calls in the reference beyond the
 * OIDN pass named above.
 */
#ifndef OHAO_DN_H
#define OHAO_DN_H

#include "ohao_pt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ohao_dn_ctx ohao_dn_ctx;

typedef struct ohao_dn_desc {
    int32_t device;
    uint32_t seed;          /* weight initialisation (He-normal) */
    uint64_t max_pixels;    /* largest n_images * padded width * padded height of any call */
} ohao_dn_desc;

ohao_status ohao_dn_create(const ohao_dn_desc* desc, ohao_dn_ctx** out);
void ohao_dn_destroy(ohao_dn_ctx* ctx);
const char* ohao_dn_last_error(const ohao_dn_ctx* ctx);

/* Check of the tensor-core pipeline's bounded waits (no counterpart in the
 * reference): one kernel waits spin_limit polls (1..65536) on an mbarrier
 * whose phase never completes -- no MMA is issued and no tensor memory is
 * held -- and records the timeout as every convolution kernel does. Returns
 * OHAO_ERR_TIMEOUT, the status a convolution reports when one of its waits
 * gives up; the context stays usable. */
ohao_status ohao_dn_wait_selftest(ohao_dn_ctx* ctx, uint32_t spin_limit, ohao_stream stream);

/* Parameters as FP32 host arrays, layer by layer: W[cout][3][3][cin] then
 * bias[cout]. */
uint64_t ohao_dn_param_count(const ohao_dn_ctx* ctx);
ohao_status ohao_dn_get_params(ohao_dn_ctx* ctx, float* host, uint64_t n);
ohao_status ohao_dn_set_params(ohao_dn_ctx* ctx, const float* host, uint64_t n);
ohao_status ohao_dn_save(ohao_dn_ctx* ctx, const char* path);
ohao_status ohao_dn_load(ohao_dn_ctx* ctx, const char* path);

/* Denoises n_images images of width x height (padded internally to
 * multiples of 16). d_out[i]: device RGBA32F width*height. */
ohao_status ohao_dn_infer(ohao_dn_ctx* ctx, const float* const* d_radiance, const float* const* d_aov,
                          uint32_t n_images, uint32_t width, uint32_t height, float* const* d_out,
                          ohao_stream stream);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) of the loss between the
 * network output y and the reference d_target (device RGBA32F) over a batch:
 * per channel |y - log(1 + t)| + |D(exp(y) - 1) - D(t)|, D the display
 * transform pow(ACES(x / 2), 1/2.2) of pt_raygen.rgen:1263-1264, averaged.
 * *loss (host) receives the batch loss before the step. width and height
 * must be multiples of 16. */
ohao_status ohao_dn_train_step(ohao_dn_ctx* ctx, const float* const* d_radiance, const float* const* d_aov,
                               const float* const* d_target, uint32_t n_images, uint32_t width, uint32_t height,
                               float lr, float* loss, ohao_stream stream);

/* Gradients of the last ohao_dn_train_step's loss in the ohao_dn_get_params
 * layout (before the Adam update was applied). For gradient checks. */
ohao_status ohao_dn_get_grads(ohao_dn_ctx* ctx, float* host, uint64_t n);

/* Inspection (tests): tensor `index` of the last forward pass (0 = packed
 * input, then one per layer output and pool in execution order), or with
 * grad != 0 its loss gradient from the last ohao_dn_train_step, as FP32
 * [pixels][stored channels]; *channels receives the stored channel count
 * and *pixels the pixel count. */
ohao_status ohao_dn_tensor(ohao_dn_ctx* ctx, int32_t index, int32_t grad, float* host, uint64_t n,
                           uint32_t* channels, uint64_t* pixels);

#ifdef __cplusplus
}
#endif

#endif /* OHAO_DN_H */
