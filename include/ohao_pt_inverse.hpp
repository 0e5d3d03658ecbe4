/*
 * ohao_pt_inverse.hpp -- C++20 image formation for OHAO's inverse lab on the
 * C ABI of ohao_pt.h (header only, host memory only, no CUDA headers).
 *
 * The reference's inverse optimisers render through the plug-in interface
 * IInverseImageFormation (ohao/inverse/backend/image_formation.hpp:40-60):
 *   forward(InverseRenderRequest{viewIndex, RenderBudget{width, height, spp},
 *           seed, denoise}) -> ImageRGBA8
 * and, lacking gradients (supportsAnalyticGrads() == false), differentiate it
 * by coordinate finite differences: two full renders per parameter
 * (ohao/inverse/staged_fit.hpp:316-332). PtImageFormation provides both
 * halves on one GPU: forward() returns the RGBA8 display image that the
 * Vulkan path tracer's getPixels readback returns (render_dispatch.cpp:
 * 170-186), and gradient() returns the analytic gradient of the lab's
 * display-space loss mseRGB (ohao/inverse/image_loss.hpp:59-80) over a set of
 * views with respect to the tile albedo map and every material's roughness,
 * from one path-replay adjoint pass (ohao_pt_adjoint_host). The wrapper a
 * reference maintainer adds around it (an IInverseImageFormation subclass
 * with supportsAnalyticGrads() == true) is shown in INTEGRATION.md.
 *
 * Status codes are those of ohao_pt.h; lastError() explains the last failure.
 * Like the context it wraps, an instance is externally synchronised.
 */
#ifndef OHAO_PT_INVERSE_HPP
#define OHAO_PT_INVERSE_HPP

#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "ohao_pt.h"

namespace ohao_gb300 {

/* One camera of the lab's view set: column-major inverse view and inverse
 * projection matrices (glm layout, the push constants of pt_raygen.rgen:41-49). */
struct Camera {
    float inv_view[16];
    float inv_proj[16];
};

class PtImageFormation {
public:
    /* ctx: a built context (geometry, materials, environment, tile albedo
     * map and ohao_pt_build already done); not owned. */
    explicit PtImageFormation(ohao_pt_ctx* ctx, std::vector<Camera> cameras, uint32_t max_bounces = 4)
        : ctx_(ctx), cams_(std::move(cameras)), max_bounces_(max_bounces) {}

    [[nodiscard]] bool supportsAnalyticGrads() const noexcept { return true; }
    [[nodiscard]] size_t viewCount() const noexcept { return cams_.size(); }
    [[nodiscard]] const char* lastError() const noexcept { return ohao_pt_last_error(ctx_); }

    /* Renders camera view_index at width x height with spp samples per pixel
     * into rgba8 (width*height*4 bytes, the display image). The request's
     * seed selects the sample stream: sample indices start at seed * spp, so
     * successive seeds use disjoint samples. */
    [[nodiscard]] ohao_status forward(int view_index, uint32_t width, uint32_t height, int spp, uint32_t seed,
                                      std::vector<uint8_t>& rgba8) const {
        if (view_index < 0 || static_cast<size_t>(view_index) >= cams_.size() || spp <= 0) return OHAO_ERR_INVALID_ARG;
        const size_t npix = static_cast<size_t>(width) * height;
        std::vector<float> accum(npix * 4, 0.0f);
        rgba8.assign(npix * 4, 0);
        ohao_pt_view v = view_of(view_index, width, height);
        v.display = rgba8.data();
        ohao_pt_settings st = settings(spp, seed, 0u);
        float* acc = accum.data();
        return ohao_pt_render_host(ctx_, &v, 1, &st, &acc, nullptr);
    }

    /* Gradient of L = mean over the given views of mseRGB(display(render),
     * target), targets as RGBA8 display images (width*height*4 bytes each,
     * alpha ignored), with respect to the tile albedo map (d_map, map_h *
     * map_w * 3 floats) and each material's roughness (d_rough, one float per
     * material). The adjoint replays the paths with fresh samples, so it
     * estimates the gradient of the loss of the expected image. */
    [[nodiscard]] ohao_status gradient(const std::vector<int>& view_indices, uint32_t width, uint32_t height,
                                       const std::vector<const uint8_t*>& targets_rgba8, int spp, uint32_t seed,
                                       std::vector<float>& d_map, std::vector<float>& d_rough, float& loss) const {
        if (view_indices.empty() || view_indices.size() != targets_rgba8.size() || spp <= 0) return OHAO_ERR_INVALID_ARG;
        const size_t npix = static_cast<size_t>(width) * height;
        std::vector<ohao_pt_view> views;
        std::vector<std::vector<float>> targets(view_indices.size());
        std::vector<const float*> tptr;
        for (size_t k = 0; k < view_indices.size(); ++k) {
            const int vi = view_indices[k];
            if (vi < 0 || static_cast<size_t>(vi) >= cams_.size() || !targets_rgba8[k]) return OHAO_ERR_INVALID_ARG;
            views.push_back(view_of(vi, width, height));
            targets[k].resize(npix * 4);
            for (size_t i = 0; i < npix * 4; ++i) targets[k][i] = static_cast<float>(targets_rgba8[k][i]) / 255.0f;
            tptr.push_back(targets[k].data());
        }
        ohao_pt_settings st = settings(spp, seed, OHAO_PT_FLAG_ADJOINT_LDR_LOSS | OHAO_PT_FLAG_ADJOINT_DECORRELATE);
        return ohao_pt_adjoint_host(ctx_, views.data(), static_cast<uint32_t>(views.size()), &st, tptr.data(),
                                    d_map.empty() ? nullptr : d_map.data(), d_rough.empty() ? nullptr : d_rough.data(),
                                    &loss, nullptr);
    }

private:
    ohao_pt_view view_of(int view_index, uint32_t width, uint32_t height) const {
        ohao_pt_view v;
        std::memset(&v, 0, sizeof v);
        std::memcpy(v.inv_view, cams_[static_cast<size_t>(view_index)].inv_view, sizeof v.inv_view);
        std::memcpy(v.inv_proj, cams_[static_cast<size_t>(view_index)].inv_proj, sizeof v.inv_proj);
        v.width = width;
        v.height = height;
        v.history = 0;
        return v;
    }
    ohao_pt_settings settings(int spp, uint32_t seed, uint32_t flags) const {
        ohao_pt_settings st;
        std::memset(&st, 0, sizeof st);
        st.spp = static_cast<uint32_t>(spp);
        st.max_bounces = max_bounces_;
        st.sample_index_base = seed * static_cast<uint32_t>(spp);
        st.sampler = OHAO_SAMPLER_PCG;
        st.flags = flags;
        st.mode = OHAO_PT_MODE_WAVEFRONT;
        return st;
    }

    ohao_pt_ctx* ctx_;
    std::vector<Camera> cams_;
    uint32_t max_bounces_;
};

}  // namespace ohao_gb300

#endif /* OHAO_PT_INVERSE_HPP */
