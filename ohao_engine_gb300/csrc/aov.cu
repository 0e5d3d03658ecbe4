// aov.cu -- first-hit features averaged over several camera samples per
// pixel (ohao_pt_aov): the auxiliary inputs a denoiser takes beside a
// low-sample radiance image. Each sample is the camera ray of path_start for
// (pixel, sample index), its closest hit and the surface that hit_shade
// reconstructs, reduced by aov_of -- the same record a render writes for its
// last sample -- so one sample reproduces the render's record bit for bit.
// Means: albedo, normal (encoded), roughness and metallic over all samples
// (a miss contributes the environment colour and zeros, as in the render's
// record), the hit flag as the fraction of samples that hit, the view depth
// over the samples that hit (1e30 when none did).
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "pt_path.cuh"

namespace ohao {

namespace {

// kTex: bindless textures in the scene (as the render's shading kernel);
// kLevels: 1 flat BVH (its first 8 stack entries in shared memory, as the
// render's closest-hit kernel), 2 two-level
constexpr int kAovShStack = 8;
template <bool kTex, int kLevels>
__global__ void __launch_bounds__(128) k_aov_mean(DScene sc, PathParams pp, ViewParams vp, uint32_t nsamp,
                                                  float* __restrict__ out, int* err) {
    constexpr int kSh = kLevels == 1 ? kAovShStack : 0;
    __shared__ uint2 s_stack[kSh > 0 ? kSh * kShStride : 1];
    const uint32_t npix = vp.width * vp.height;
    int e = 0;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        const uint32_t px = pix % vp.width, py = pix / vp.width;
        V3 alb = v3s(0.0f), nrm = v3s(0.0f);
        float depth = 0.0f, hits = 0.0f, rough = 0.0f, metal = 0.0f;
        for (uint32_t k = 0; k < nsamp; ++k) {
            PathState ps;
            path_start(vp, pp, px, py, pp.sample_base + k, ps);
            TravCount tc{0, 0};
            const Hit h = scene_closest<false, kLevels, true, kSh>(sc, ps.ro, ps.rd, 0.001f, 10000.0f, tc, e,
                                                                   s_stack + threadIdx.x);
            Surf s;
            if (h.prim != 0xFFFFFFFFu) hit_shade<kTex>(sc, ps.ro, ps.rd, h, s);
            else miss_shade(sc, pp, ps.rd, s);
            AovOut ao;
            aov_of(s, vp, ao);
            alb = alb + ao.albedo;
            nrm = nrm + ao.normal;
            if (ao.hit > 0.0f) depth += ao.depth;
            hits += ao.hit;
            rough += ao.rough;
            metal += ao.metal;
        }
        const float inv = 1.0f / static_cast<float>(nsamp);
        float4* a = reinterpret_cast<float4*>(out + static_cast<size_t>(pix) * OHAO_PT_AOV_FLOATS);
        a[0] = make_float4(alb.x * inv, alb.y * inv, alb.z * inv, nrm.x * inv);
        a[1] = make_float4(nrm.y * inv, nrm.z * inv, hits > 0.0f ? depth / hits : 1e30f, hits * inv);
        a[2] = make_float4(rough * inv, metal * inv, 0.0f, 0.0f);
    }
    if (e) atomicOr(err, 1);
}

}  // namespace

cudaError_t launch_aov_mean(const DScene& sc, const PathParams& pp, const ViewParams& vp, uint32_t nsamp, float* out,
                            int* err, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t npix = vp.width * vp.height;
    const uint32_t blocks = std::max(1u, std::min((npix + 127u) / 128u, static_cast<uint32_t>(std::max(sms, 1)) * 16u));
    if (sc.two_level) {
        if (sc.ntex) k_aov_mean<true, 2><<<blocks, 128, 0, st>>>(sc, pp, vp, nsamp, out, err);
        else k_aov_mean<false, 2><<<blocks, 128, 0, st>>>(sc, pp, vp, nsamp, out, err);
    } else {
        if (sc.ntex) k_aov_mean<true, 1><<<blocks, 128, 0, st>>>(sc, pp, vp, nsamp, out, err);
        else k_aov_mean<false, 1><<<blocks, 128, 0, st>>>(sc, pp, vp, nsamp, out, err);
    }
    return cudaGetLastError();
}

}  // namespace ohao
