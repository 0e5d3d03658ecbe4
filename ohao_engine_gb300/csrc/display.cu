// display.cu -- the reference's display transform to RGBA8: per channel
// ldr = pow(ACES(radiance * 0.5), 1/2.2) stored to an RGBA8 UNORM image
// with alpha 1 (pt_raygen.rgen:99-102, 1262-1269; readback
// render_dispatch.cpp:170-186).
//
// The 8-bit value is the round-to-nearest quantisation of pow(y, 1/2.2)
// (y = ACES(x * 0.5) in float): byte = #{k : y >= t_k} with thresholds
// t_k = ((k + 0.5) / 255)^2.2, k = 0..254 (computed in double, rounded to
// float). Counting thresholds replaces the pow and its rounding with 8
// float comparisons, so host and device give the same bytes.
#include <cstdint>
#include <cuda_runtime.h>

#include "pt_types.hpp"

namespace ohao {

namespace {

__constant__ float c_display_thr[255] = {
    0x1.289c1cp-20f, 0x1.9faedap-17f, 0x1.3fb844p-15f, 0x1.4f22d8p-14f, 0x1.234766p-13f, 0x1.c4f04ep-13f,
    0x1.470e1ap-12f, 0x1.c01208p-12f, 0x1.270e1cp-11f, 0x1.78dab2p-11f, 0x1.d5acf2p-11f, 0x1.1edfp-10f,
    0x1.58a16p-10f, 0x1.983648p-10f, 0x1.ddb4dcp-10f, 0x1.149974p-9f, 0x1.3d6286p-9f, 0x1.693f72p-9f,
    0x1.98398ap-9f, 0x1.ca59b8p-9f, 0x1.ffa886p-9f, 0x1.1c1712p-8f, 0x1.39f93cp-8f, 0x1.597e88p-8f,
    0x1.7aaaa2p-8f, 0x1.9d8114p-8f, 0x1.c2054ap-8f, 0x1.e83a98p-8f, 0x1.08121ap-7f, 0x1.1ce2ap-7f,
    0x1.329064p-7f, 0x1.491cep-7f, 0x1.608984p-7f, 0x1.78d7bcp-7f, 0x1.9208e2p-7f, 0x1.ac1e5p-7f,
    0x1.c71956p-7f, 0x1.e2fb38p-7f, 0x1.ffc538p-7f, 0x1.0ebc48p-6f, 0x1.1e0b38p-6f, 0x1.2dd006p-6f,
    0x1.3e0b42p-6f, 0x1.4ebd8p-6f, 0x1.5fe74ap-6f, 0x1.71893p-6f, 0x1.83a3b8p-6f, 0x1.963768p-6f,
    0x1.a944c6p-6f, 0x1.bccc54p-6f, 0x1.d0ce92p-6f, 0x1.e54bfcp-6f, 0x1.fa451p-6f, 0x1.07dd24p-5f,
    0x1.12d60ep-5f, 0x1.1e0d8p-5f, 0x1.2983b6p-5f, 0x1.3538e8p-5f, 0x1.412d5p-5f, 0x1.4d6126p-5f,
    0x1.59d4ap-5f, 0x1.6687f4p-5f, 0x1.737b5ap-5f, 0x1.80af04p-5f, 0x1.8e232ap-5f, 0x1.9bd7fcp-5f,
    0x1.a9cdaep-5f, 0x1.b80474p-5f, 0x1.c67c7ep-5f, 0x1.d536p-5f, 0x1.e43126p-5f, 0x1.f36e24p-5f,
    0x1.017694p-4f, 0x1.095732p-4f, 0x1.1159p-4f, 0x1.197c18p-4f, 0x1.21c08ep-4f, 0x1.2a267cp-4f,
    0x1.32adf6p-4f, 0x1.3b5712p-4f, 0x1.4421e8p-4f, 0x1.4d0e8ap-4f, 0x1.561d1p-4f, 0x1.5f4d8ep-4f,
    0x1.68a01ap-4f, 0x1.7214c8p-4f, 0x1.7babaep-4f, 0x1.8564dep-4f, 0x1.8f406ep-4f, 0x1.993e72p-4f,
    0x1.a35efcp-4f, 0x1.ada222p-4f, 0x1.b807f6p-4f, 0x1.c2908cp-4f, 0x1.cd3bf6p-4f, 0x1.d80a4ap-4f,
    0x1.e2fb96p-4f, 0x1.ee0ff2p-4f, 0x1.f9476ep-4f, 0x1.02510ep-3f, 0x1.081006p-3f, 0x1.0de0aap-3f,
    0x1.13c304p-3f, 0x1.19b71ap-3f, 0x1.1fbcf6p-3f, 0x1.25d4ap-3f, 0x1.2bfe22p-3f, 0x1.323984p-3f,
    0x1.3886cep-3f, 0x1.3ee60ap-3f, 0x1.45574p-3f, 0x1.4bda78p-3f, 0x1.526fbap-3f, 0x1.59170ep-3f,
    0x1.5fd07ep-3f, 0x1.669c1p-3f, 0x1.6d79ccp-3f, 0x1.7469bcp-3f, 0x1.7b6be6p-3f, 0x1.828054p-3f,
    0x1.89a70cp-3f, 0x1.90e018p-3f, 0x1.982b7ep-3f, 0x1.9f8944p-3f, 0x1.a6f976p-3f, 0x1.ae7c18p-3f,
    0x1.b61132p-3f, 0x1.bdb8cep-3f, 0x1.c572fp-3f, 0x1.cd3fa4p-3f, 0x1.d51eecp-3f, 0x1.dd10d4p-3f,
    0x1.e5156p-3f, 0x1.ed2c98p-3f, 0x1.f55684p-3f, 0x1.fd932ap-3f, 0x1.02f14ap-2f, 0x1.072262p-2f,
    0x1.0b5ce4p-2f, 0x1.0fa0dp-2f, 0x1.13ee2cp-2f, 0x1.1844fap-2f, 0x1.1ca53cp-2f, 0x1.210efap-2f,
    0x1.258234p-2f, 0x1.29feecp-2f, 0x1.2e852ap-2f, 0x1.3314eep-2f, 0x1.37ae3cp-2f, 0x1.3c5116p-2f,
    0x1.40fd82p-2f, 0x1.45b382p-2f, 0x1.4a7318p-2f, 0x1.4f3c4ap-2f, 0x1.540f18p-2f, 0x1.58eb88p-2f,
    0x1.5dd19cp-2f, 0x1.62c156p-2f, 0x1.67babap-2f, 0x1.6cbdcep-2f, 0x1.71ca9p-2f, 0x1.76e106p-2f,
    0x1.7c0134p-2f, 0x1.812b1ap-2f, 0x1.865ebep-2f, 0x1.8b9c22p-2f, 0x1.90e34ap-2f, 0x1.963436p-2f,
    0x1.9b8eecp-2f, 0x1.a0f36ep-2f, 0x1.a661bep-2f, 0x1.abd9ep-2f, 0x1.b15bd8p-2f, 0x1.b6e7a6p-2f,
    0x1.bc7d5p-2f, 0x1.c21cd8p-2f, 0x1.c7c63ep-2f, 0x1.cd798ap-2f, 0x1.d336bap-2f, 0x1.d8fdd4p-2f,
    0x1.decedap-2f, 0x1.e4a9cep-2f, 0x1.ea8eb4p-2f, 0x1.f07d8ep-2f, 0x1.f6766p-2f, 0x1.fc792cp-2f,
    0x1.0142fap-1f, 0x1.044e5ep-1f, 0x1.075ec2p-1f, 0x1.0a7428p-1f, 0x1.0d8e94p-1f, 0x1.10ae04p-1f,
    0x1.13d27ap-1f, 0x1.16fbf8p-1f, 0x1.1a2a8p-1f, 0x1.1d5e12p-1f, 0x1.2096bp-1f, 0x1.23d45ap-1f,
    0x1.271712p-1f, 0x1.2a5edcp-1f, 0x1.2dabb6p-1f, 0x1.30fda2p-1f, 0x1.3454a2p-1f, 0x1.37b0b6p-1f,
    0x1.3b11e2p-1f, 0x1.3e7824p-1f, 0x1.41e38p-1f, 0x1.4553f6p-1f, 0x1.48c986p-1f, 0x1.4c4432p-1f,
    0x1.4fc3fep-1f, 0x1.5348e8p-1f, 0x1.56d2f2p-1f, 0x1.5a621ep-1f, 0x1.5df66cp-1f, 0x1.618fdep-1f,
    0x1.652e76p-1f, 0x1.68d234p-1f, 0x1.6c7b1ap-1f, 0x1.702928p-1f, 0x1.73dc62p-1f, 0x1.7794c6p-1f,
    0x1.7b5256p-1f, 0x1.7f1514p-1f, 0x1.82ddp-1f, 0x1.86aa1ep-1f, 0x1.8a7c6cp-1f, 0x1.8e53ecp-1f,
    0x1.9230ap-1f, 0x1.96128ap-1f, 0x1.99f9a8p-1f, 0x1.9de5fep-1f, 0x1.a1d78cp-1f, 0x1.a5ce54p-1f,
    0x1.a9ca56p-1f, 0x1.adcb92p-1f, 0x1.b1d20ep-1f, 0x1.b5ddc6p-1f, 0x1.b9eebcp-1f, 0x1.be04f4p-1f,
    0x1.c2206ep-1f, 0x1.c64128p-1f, 0x1.ca6728p-1f, 0x1.ce926ap-1f, 0x1.d2c2f4p-1f, 0x1.d6f8c4p-1f,
    0x1.db33dcp-1f, 0x1.df743ep-1f, 0x1.e3b9eap-1f, 0x1.e804ep-1f, 0x1.ec5524p-1f, 0x1.f0aab4p-1f,
    0x1.f50594p-1f, 0x1.f965c2p-1f, 0x1.fdcb42p-1f,
};

__device__ __forceinline__ float aces(float x) {
    const float y = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    const float lo = y > 0.0f ? y : 0.0f;   // clamp(y, 0, 1); NaN -> 0
    return lo < 1.0f ? lo : 1.0f;
}

__device__ __forceinline__ uint32_t display_byte(float radiance) {
    const float y = aces(radiance * 0.5f);
    uint32_t c = 0;
#pragma unroll
    for (uint32_t step = 128; step > 0; step >>= 1)
        if (y >= c_display_thr[c + step - 1]) c += step;
    return c;
}

__global__ void k_display(const float4* __restrict__ acc, uint32_t n, uchar4* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        out[i] = make_uchar4(static_cast<unsigned char>(display_byte(a.x)), static_cast<unsigned char>(display_byte(a.y)),
                             static_cast<unsigned char>(display_byte(a.z)), 255);
    }
}

}  // namespace

cudaError_t launch_display(const float* accum, uint32_t npix, uint8_t* rgba8, cudaStream_t st) {
    if (npix == 0) return cudaSuccess;
    const uint32_t want = (npix + 255u) / 256u;
    const uint32_t blocks = want < 152u * 16u ? want : 152u * 16u;
    k_display<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(accum), npix, reinterpret_cast<uchar4*>(rgba8));
    return cudaGetLastError();
}

}  // namespace ohao
