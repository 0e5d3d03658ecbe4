// dn_types.hpp -- shapes and launch arguments of the denoiser kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/ohao_pt.h"

namespace ohao {
namespace dn {

constexpr int kFwd = 0, kDgrad = 1, kWgrad = 2;

struct Geo {          // a batch of n images of h x w pixels, flattened [n][h][w]
    int n, h, w;
    int64_t npix;
};

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// One 3x3 convolution (stride 1, zero padding 1).
struct LayerShape {
    int cin;          // input channels used (<= cin8)
    int cin8;         // stored input channels: c0 + c1, multiples of 8
    int cout, cout8;  // output channels and their stored count (multiple of 8)
    int cout_n;       // MMA N of the forward GEMM: round_up(cout, 16)
    int cin_n;        // MMA N of the data-gradient GEMM: round_up(cin8, 16)
    int k_pad;        // round_up(9 * cin8, 64)
    int k2_pad;       // round_up(9 * cout8, 64)
};

struct ConvArgs {
    Geo g;                          // output grid (= input grid of the convolution)
    // input: channels [0, c0) from x0 (upsampled 2x when up0), [c0, c0+c1) from x1
    const __nv_bfloat16* x0;
    const __nv_bfloat16* x1;
    int c0, c1, c0s, c1s;           // channel counts and strides (elements per pixel)
    int up0;
    int cin8, cout, cout8;
    int k_pad, k2_pad;
    const __nv_bfloat16* w;         // [cout_n][k_pad]
    const __nv_bfloat16* wt;        // [cin_n][k2_pad]
    const float* bias;
    int relu;
    // forward outputs
    __nv_bfloat16* yout;            // [pix][cout8] BF16
    float* yf;                      // or FP32 [pix][cout8] (last layer)
    // backward inputs: dY (FP32 [pix][cout8]) and the forward output Y for relu'
    const float* dy;
    const __nv_bfloat16* y;
    // data-gradient outputs (accumulated): d x0 (low-res when up0, atomics), d x1
    float* dx0;
    float* dx1;
    // weight-gradient output (accumulated, FP32 [cout][k_pad])
    float* dw;
    // forward of an upsample + concatenation layer: room for its upsampled
    // source at full resolution ([pix][c0s] BF16), or null
    __nv_bfloat16* up_scratch;
    int bn;                         // MMA N of this launch (<= 256, multiple of 16)
    int n_tiles;                    // N tiles (forward/data grad: grid.y; weight grad: grid.x)
};

size_t conv_smem_bytes(int bn);
cudaError_t launch_wait_probe(uint32_t limit, int* err_flag, cudaStream_t st);
cudaError_t launch_conv(int mode, const ConvArgs& a, int wgrad_splits, int* err_flag, cudaStream_t st);
void launch_pool_fwd(const __nv_bfloat16* x, __nv_bfloat16* y, const Geo& lo, int c8, cudaStream_t st);
void launch_pool_bwd(const __nv_bfloat16* x, const float* dy, float* dx, const Geo& lo, int c8, cudaStream_t st);
void launch_pack(const float* rad, const float* aov, __nv_bfloat16* x, int w, int h, int wp, int hp, int64_t img_off,
                 cudaStream_t st);
void launch_unpack(const float* y, const float* aov, float* out, int w, int h, int wp, int64_t img_off,
                   cudaStream_t st);
void launch_l1(const float* y, const float* tgt, const float* aov, float* dy, int w, int h, int wp, int64_t img_off,
               float inv_count, double* loss, cudaStream_t st);
void launch_bias_grad(const float* dy, const __nv_bfloat16* y, bool relu, const Geo& g, int cout, int cout8, float* db,
                      cudaStream_t st);
void launch_refresh(const LayerShape& L, const float* w32, __nv_bfloat16* w16, __nv_bfloat16* wt16, cudaStream_t st);
void launch_adam(const LayerShape& L, float* w32, const float* gw, float* mw, float* vw, __nv_bfloat16* w16,
                 __nv_bfloat16* wt16, float* b32, const float* gb, float* mb, float* vb, float lr, int t,
                 cudaStream_t st);

}  // namespace dn
}  // namespace ohao
