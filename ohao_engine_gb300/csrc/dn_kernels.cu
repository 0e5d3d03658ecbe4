// dn_kernels.cu -- kernels of the BF16 U-Net denoiser on tcgen05 tensor cores.
//
// Every 3x3 convolution (forward, data gradient, weight gradient) is one
// implicit GEMM on tcgen05.mma: the CTA's 128 threads gather the operand
// tiles from NHWC activations straight into shared memory in the canonical
// no-swizzle layout (zero padding, nearest 2x upsampling and the skip
// concatenation are folded into the gather), one thread issues the MMAs into
// an FP32 accumulator in tensor memory, two shared-memory stages overlap the
// gather of chunk k+1 with the MMAs of chunk k (tcgen05.commit -> mbarrier),
// and the epilogue reads the accumulator with tcgen05.ld and applies bias,
// ReLU and the BF16 store (forward), the scatter into the input gradients
// (data gradient), or FP32 atomics into the weight gradient.
//
// Shapes: BF16 activations are channel-blocked, [n][C8/8][h][w][8] with
// C8 = round_up(C, 8): the 8 channels [8 cb, 8 cb + 8) of pixel (n, y, x)
// are 16 bytes at element offset ((n * C8/8 + cb) * h * w + y * w + x) * 8,
// so a row of one channel block is contiguous (the neighbourhood fill of
// k_conv_ws copies 130-pixel runs with single bulk copies). Gradients are [pixels][C8] FP32. Weights W [cout_n][k_pad] BF16, k = tap*cin8 + ci
// (tap = 3*dy + dx), and the transposed copy Wt [cin_n][k2_pad],
// k2 = tap*cout8 + co, for the data gradient.
#include <cuda_bf16.h>

#include <algorithm>

#include "dn_types.hpp"
#include "umma.cuh"

namespace ohao {
namespace dn {

namespace {

constexpr int kThreads = 128;
constexpr int kBM = 128;     // rows of the accumulator (TMEM lanes)
constexpr int kBK = 64;      // K elements per stage (8 core-matrix columns)
constexpr int kStages = 2;

__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint4 u;
    __nv_bfloat162 h0 = __floats2bfloat162_rn(f[0], f[1]);
    __nv_bfloat162 h1 = __floats2bfloat162_rn(f[2], f[3]);
    __nv_bfloat162 h2 = __floats2bfloat162_rn(f[4], f[5]);
    __nv_bfloat162 h3 = __floats2bfloat162_rn(f[6], f[7]);
    u.x = *reinterpret_cast<uint32_t*>(&h0);
    u.y = *reinterpret_cast<uint32_t*>(&h1);
    u.z = *reinterpret_cast<uint32_t*>(&h2);
    u.w = *reinterpret_cast<uint32_t*>(&h3);
    return u;
}
__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}

// Pixel coordinates of the flattened [n][h][w] grid (pixel counts < 2^31).
struct Pix {
    int x, y, n;   // n < 0: outside the grid
};
__device__ __forceinline__ Pix pix_of(const Geo& g, int p) {
    Pix r;
    if (p >= g.npix) {
        r.x = r.y = 0;
        r.n = -1;
        return r;
    }
    r.x = p % g.w;
    const int t = p / g.w;
    r.y = t % g.h;
    r.n = t / g.h;
    return r;
}

// Element offset of channel block cb of pixel rem = y * w + x of image n in
// a channel-blocked tensor of cbs blocks and hw = h * w pixels per image.
__device__ __forceinline__ int64_t blk(int64_t n, int cb, int cbs, int64_t hw, int64_t rem) {
    return ((n * cbs + cb) * hw + rem) * 8;
}

// 8 input channels [c0, c0+8) of the (possibly upsampled + concatenated)
// convolution input at pixel (n, qy, qx) of the full-res grid.
__device__ __forceinline__ uint4 load_input8(const ConvArgs& a, int n, int qy, int qx, int c0) {
    if (c0 < a.c0) {
        if (a.up0) {   // nearest 2x upsample of a half-resolution source
            const int hw2 = (a.g.w >> 1);
            return *reinterpret_cast<const uint4*>(
                a.x0 + blk(n, c0 >> 3, a.c0s >> 3, static_cast<int64_t>(a.g.h >> 1) * hw2,
                           static_cast<int64_t>(qy >> 1) * hw2 + (qx >> 1)));
        }
        return *reinterpret_cast<const uint4*>(
            a.x0 + blk(n, c0 >> 3, a.c0s >> 3, static_cast<int64_t>(a.g.h) * a.g.w, static_cast<int64_t>(qy) * a.g.w + qx));
    }
    if (c0 - a.c0 < a.c1)
        return *reinterpret_cast<const uint4*>(a.x1 + blk(n, (c0 - a.c0) >> 3, a.c1s >> 3,
                                                          static_cast<int64_t>(a.g.h) * a.g.w,
                                                          static_cast<int64_t>(qy) * a.g.w + qx));
    return make_uint4(0, 0, 0, 0);
}

// 8 channels of dZ = dY * relu'(Y) at pixel q, as BF16.
__device__ __forceinline__ uint4 load_dz8(const ConvArgs& a, int64_t q, int c0) {
    if (c0 >= a.cout8) return make_uint4(0, 0, 0, 0);
    const float4* gp = reinterpret_cast<const float4*>(a.dy + q * a.cout8 + c0);
    const float4 g0 = gp[0], g1 = gp[1];
    float f[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
    if (a.relu) {
        const int64_t hw = static_cast<int64_t>(a.g.h) * a.g.w;
        const int64_t n = q / hw;
        float yv[8];
        unpack8(*reinterpret_cast<const uint4*>(a.y + blk(n, c0 >> 3, a.cout8 >> 3, hw, q - n * hw)), yv);
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (!(yv[i] > 0.0f)) f[i] = 0.0f;
    }
    return pack8(f);
}

struct Smem {
    uint64_t bar[kStages];
    uint64_t done;
    uint32_t tmem;
};

constexpr int kRowsPerThread = (kBM * 8) / kThreads;   // 8

// Fills stage buffers for K chunk kc. A: kBM rows; B: bn rows.
// Forward / data gradient: thread t always fills the rows
// m = (2 it + t/64) * 8 + t%8 (it = 0..7) at vector t/8 % 8 of the chunk, so
// their pixel coordinates (rows[]) are computed once per tile. Weight
// gradient: px[] holds the coordinates of the chunk's 64 pixels.
template <int kMode>
__device__ __forceinline__ void gather(const ConvArgs& a, const Pix (&rows)[kRowsPerThread], const Pix* px, int ntile,
                                       int kc, int64_t kbase, uint8_t* sa, uint8_t* sb, int bn) {
    const int t = threadIdx.x;
    if constexpr (kMode == kFwd || kMode == kDgrad) {
        // A, K-major: offset(row m, vector kb) = ((m/8)*8 + kb)*128 + (m%8)*16 = L*16
        const int vpt = (kMode == kFwd ? a.cin8 : a.cout8) >> 3;
        const int kv = kc * 8 + ((t >> 3) & 7);
        const bool kvalid = kv < 9 * vpt;
        const int tap = kvalid ? kv / vpt : 0;
        const int c0 = kvalid ? (kv - tap * vpt) * 8 : 0;
        const int sgn = kMode == kFwd ? 1 : -1;
        const int ty = sgn * (tap / 3 - 1), tx = sgn * (tap % 3 - 1);
        uint4 v[kRowsPerThread];
#pragma unroll
        for (int it = 0; it < kRowsPerThread; ++it) {
            v[it] = make_uint4(0, 0, 0, 0);
            const int qy = rows[it].y + ty, qx = rows[it].x + tx;
            if (kvalid && rows[it].n >= 0 && qy >= 0 && qy < a.g.h && qx >= 0 && qx < a.g.w) {
                const int q = (rows[it].n * a.g.h + qy) * a.g.w + qx;
                if constexpr (kMode == kFwd) v[it] = load_input8(a, rows[it].n, qy, qx, c0);
                else v[it] = load_dz8(a, q, c0);
            }
        }
#pragma unroll
        for (int it = 0; it < kRowsPerThread; ++it) *reinterpret_cast<uint4*>(sa + (it * kThreads + t) * 16) = v[it];
        // B, K-major weights: row n, vector kb
        const __nv_bfloat16* wsrc = (kMode == kFwd) ? a.w : a.wt;
        const int kpad = (kMode == kFwd) ? a.k_pad : a.k2_pad;
        for (int L = t; L < bn * 8; L += kThreads) {
            const int r = L & 7, kb = (L >> 3) & 7, nb = L >> 6;
            const int n = nb * 8 + r;
            const uint4 v = *reinterpret_cast<const uint4*>(wsrc + static_cast<int64_t>(n) * kpad + kc * kBK + kb * 8);
            *reinterpret_cast<uint4*>(sb + L * 16) = v;
        }
    } else {
        // weight gradient: K = pixels. A (MN-major): row k = pixel, 16 B = 8 output channels.
        // offset(mn_blk, k_blk) = (k_blk*16 + mn_blk)*128 + (k%8)*16 = L*16; thread t
        // always loads channels ((t/8) % 16) * 8 of pixel kbase + 8 it + t%8.
        uint4 v[kRowsPerThread];
        const int c0a = ((t >> 3) & 15) * 8;
#pragma unroll
        for (int it = 0; it < kRowsPerThread; ++it) {
            const int64_t p = kbase + it * 8 + (t & 7);
            v[it] = p < a.g.npix ? load_dz8(a, p, c0a) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int it = 0; it < kRowsPerThread; ++it) *reinterpret_cast<uint4*>(sa + (it * kThreads + t) * 16) = v[it];
        // B (MN-major): row k = pixel, 16 B = 8 consecutive features (tap, ci..ci+7)
        const int nb_count = bn / 8;
        for (int L = t; L < bn * 8; L += kThreads) {
            const int k = L >> 3;
            const int nb = k % nb_count, kb = k / nb_count;
            const Pix pp = px[kb * 8 + (L & 7)];
            const int f = ntile * a.bn + nb * 8;
            uint4 w = make_uint4(0, 0, 0, 0);
            if (pp.n >= 0 && f < 9 * a.cin8) {
                const int tap = f / a.cin8, c0 = f - tap * a.cin8;
                const int qy = pp.y + tap / 3 - 1, qx = pp.x + tap % 3 - 1;
                if (qy >= 0 && qy < a.g.h && qx >= 0 && qx < a.g.w)
                    w = load_input8(a, pp.n, qy, qx, c0);
            }
            *reinterpret_cast<uint4*>(sb + L * 16) = w;
        }
    }
}

template <int kMode>
__global__ void __launch_bounds__(kThreads) k_conv(ConvArgs a, int* err_flag) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    __shared__ Smem ss;
    const int bn = a.bn;
    const uint32_t a_bytes = kBM * kBK * 2, b_bytes = static_cast<uint32_t>(bn) * kBK * 2;
    uint8_t* stage_a[kStages];
    uint8_t* stage_b[kStages];
    for (int s = 0; s < kStages; ++s) {
        stage_a[s] = dsm + s * (a_bytes + b_bytes);
        stage_b[s] = stage_a[s] + a_bytes;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t ncols = 32;
    while (ncols < static_cast<uint32_t>(bn)) ncols <<= 1;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) umma::mbar_init(&ss.bar[s], 1);
        umma::mbar_init(&ss.done, 1);
        umma::mbar_fence_init();
    }
    if (warp == 0) umma::tmem_alloc(&ss.tmem, ncols);
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    const uint32_t tmem = ss.tmem;

    // tiles: fwd/dgrad -> blockIdx.x = pixel tile, blockIdx.y = N tile
    //        wgrad     -> blockIdx.x = N tile, blockIdx.y = pixel split
    int64_t mtile;
    int ntile, kchunks;
    int64_t wg_first = 0, wg_last = 0;
    if constexpr (kMode == kWgrad) {
        ntile = blockIdx.x;
        const int64_t nchunks_total = (a.g.npix + kBK - 1) / kBK;
        const int64_t per = (nchunks_total + gridDim.y - 1) / gridDim.y;
        wg_first = blockIdx.y * per;
        wg_last = wg_first + per < nchunks_total ? wg_first + per : nchunks_total;
        kchunks = wg_last > wg_first ? static_cast<int>(wg_last - wg_first) : 0;
        mtile = wg_first;
    } else {
        mtile = blockIdx.x;
        ntile = blockIdx.y;
        kchunks = (kMode == kFwd ? a.k_pad : a.k2_pad) / kBK;
    }
    const uint32_t idesc = umma::idesc_bf16(kBM, static_cast<uint32_t>(bn), kMode == kWgrad, kMode == kWgrad);
    // per-thread pixel rows (forward / data gradient) or the chunk's pixels (weight gradient)
    Pix rows[kRowsPerThread];
    __shared__ Pix s_px[kBK];
    if constexpr (kMode != kWgrad) {
#pragma unroll
        for (int it = 0; it < kRowsPerThread; ++it)
            rows[it] = pix_of(a.g, static_cast<int>(mtile * kBM) + (2 * it + (threadIdx.x >> 6)) * 8 + (threadIdx.x & 7));
    }
    bool ok = true;
    for (int kc = 0; kc < kchunks && ok; ++kc) {
        const int s = kc % kStages;
        if (kc >= kStages) ok = umma::mbar_wait(&ss.bar[s], ((kc / kStages) - 1) & 1);
        if constexpr (kMode == kWgrad) {
            if (threadIdx.x < kBK) s_px[threadIdx.x] = pix_of(a.g, static_cast<int>((wg_first + kc) * kBK) + threadIdx.x);
        }
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        gather<kMode>(a, rows, s_px, ntile, kc, (wg_first + kc) * kBK, stage_a[s], stage_b[s], bn);
        umma::fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            umma::tc_fence_after();
            const uint32_t sa = umma::smem_u32(stage_a[s]), sb = umma::smem_u32(stage_b[s]);
#pragma unroll
            for (int i = 0; i < kBK / 16; ++i) {
                uint64_t da, db;
                if constexpr (kMode == kWgrad) {
                    // MN-major, no swizzle: SBO = stride between 8-element M/N groups (128 B),
                    // LBO = stride between 8-row K groups
                    da = umma::smem_desc(sa + i * 2 * 2048, 2048, 128);
                    db = umma::smem_desc(sb + i * 2 * (bn / 8) * 128, (bn / 8) * 128, 128);
                } else {
                    // K-major: LBO = 128 (next 8 K), SBO = 1024 (next 8 rows)
                    da = umma::smem_desc(sa + i * 256, 128, 1024);
                    db = umma::smem_desc(sb + i * 256, 128, 1024);
                }
                umma::mma_bf16(tmem, da, db, idesc, kc > 0 || i > 0);
            }
            umma::mma_commit(&ss.bar[s]);
        }
    }
    // drain: the last commit covers every MMA issued before it
    if (threadIdx.x == 0) umma::mma_commit(&ss.done);
    bool drained = umma::mbar_wait(&ss.done, 0);
    if (!ok || !drained) {
        if (threadIdx.x == 0) atomicOr(err_flag, 2);
    }
    umma::tc_fence_after();
    const bool good = __syncthreads_and(ok && drained);
    if (good && kchunks > 0) {
        const int row = warp * 32 + lane;
        const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
        if constexpr (kMode == kFwd) {
            const int64_t p = mtile * kBM + row;
            const int64_t hw = static_cast<int64_t>(a.g.h) * a.g.w;
            const int64_t pn = p / hw;
            for (int c = 0; c < bn; c += 8) {
                float v[8];
                umma::tmem_ld8(trow + c, v);
                const int co = ntile * a.bn + c;
                if (p < a.g.npix && co < a.cout8) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        v[i] += (co + i < a.cout) ? a.bias[co + i] : 0.0f;
                        if (a.relu) v[i] = fmaxf(v[i], 0.0f);
                        if (co + i >= a.cout) v[i] = 0.0f;
                    }
                    if (a.yf) {
                        float4* o = reinterpret_cast<float4*>(a.yf + p * a.cout8 + co);
                        o[0] = make_float4(v[0], v[1], v[2], v[3]);
                        o[1] = make_float4(v[4], v[5], v[6], v[7]);
                    } else {
                        *reinterpret_cast<uint4*>(a.yout + blk(pn, co >> 3, a.cout8 >> 3, hw, p - pn * hw)) = pack8(v);
                    }
                }
            }
        } else if constexpr (kMode == kDgrad) {
            // tcgen05.ld is warp-collective (.sync.aligned): every lane loads,
            // the row test comes after
            const int64_t p = mtile * kBM + row;
            const bool live = p < a.g.npix;
            const int64_t pc = live ? p : 0;
            const int x = static_cast<int>(pc % a.g.w);
            const int64_t tt = pc / a.g.w;
            const int y = static_cast<int>(tt % a.g.h);
            const int64_t n = tt / a.g.h;
            for (int c = 0; c < bn; c += 8) {
                float v[8];
                umma::tmem_ld8(trow + c, v);
                const int ci = ntile * a.bn + c;
                if (live) {
                    if (ci < a.c0) {
                        if (a.up0) {
                            const int64_t lq = (n * (a.g.h / 2) + y / 2) * (a.g.w / 2) + x / 2;
                            float* d = a.dx0 + lq * a.c0s + ci;
#pragma unroll
                            for (int i = 0; i < 8; ++i) atomicAdd(d + i, v[i]);
                        } else {
                            float* d = a.dx0 + p * a.c0s + ci;
#pragma unroll
                            for (int i = 0; i < 8; ++i) d[i] += v[i];
                        }
                    } else if (ci - a.c0 < a.c1) {
                        float* d = a.dx1 + p * a.c1s + (ci - a.c0);
#pragma unroll
                        for (int i = 0; i < 8; ++i) d[i] += v[i];
                    }
                }
            }
        } else {
            // weight gradient: row = output channel, columns = features
            // (warp-collective load first, row test after)
            for (int c = 0; c < bn; c += 8) {
                float v[8];
                umma::tmem_ld8(trow + c, v);
                const int f = ntile * a.bn + c;
                if (row < a.cout) {
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        if (f + i < 9 * a.cin8 && v[i] != 0.0f)
                            atomicAdd(a.dw + static_cast<int64_t>(row) * a.k_pad + f + i, v[i]);
                }
            }
        }
    }
    // A CTA must not exit holding tensor memory, so the columns are freed even
    // after a wait gave up; MMAs still in flight then may write columns that
    // are no longer this CTA's. The host reports OHAO_ERR_TIMEOUT and the
    // denoiser context is to be destroyed and re-created after it.
    umma::tc_fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}

// Forward convolution on rows of at least kHaloMinW pixels (single-source
// inputs, see launch_conv). A CTA's 128
// output pixels are x0 .. x0+127 of one image row; their 3 x 130-pixel
// neighbourhood is loaded once into shared memory, channel-blocked as
// [row 0..2][channel block][x 0..129][8 channels] (16 B per entry), and the
// A operand of every tap is a descriptor into it: a core matrix is 8
// consecutive x (16 B apart), the next 8 output pixels start 128 B on (SBO)
// and the next 8 channels kHaloX * 16 B on (LBO); tap (dy, dx) starts at row
// dy, x offset dx. Each input pixel is read 3 times per row of tiles instead
// of once per tap and channel chunk. Weights stream through two stages in
// 64-wide K chunks as in k_conv; a K step of 16 never crosses a tap because
// cin8 is a multiple of 16 on this path.
constexpr int kHaloX = kBM + 2;
constexpr int kHaloMinW = 96;

size_t halo_bytes(int cin8) { return static_cast<size_t>(3) * (cin8 / 8) * kHaloX * 16; }

__global__ void __launch_bounds__(kThreads) k_conv_halo(ConvArgs a, int* err_flag) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    __shared__ Smem ss;
    const int bn = a.bn;
    const int cb_count = a.cin8 / 8;
    const uint32_t hbytes = static_cast<uint32_t>(3 * cb_count * kHaloX * 16);
    const uint32_t b_off = (hbytes + 1023u) & ~1023u;
    const uint32_t b_bytes = static_cast<uint32_t>(bn) * kBK * 2;
    uint8_t* halo = dsm;
    uint8_t* stage_b[kStages];
    for (int s = 0; s < kStages; ++s) stage_b[s] = dsm + b_off + s * b_bytes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t ncols = 32;
    while (ncols < static_cast<uint32_t>(bn)) ncols <<= 1;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) umma::mbar_init(&ss.bar[s], 1);
        umma::mbar_init(&ss.done, 1);
        umma::mbar_fence_init();
    }
    if (warp == 0) umma::tmem_alloc(&ss.tmem, ncols);
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    const uint32_t tmem = ss.tmem;

    // tile -> (image n, row y, first column x0)
    const int xtiles = (a.g.w + kBM - 1) / kBM;
    const int x0 = static_cast<int>(blockIdx.x % xtiles) * kBM;
    const int ny = static_cast<int>(blockIdx.x / xtiles);
    const int y = ny % a.g.h, n = ny / a.g.h;
    // the neighbourhood, zero outside the image (padding 1); 8 independent
    // 16-byte loads in flight per thread before their shared-memory stores
    const int items = 3 * kHaloX * cb_count;
    constexpr int kBatch = 8;
    for (int base = 0; base < items; base += kThreads * kBatch) {
        uint4 v[kBatch];
        uint32_t dst[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int i = base + u * kThreads + static_cast<int>(threadIdx.x);
            v[u] = make_uint4(0, 0, 0, 0);
            dst[u] = 0xFFFFFFFFu;
            if (i < items) {
                const int cb = i % cb_count, rj = i / cb_count;
                const int j = rj % kHaloX, r = rj / kHaloX;
                const int qy = y - 1 + r, qx = x0 - 1 + j;
                dst[u] = static_cast<uint32_t>(((r * cb_count + cb) * kHaloX + j) * 16);
                if (qy >= 0 && qy < a.g.h && qx >= 0 && qx < a.g.w)
                    v[u] = load_input8(a, n, qy, qx, cb * 8);
            }
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
            if (dst[u] != 0xFFFFFFFFu) *reinterpret_cast<uint4*>(halo + dst[u]) = v[u];
    }
    const uint32_t idesc = umma::idesc_bf16(kBM, static_cast<uint32_t>(bn), false, false);
    const uint32_t hbase = umma::smem_u32(halo);
    const int kchunks = a.k_pad / kBK;
    const int kreal = 9 * a.cin8;
    // A descriptor offset (16-byte units) of each K step of 16: descriptors
    // are linear in the start address, so the MMA loop adds it to a base
    __shared__ uint32_t s_off[9 * 256 / 16];
    for (int k = threadIdx.x; k < kreal / 16; k += kThreads) {
        const int k0 = k * 16;
        const int tap = k0 / a.cin8, cb = (k0 - tap * a.cin8) >> 3;
        const int dy = tap / 3, dx = tap % 3;
        s_off[k] = static_cast<uint32_t>(((dy * cb_count + cb) * kHaloX + dx) * 16) >> 4;
    }
    const uint64_t da0 = umma::smem_desc(hbase, kHaloX * 16, 128);
    bool ok = true;
    for (int kc = 0; kc < kchunks && ok; ++kc) {
        const int s = kc % kStages;
        if (kc >= kStages) ok = umma::mbar_wait(&ss.bar[s], ((kc / kStages) - 1) & 1);
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        uint8_t* sb = stage_b[s];
        for (int L = threadIdx.x; L < bn * 8; L += kThreads) {
            const int r = L & 7, kb = (L >> 3) & 7, nb = L >> 6;
            const uint4 v =
                *reinterpret_cast<const uint4*>(a.w + static_cast<int64_t>(nb * 8 + r) * a.k_pad + kc * kBK + kb * 8);
            *reinterpret_cast<uint4*>(sb + L * 16) = v;
        }
        umma::fence_async_smem();   // also publishes the neighbourhood before the first MMA
        __syncthreads();
        if (threadIdx.x == 0) {
            umma::tc_fence_after();
            const uint32_t sbu = umma::smem_u32(sb);
#pragma unroll
            for (int i = 0; i < kBK / 16; ++i) {
                const int k0 = kc * kBK + i * 16;
                if (k0 >= kreal) break;   // zero-padded tail of K
                const uint64_t db = umma::smem_desc(sbu + i * 256, 128, 1024);
                umma::mma_bf16(tmem, da0 + s_off[k0 >> 4], db, idesc, k0 > 0);
            }
            umma::mma_commit(&ss.bar[s]);
        }
    }
    if (threadIdx.x == 0) umma::mma_commit(&ss.done);
    const bool drained = umma::mbar_wait(&ss.done, 0);
    if (!ok || !drained) {
        if (threadIdx.x == 0) atomicOr(err_flag, 2);
    }
    umma::tc_fence_after();
    const bool good = __syncthreads_and(ok && drained);
    if (good && kchunks > 0) {
        const int row = warp * 32 + lane;
        const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
        const bool live = x0 + row < a.g.w;
        const int64_t p = (static_cast<int64_t>(n) * a.g.h + y) * a.g.w + x0 + row;
        for (int c = 0; c < bn; c += 8) {
            float v[8];
            umma::tmem_ld8(trow + c, v);   // warp-collective: every lane loads, the row test comes after
            if (live && c < a.cout8) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    v[i] += (c + i < a.cout) ? a.bias[c + i] : 0.0f;
                    if (a.relu) v[i] = fmaxf(v[i], 0.0f);
                    if (c + i >= a.cout) v[i] = 0.0f;
                }
                if (a.yf) {
                    float4* o = reinterpret_cast<float4*>(a.yf + p * a.cout8 + c);
                    o[0] = make_float4(v[0], v[1], v[2], v[3]);
                    o[1] = make_float4(v[4], v[5], v[6], v[7]);
                } else {
                    *reinterpret_cast<uint4*>(a.yout + blk(n, c >> 3, a.cout8 >> 3, static_cast<int64_t>(a.g.h) * a.g.w,
                                                           static_cast<int64_t>(y) * a.g.w + x0 + row)) = pack8(v);
                }
            }
        }
    }
    umma::tc_fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}

// Forward convolution with bulk-copied neighbourhoods, warp-specialised and
// persistent (the wide levels' layers; the upsample + concatenation layers
// after their upsampled source is written out at full resolution by
// k_upsample2). A tile is R image rows y0 .. y0+R-1 (R = 1, 2 or 4) of 128
// output pixels x0 .. x0+127; its (R+2) x 130-pixel input neighbourhood is
// laid out [channel block][row 0..R+1][x 0..129][8 channels] (one slab of
// ws_slab(R) bytes per channel block). In the channel-blocked layout a row
// of a channel block is contiguous, so the fill is one cp.async.bulk per
// (channel block, row), with zeros written where the neighbourhood leaves
// the image (the padding). Tap descriptors read it in place: output row r,
// tap (dy, dx), channel block cb starts at cb * slab + ((r + dy) * 130 + dx)
// * 16, SBO 128 B (the next 8 pixels), LBO slab (the next 8 channels). The R
// rows share the fill ((R+2)/R input rows per output row instead of 3). The
// layer's weights and bias stay in shared memory. Roles: warp 0 fills a ring
// of nstages neighbourhood buffers, warp 1 issues the MMAs of a tile into
// one of two sets of R tensor-memory accumulators, warps 2-9 (two per
// 32-lane quarter of tensor memory, alternate rows) read the accumulators,
// add the bias, apply ReLU and store while the next tile is being
// multiplied. mbarriers hand over each buffer and accumulator set; every
// wait is bounded and also ends when another role has given up (ws.abort).
constexpr int kWsX = kBM + 2;   // neighbourhood width: 128 output pixels and the two side columns
constexpr int kWsEpiWarps = 8;        // two per 32-lane quarter of tensor memory
constexpr int kWsThreads = 64 + 32 * kWsEpiWarps;   // producer, MMA issuer, epilogue
constexpr int kWsMaxStages = 4;

__host__ __device__ inline uint32_t ws_slab(int rows) {   // (R+2) * 130 * 16 B, rounded up to 128 B
    return (static_cast<uint32_t>(rows + 2) * kWsX * 16u + 127u) & ~127u;
}

constexpr int kWsMaxKSteps = 9 * 256 / 16;   // K steps of 16 for cin8 <= 256

struct WsSmem {
    // descriptor offsets (16-byte units) of each K step: A within a
    // neighbourhood buffer (channel block, tap), B within the weights
    uint32_t off_a[kWsMaxKSteps], off_b[kWsMaxKSteps];
    float bias[256];   // the layer's bias, zero past cout
    uint64_t full[kWsMaxStages], empty[kWsMaxStages];
    uint64_t acc_full[2], acc_empty[2];
    uint64_t drain;
    uint32_t tmem;
    int abort;
};

// weights after the nstages neighbourhood buffers, on a 1024-byte boundary
__host__ __device__ inline uint32_t ws_weights_off(int cb_total, int nstages, int rows) {
    return (static_cast<uint32_t>(nstages) * static_cast<uint32_t>(cb_total) * ws_slab(rows) + 1023u) & ~1023u;
}
__host__ __device__ inline uint32_t ws_smem_bytes(int cb_total, int nstages, int rows, int bn, int k_pad) {
    return ws_weights_off(cb_total, nstages, rows) +
           static_cast<uint32_t>(k_pad / kBK) * static_cast<uint32_t>(bn) * kBK * 2;
}

// bounded wait that also gives up when another role has aborted
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
    for (uint32_t i = 0; i < umma::kSpinLimit; ++i) {
        if (umma::mbar_try_wait(bar, parity)) return true;
        if ((i & 63u) == 63u && *abort) return false;
    }
    *abort = 1;
    return false;
}

__global__ void __launch_bounds__(kWsThreads) k_conv_ws(ConvArgs a, const __nv_bfloat16* __restrict__ src_a,
                                                        const __nv_bfloat16* __restrict__ src_b, int cb_a, int cbs_a,
                                                        int cbs_b, int ntiles, int nstages, int rows, int co0,
                                                        int stack, int* err_flag) {
    extern __shared__ __align__(1024) uint8_t dsm_raw[];
    __shared__ WsSmem ws;
    // offsets are from a 1024-byte aligned base (the copies need 16-byte
    // alignment); the launch adds 1024 bytes of slack
    uint8_t* dsm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023u) & ~uintptr_t{1023});
    const int bn = a.bn;
    const int cb_total = a.cin8 / 8;
    const uint32_t slab = ws_slab(rows);
    const uint32_t w_off = ws_weights_off(cb_total, nstages, rows);
    const uint32_t stage_bytes = static_cast<uint32_t>(cb_total) * slab;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t ncols = 32;
    while (ncols < static_cast<uint32_t>(bn)) ncols <<= 1;
    // one accumulator set: R accumulators of ncols columns; stacked (see
    // below): R + 4 slots of bn columns, slot R + 1 - r for output row r
    // (r = -2 .. R+1), rounded up to a power of two
    uint32_t set_cols = static_cast<uint32_t>(rows) * ncols;
    if (stack) {
        set_cols = 32;
        while (set_cols < static_cast<uint32_t>((rows + 4) * bn)) set_cols <<= 1;
    }
    const int cbh = cb_total >> 1;   // K steps of 16 channels per tap
    if (threadIdx.x == 0) {
        for (int s = 0; s < nstages; ++s) {
            umma::mbar_init(&ws.full[s], 1);
            umma::mbar_init(&ws.empty[s], 1);
        }
        for (int k = 0; k < 2; ++k) {
            umma::mbar_init(&ws.acc_full[k], 1);
            umma::mbar_init(&ws.acc_empty[k], kWsEpiWarps);
        }
        umma::mbar_init(&ws.drain, 1);
        ws.abort = 0;
        umma::mbar_fence_init();
    }
    if (warp == 0) umma::tmem_alloc(&ws.tmem, 2 * set_cols);
    // resident weights: chunk kc of 64 K at w_off + kc * bn * 128, in the
    // K-major core-matrix order of k_conv (row n, 16-byte vector kb at
    // ((n/8)*8 + kb)*128 + (n%8)*16)
    const int ksteps = 9 * a.cin8 / 16;
    for (int k = threadIdx.x; k < ksteps; k += kWsThreads) {
        const int k0 = k * 16;
        const int tap = k0 / a.cin8, cb = (k0 - tap * a.cin8) >> 3;
        const int dy = tap / 3, dx = tap - 3 * (tap / 3);
        ws.off_a[k] = (static_cast<uint32_t>(cb) * slab + static_cast<uint32_t>((dy * kWsX + dx) * 16)) >> 4;
        ws.off_b[k] = (static_cast<uint32_t>(k0 / kBK) * static_cast<uint32_t>(bn) * 128u + ((k0 % kBK) / 16) * 256u) >> 4;
    }
    for (int c = threadIdx.x; c < bn; c += kWsThreads) ws.bias[c] = co0 + c < a.cout ? a.bias[co0 + c] : 0.0f;
    if (!stack) {
        const int kchunks = a.k_pad / kBK;
        for (int L = threadIdx.x; L < kchunks * bn * 8; L += kWsThreads) {
            const int kc = L / (bn * 8), l = L - kc * bn * 8;
            const int r = l & 7, kb = (l >> 3) & 7, nb = l >> 6;
            *reinterpret_cast<uint4*>(dsm + w_off + static_cast<uint32_t>(L) * 16) = *reinterpret_cast<const uint4*>(
                a.w + static_cast<int64_t>(co0 + nb * 8 + r) * a.k_pad + kc * kBK + kb * 8);
        }
    } else {
        // stacked weights: for each (dx, channel-block pair c) a B tile of
        // 3 bn rows (row dy * bn + co: the tap (dy, dx) of output channel co)
        // x 16 channels, K-major core matrices (8 rows x 16 B; LBO 128 B =
        // the next 8 channels, SBO 256 B = the next 8 rows)
        const int nrow = 3 * bn;
        for (int L = threadIdx.x; L < 3 * cbh * nrow * 2; L += kWsThreads) {
            const int blk_i = L / (nrow * 2), l = L - blk_i * nrow * 2;
            const int dx = blk_i / cbh, c = blk_i - dx * cbh;
            const int n = l >> 1, kb = l & 1;
            const int dy = n / bn, co = n - dy * bn;
            const uint32_t off = static_cast<uint32_t>(blk_i) * static_cast<uint32_t>(nrow) * 32u +
                                 static_cast<uint32_t>(((n >> 3) * 2 + kb) * 128 + (n & 7) * 16);
            *reinterpret_cast<uint4*>(dsm + w_off + off) = *reinterpret_cast<const uint4*>(
                a.w + static_cast<int64_t>(co0 + co) * a.k_pad + (dy * 3 + dx) * a.cin8 + c * 16 + kb * 8);
        }
    }
    umma::fence_async_smem();
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    const uint32_t tmem = ws.tmem;
    if (stack) {   // the accumulators start at zero: every MMA of the stacked form adds
        if (warp >= 2) {
            const uint32_t q = static_cast<uint32_t>(warp & 3), half = static_cast<uint32_t>((warp - 2) >> 2);
            for (uint32_t col = half * 32u; col < 2u * set_cols; col += 64u)
                umma::tmem_zero32(tmem + ((q * 32u) << 16) + col);
            umma::tmem_st_wait();
        }
        umma::tc_fence_before();
        __syncthreads();
        umma::tc_fence_after();
    }
    const int xtiles = (a.g.w + kBM - 1) / kBM;
    const int ygroups = (a.g.h + rows - 1) / rows;
    const int first = static_cast<int>(blockIdx.x), step = static_cast<int>(gridDim.x);
    volatile int* abort = &ws.abort;

    if (warp == 0) {
        // producer: the neighbourhood of tile i into stage i % nstages, one
        // bulk copy per (channel block, row) -- a row of a channel block is
        // contiguous in the channel-blocked layout -- and zeros where the
        // neighbourhood leaves the image (the padding)
        const int nitems = cb_total * (rows + 2);
        const int64_t hw = static_cast<int64_t>(a.g.h) * a.g.w;
        int i = 0, issued = 0;
        for (int t = first; t < ntiles; t += step, ++i) {
            const int s = i % nstages;
            if (i >= nstages &&
                !__all_sync(0xFFFFFFFFu, ws_wait(&ws.empty[s], static_cast<uint32_t>(i / nstages - 1) & 1u, abort)))
                break;
            const int x0 = (t % xtiles) * kBM;
            const int ny = t / xtiles;
            const int y0 = (ny % ygroups) * rows, n = ny / ygroups;
            uint8_t* dst = dsm + static_cast<uint32_t>(s) * stage_bytes;
            const int lo = x0 - 1 > 0 ? x0 - 1 : 0;                              // valid columns lo..hi
            const int hi = x0 + kBM < a.g.w - 1 ? x0 + kBM : a.g.w - 1;
            const int j_lo = lo - (x0 - 1), j_hi = hi - (x0 - 1);                // their entries in a row
            const uint32_t nbytes = static_cast<uint32_t>(hi - lo + 1) * 16u;
            uint32_t mine = 0;
            for (int it = lane; it < nitems; it += 32) {
                const int cb = it / (rows + 2), r = it - cb * (rows + 2);
                const int y = y0 - 1 + r;
                uint4* rowp = reinterpret_cast<uint4*>(dst + static_cast<uint32_t>(cb) * slab +
                                                       static_cast<uint32_t>(r * kWsX) * 16u);
                if (y < 0 || y >= a.g.h) {
                    for (int j = 0; j < kWsX; ++j) rowp[j] = make_uint4(0, 0, 0, 0);
                } else {
                    for (int j = 0; j < j_lo; ++j) rowp[j] = make_uint4(0, 0, 0, 0);
                    for (int j = j_hi + 1; j < kWsX; ++j) rowp[j] = make_uint4(0, 0, 0, 0);
                    mine += nbytes;
                }
            }
            umma::fence_async_smem();   // the zeros, for the MMAs' async-proxy reads
            const uint32_t total = __reduce_add_sync(0xFFFFFFFFu, mine);
            __syncwarp();
            if (lane == 0) umma::mbar_arrive_expect_tx(&ws.full[s], total);
            __syncwarp();
            for (int it = lane; it < nitems; it += 32) {
                const int cb = it / (rows + 2), r = it - cb * (rows + 2);
                const int y = y0 - 1 + r;
                if (y < 0 || y >= a.g.h) continue;
                const __nv_bfloat16* src = cb < cb_a ? src_a + blk(n, cb, cbs_a, hw, static_cast<int64_t>(y) * a.g.w + lo)
                                                     : src_b + blk(n, cb - cb_a, cbs_b, hw,
                                                                   static_cast<int64_t>(y) * a.g.w + lo);
                umma::bulk_load(dst + static_cast<uint32_t>(cb) * slab + static_cast<uint32_t>(r * kWsX + j_lo) * 16u,
                                src, nbytes, &ws.full[s]);
            }
            issued = i + 1;
        }
        // copies in flight land before the CTA's shared memory is released:
        // the last nstages issued tiles' fills (bounded, regardless of abort)
        if (lane == 0)
            for (int k = issued - nstages > 0 ? issued - nstages : 0; k < issued; ++k)
                if (!umma::mbar_wait(&ws.full[k % nstages], static_cast<uint32_t>(k / nstages) & 1u))
                    atomicOr(err_flag, 2);
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer: tile i from stage i % nstages into accumulator set i & 1
            const uint32_t idesc = umma::idesc_bf16(kBM, static_cast<uint32_t>(stack ? 3 * bn : bn), false, false);
            // descriptors are linear in the start address (its low 14 bits,
            // in 16-byte units; every address here is below 256 KB), so a K
            // step's descriptor is a base plus the step's offset
            const uint64_t db0 = umma::smem_desc(umma::smem_u32(dsm + w_off), 128, 1024);
            int i = 0;
            for (int t = first; t < ntiles; t += step, ++i) {
                const int s = i % nstages, acc = i & 1;
                if (!ws_wait(&ws.full[s], static_cast<uint32_t>(i / nstages) & 1u, abort)) break;
                if (i >= 2 && !ws_wait(&ws.acc_empty[acc], static_cast<uint32_t>((i >> 1) - 1) & 1u, abort)) break;
                umma::tc_fence_after();
                const uint64_t da0 = umma::smem_desc(umma::smem_u32(dsm + static_cast<uint32_t>(s) * stage_bytes), slab, 128);
                if (!stack) {
                    for (int r = 0; r < rows; ++r) {
                        const uint32_t d = tmem + static_cast<uint32_t>(acc) * set_cols + static_cast<uint32_t>(r) * ncols;
                        const uint64_t dar = da0 + static_cast<uint64_t>(r * kWsX);   // output row r: input rows r + dy
#pragma unroll 4
                        for (int k = 0; k < ksteps; ++k)
                            umma::mma_bf16(d, dar + ws.off_a[k], db0 + ws.off_b[k], idesc, k > 0);
                    }
                } else {
                    // stacked: neighbourhood row ri (input row y0 - 1 + ri) times
                    // the three vertical taps at once -- N = 3 bn columns: the
                    // slots of output rows ri, ri - 1, ri - 2 (taps dy = 0, 1, 2),
                    // adjacent because slot(r) = R + 1 - r
                    const uint64_t dbs = umma::smem_desc(umma::smem_u32(dsm + w_off), 128, 256);
                    const uint64_t b_step = static_cast<uint64_t>(3 * bn * 32) >> 4;
                    for (int ri = 0; ri < rows + 2; ++ri) {
                        const uint32_t d = tmem + static_cast<uint32_t>(acc) * set_cols +
                                           static_cast<uint32_t>((rows + 1 - ri) * bn);
                        uint64_t db = dbs;
                        for (int dx = 0; dx < 3; ++dx) {
                            const uint64_t da = da0 + static_cast<uint64_t>(ri * kWsX + dx);
                            for (int c = 0; c < cbh; ++c) {
                                umma::mma_bf16(d, da + static_cast<uint64_t>(2 * c) * (slab >> 4), db, idesc, true);
                                db += b_step;
                            }
                        }
                    }
                }
                umma::mma_commit(&ws.empty[s]);       // the stage is read
                umma::mma_commit(&ws.acc_full[acc]);  // the accumulator set is complete
            }
            // every MMA issued has completed before the columns are freed
            // (bounded, regardless of abort)
            umma::mma_commit(&ws.drain);
            if (!umma::mbar_wait(&ws.drain, 0)) atomicOr(err_flag, 2);
        }
    } else {
        // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. +31 of the
        // output rows r = half, half + 2, ... of the tile (two warps per quarter)
        const int q = warp & 3, half = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const int64_t hw = static_cast<int64_t>(a.g.h) * a.g.w;
        const int cbo = a.cout8 >> 3;
        int i = 0;
        for (int t = first; t < ntiles; t += step, ++i) {
            const int acc = i & 1;
            // the whole warp leaves together (tcgen05.ld below is warp-collective)
            if (!__all_sync(0xFFFFFFFFu, ws_wait(&ws.acc_full[acc], static_cast<uint32_t>(i >> 1) & 1u, abort))) break;
            umma::tc_fence_after();
            const int x0 = (t % xtiles) * kBM;
            const int ny = t / xtiles;
            const int y0 = (ny % ygroups) * rows, n = ny / ygroups;
            for (int r = half; r < rows; r += 2) {
                const int y = y0 + r;
                const bool live = x0 + row < a.g.w && y < a.g.h;
                const int64_t rem = static_cast<int64_t>(y) * a.g.w + x0 + row;
                const uint32_t col = stack ? static_cast<uint32_t>((rows + 1 - r) * bn) : static_cast<uint32_t>(r) * ncols;
                const uint32_t trow = tmem + static_cast<uint32_t>(acc) * set_cols + col + (static_cast<uint32_t>(q * 32) << 16);
                for (int c0 = 0; c0 < bn; c0 += 32) {
                    float v[32];
                    // warp-collective: every lane loads, the row test comes after
                    if (bn - c0 >= 32) umma::tmem_ld32(trow + c0, v);
                    else umma::tmem_ld16(trow + c0, v);   // a 16-column slot: its neighbour is another row's
                    if (!live) continue;
#pragma unroll
                    for (int c8 = 0; c8 < 32; c8 += 8) {
                        const int c = c0 + c8, cg = co0 + c;   // this launch's and the layer's channel
                        if (cg >= a.cout8) break;
                        float o[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const float x = v[c8 + k] + ws.bias[c + k];   // bias is zero past cout
                            o[k] = a.relu ? fmaxf(x, 0.0f) : x;
                        }
                        if (a.yf) {
                            float4* op = reinterpret_cast<float4*>(a.yf + (n * hw + rem) * a.cout8 + cg);
                            op[0] = make_float4(o[0], o[1], o[2], o[3]);
                            op[1] = make_float4(o[4], o[5], o[6], o[7]);
                        } else {
                            *reinterpret_cast<uint4*>(a.yout + blk(n, cg >> 3, cbo, hw, rem)) = pack8(o);
                        }
                    }
                }
            }
            if (stack) {
                // back to zero for the set's next tile: the slots of this
                // warp's rows (read above) and, per half, two of the four
                // slots no output row reads (rows -2, -1, R, R+1)
                const uint32_t tq = tmem + static_cast<uint32_t>(acc) * set_cols + (static_cast<uint32_t>(q * 32) << 16);
                auto zero_slot = [&](int slot) {
                    for (int c = 0; c < bn; c += 16) umma::tmem_zero16(tq + static_cast<uint32_t>(slot * bn + c));
                };
                for (int r = half; r < rows; r += 2) zero_slot(rows + 1 - r);
                const int g0 = half ? rows + 2 : 0;
                zero_slot(g0);
                zero_slot(g0 + 1);
                umma::tmem_st_wait();
            }
            umma::tc_fence_before();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&ws.acc_empty[acc]);
        }
    }
    __syncwarp();
    umma::tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && ws.abort) atomicOr(err_flag, 2);
    if (warp == 0) umma::tmem_dealloc(tmem, 2 * set_cols);
}

// out(n, cb, y, x) = in(n, cb, y/2, x/2): the nearest 2x upsample of a
// channel-blocked BF16 tensor of cs channels, 8 channels (16 bytes) per thread.
__global__ void k_upsample2(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, Geo g, int cs) {
    const int cbs = cs / 8;
    const int64_t total = g.npix * cbs;
    const int w2 = g.w >> 1;
    const int64_t hw2 = static_cast<int64_t>(g.h >> 1) * w2;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(i % g.w);
        int64_t t = i / g.w;
        const int y = static_cast<int>(t % g.h);
        t /= g.h;   // n * cbs + cb
        reinterpret_cast<uint4*>(out)[i] =
            reinterpret_cast<const uint4*>(in)[t * hw2 + static_cast<int64_t>(y >> 1) * w2 + (x >> 1)];
    }
}

// ---- elementwise kernels ----
__global__ void k_pool_fwd(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, Geo lo, int c8) {
    const int64_t total = lo.npix * (c8 / 8);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        // i runs over the output in its channel-blocked order
        const int lx = static_cast<int>(i % lo.w);
        int64_t t = i / lo.w;
        const int ly = static_cast<int>(t % lo.h);
        t /= lo.h;   // n * (c8 / 8) + channel block
        const int W = lo.w * 2, H = lo.h * 2;
        float m[8];
        for (int j = 0; j < 8; ++j) m[j] = -3.0e38f;
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const int64_t q = (t * H + ly * 2 + dy) * W + lx * 2 + dx;
                float f[8];
                unpack8(*reinterpret_cast<const uint4*>(x + q * 8), f);
                for (int j = 0; j < 8; ++j) m[j] = fmaxf(m[j], f[j]);
            }
        *reinterpret_cast<uint4*>(y + i * 8) = pack8(m);
    }
}

// d x[argmax of each 2x2 window] += d y (first maximum in dy, dx order)
__global__ void k_pool_bwd(const __nv_bfloat16* __restrict__ x, const float* __restrict__ dy, float* __restrict__ dx,
                           Geo lo, int c8) {
    const int64_t total = lo.npix * c8;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(i % c8);
        const int64_t p = i / c8;
        const int lx = static_cast<int>(p % lo.w);
        const int64_t t = p / lo.w;
        const int ly = static_cast<int>(t % lo.h);
        const int64_t n = t / lo.h;
        const int W = lo.w * 2, H = lo.h * 2;
        float best = -3.0e38f;
        int64_t bq = 0;
        const int64_t hw = static_cast<int64_t>(H) * W;
        for (int ddy = 0; ddy < 2; ++ddy)
            for (int ddx = 0; ddx < 2; ++ddx) {
                const int64_t rem = static_cast<int64_t>(ly * 2 + ddy) * W + lx * 2 + ddx;
                const float v = __bfloat162float(x[blk(n, c >> 3, c8 >> 3, hw, rem) + (c & 7)]);
                if (v > best) { best = v; bq = n * hw + rem; }
            }
        dx[bq * c8 + c] += dy[p * c8 + c];
    }
}

// features: log1p(radiance), albedo, normal (encoded 0..1), 1/(1+depth) on hits
// Albedo demodulation of the radiance channels: the network sees and predicts
// log1p(radiance / m), m = first-hit albedo + kDemodEps at surface hits and 1
// on background pixels, so surface texture passes through the AOV instead of
// being rebuilt from noise; the output is remodulated by the same m.
constexpr float kDemodEps = 0.04f;
// Output cap in log1p space (radiance ~1e13): keeps expm1 finite while the
// first optimiser steps move the output far from the data.
constexpr float kMaxLog = 30.0f;
__device__ __forceinline__ float demod_of(const float* a, int c) {
    return a[7] > 0.5f ? fmaxf(a[c], 0.0f) + kDemodEps : 1.0f;
}

__global__ void k_pack(const float4* __restrict__ rad, const float* __restrict__ aov, __nv_bfloat16* __restrict__ x,
                       int64_t npix_img, int w, int h, int wp, int hp, int64_t img_offset) {
    const int64_t total = static_cast<int64_t>(wp) * hp;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int px = static_cast<int>(i % wp), py = static_cast<int>(i / wp);
        float f[16];
        for (int j = 0; j < 16; ++j) f[j] = 0.0f;
        if (px < w && py < h) {
            const int64_t s = static_cast<int64_t>(py) * w + px;
            const float4 r = rad[s];
            const float* a = aov + s * OHAO_PT_AOV_FLOATS;
            f[0] = log1pf(fmaxf(r.x, 0.0f) / demod_of(a, 0));
            f[1] = log1pf(fmaxf(r.y, 0.0f) / demod_of(a, 1));
            f[2] = log1pf(fmaxf(r.z, 0.0f) / demod_of(a, 2));
            f[3] = a[0]; f[4] = a[1]; f[5] = a[2];
            f[6] = a[3]; f[7] = a[4]; f[8] = a[5];
            f[9] = a[7] > 0.5f ? 1.0f / (1.0f + fmaxf(a[6], 0.0f)) : 0.0f;
            f[10] = a[8];
            f[11] = a[9];
        }
        float lo8[8], hi8[8];
        for (int j = 0; j < 8; ++j) { lo8[j] = f[j]; hi8[j] = f[8 + j]; }
        // image img_offset / (wp hp), two channel blocks
        const int64_t n = img_offset / total;
        *reinterpret_cast<uint4*>(x + blk(n, 0, 2, total, i)) = pack8(lo8);
        *reinterpret_cast<uint4*>(x + blk(n, 1, 2, total, i)) = pack8(hi8);
    }
    (void)npix_img;
}

// out: [pixels][8] FP32 log1p demodulated radiance -> RGBA32F linear
// radiance (crop from the padded grid)
__global__ void k_unpack(const float* __restrict__ y, const float* __restrict__ aov, float4* __restrict__ out, int w,
                         int h, int wp, int64_t img_offset) {
    const int64_t total = static_cast<int64_t>(w) * h;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int px = static_cast<int>(i % w), py = static_cast<int>(i / w);
        const float* s = y + (img_offset + static_cast<int64_t>(py) * wp + px) * 8;
        const float* a = aov + i * OHAO_PT_AOV_FLOATS;
        out[i] = make_float4(expm1f(fminf(fmaxf(s[0], 0.0f), kMaxLog)) * demod_of(a, 0),
                             expm1f(fminf(fmaxf(s[1], 0.0f), kMaxLog)) * demod_of(a, 1),
                             expm1f(fminf(fmaxf(s[2], 0.0f), kMaxLog)) * demod_of(a, 2), 1.0f);
    }
}

// The reference's display transform pow(ACES(x / 2), 1/2.2) with
// ACES(u) = clamp(u (2.51 u + 0.03) / (u (2.43 u + 0.59) + 0.14), 0, 1)
// (pt_raygen.rgen:99-102, 1263-1264) and its derivative in x (the slope at
// black is bounded by evaluating it at ACES >= 1e-3).
__device__ __forceinline__ float display_tf(float x, float& slope) {
    const float u = 0.5f * fmaxf(x, 0.0f);
    const float num = u * (2.51f * u + 0.03f), den = u * (2.43f * u + 0.59f) + 0.14f;
    const float a = num / den;
    if (a >= 1.0f) {
        slope = 0.0f;
        return 1.0f;
    }
    const float da = ((5.02f * u + 0.03f) * den - num * (4.86f * u + 0.59f)) / (den * den) * 0.5f;
    const float ac = fmaxf(a, 1e-3f);
    slope = (1.0f / 2.2f) * powf(ac, 1.0f / 2.2f) / ac * da;
    return powf(fmaxf(a, 0.0f), 1.0f / 2.2f);
}

// Loss per channel: |y - log1p(t / m)| + kDisplayWeight |D(m expm1(y')) - D(t)|
// (y = prediction in demodulated log1p space, y' = min(y, kMaxLog), m its
// albedo modulation, D = display transform); d out = its (sub)gradient / count.
constexpr float kDisplayWeight = 1.0f;
__global__ void k_l1(const float* __restrict__ y, const float4* __restrict__ tgt, const float* __restrict__ aov,
                     float* __restrict__ dy, int w, int h, int wp, int64_t img_offset, float inv_count,
                     double* __restrict__ loss) {
    double part = 0.0;
    const int64_t total = static_cast<int64_t>(w) * h;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int px = static_cast<int>(i % w), py = static_cast<int>(i / w);
        const int64_t q = img_offset + static_cast<int64_t>(py) * wp + px;
        const float4 t = tgt[i];
        const float tl[3] = {fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f), fmaxf(t.z, 0.0f)};
        const float* a = aov + i * OHAO_PT_AOV_FLOATS;
        for (int c = 0; c < 3; ++c) {
            const float m = demod_of(a, c);
            const float yv = y[q * 8 + c];
            const float d = yv - log1pf(tl[c] / m);
            float s_unused, slope;
            const float dt = display_tf(tl[c], s_unused);
            const bool live = yv > 0.0f && yv < kMaxLog;
            const float e = yv > 0.0f ? expm1f(fminf(yv, kMaxLog)) : 0.0f;
            const float dd = display_tf(e * m, slope) - dt;
            part += fabs(static_cast<double>(d)) + kDisplayWeight * fabs(static_cast<double>(dd));
            const float g_log = d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f);
            const float g_disp =
                live ? (dd > 0.0f ? 1.0f : (dd < 0.0f ? -1.0f : 0.0f)) * slope * m * (e + 1.0f) : 0.0f;
            dy[q * 8 + c] = (g_log + kDisplayWeight * g_disp) * inv_count;
        }
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xFFFFFFFFu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, part * inv_count);
}

// bias gradient: db[co] += sum over pixels of dZ
__global__ void k_bias_grad(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ y, int relu, Geo g,
                            int cout, int cout8, float* __restrict__ db) {
    const int co = blockIdx.y;
    float s = 0.0f;
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < g.npix;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float v = dy[p * cout8 + co];
        if (relu) {
            const int64_t hw = static_cast<int64_t>(g.h) * g.w;
            const int64_t n = p / hw;
            if (!(__bfloat162float(y[blk(n, co >> 3, cout8 >> 3, hw, p - n * hw) + (co & 7)]) > 0.0f)) v = 0.0f;
        }
        s += v;
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, off);
    if ((threadIdx.x & 31) == 0 && co < cout) atomicAdd(db + co, s);
}

// Adam (ohao/inverse/optimizer.hpp:26-39 update rule) on FP32 master weights;
// refreshes the BF16 copy W [cout_n][k_pad] and its transpose Wt [cin_n][k2_pad].
__global__ void k_adam_w(float* __restrict__ w32, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, __nv_bfloat16* __restrict__ w16, __nv_bfloat16* __restrict__ wt16,
                         LayerShape L, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t total = static_cast<int64_t>(L.cout) * 9 * L.cin8;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int co = static_cast<int>(i / (9 * L.cin8));
        const int f = static_cast<int>(i % (9 * L.cin8));
        const int tap = f / L.cin8, ci = f % L.cin8;
        const int64_t wi = static_cast<int64_t>(co) * L.k_pad + f;
        float wv = w32[wi];
        if (ci < L.cin) {
            const float gv = g[wi];
            const float mv = b1 * m[wi] + (1.0f - b1) * gv;
            const float vv = b2 * v[wi] + (1.0f - b2) * gv * gv;
            m[wi] = mv;
            v[wi] = vv;
            wv -= lr * (mv / c1) / (sqrtf(vv / c2) + eps);
            w32[wi] = wv;
        }
        const __nv_bfloat16 b = __float2bfloat16_rn(ci < L.cin ? wv : 0.0f);
        w16[wi] = b;
        wt16[static_cast<int64_t>(ci) * L.k2_pad + tap * L.cout8 + co] = b;
    }
}

__global__ void k_refresh(const float* __restrict__ w32, __nv_bfloat16* __restrict__ w16,
                          __nv_bfloat16* __restrict__ wt16, LayerShape L) {
    const int64_t total = static_cast<int64_t>(L.cout) * 9 * L.cin8;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int co = static_cast<int>(i / (9 * L.cin8));
        const int f = static_cast<int>(i % (9 * L.cin8));
        const int tap = f / L.cin8, ci = f % L.cin8;
        const int64_t wi = static_cast<int64_t>(co) * L.k_pad + f;
        const __nv_bfloat16 b = __float2bfloat16_rn(ci < L.cin ? w32[wi] : 0.0f);
        w16[wi] = b;
        wt16[static_cast<int64_t>(ci) * L.k2_pad + tap * L.cout8 + co] = b;
    }
}

__global__ void k_adam_b(float* __restrict__ b32, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gv = g[i];
    const float mv = b1 * m[i] + (1.0f - b1) * gv;
    const float vv = b2 * v[i] + (1.0f - b2) * gv * gv;
    m[i] = mv;
    v[i] = vv;
    b32[i] -= lr * (mv / c1) / (sqrtf(vv / c2) + eps);
}

// Exercises the bounded wait of the tensor-core pipeline: thread 0 waits
// with `limit` polls on an mbarrier whose phase never completes (no MMA and
// no arrival is ever issued, no tensor memory is held), records the timeout
// in err_flag exactly as k_conv does, and returns.
__global__ void k_wait_probe(uint32_t limit, int* err_flag) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar, 1);
        umma::mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !umma::mbar_wait(&bar, 0, limit)) atomicOr(err_flag, 2);
}

int grid_for(int64_t n, int block) {
    return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + block - 1) / block, 152 * 16)));
}

}  // namespace

size_t conv_smem_bytes(int bn) {
    return static_cast<size_t>(kStages) * (kBM * kBK * 2 + bn * kBK * 2) + 1024;
}

size_t conv_halo_smem_bytes(int cin8, int bn) {
    return ((halo_bytes(cin8) + 1023) & ~static_cast<size_t>(1023)) + static_cast<size_t>(kStages) * bn * kBK * 2 + 1024;
}

namespace {

// The warp-specialised forward (k_conv_ws) when the layer fits it:
// false leaves the layer to the other kernels. An upsample + concatenation
// layer first writes its upsampled source at full resolution into
// a.up_scratch.
bool try_conv_ws(const ConvArgs& a, int* err_flag, cudaStream_t st) {
    const bool single = a.c1 == 0 && !a.up0;
    const bool concat = a.up0 && a.c1 > 0 && a.up_scratch && a.c0 % 8 == 0 && a.c0s == a.c0 && a.g.w % 2 == 0 &&
                        a.g.h % 2 == 0;
    if (!(single || concat) || a.n_tiles != 1 || a.cin8 % 16 != 0 || a.cin8 > 256 || a.g.w < kHaloMinW) return false;
    const int cb_total = a.cin8 / 8;
    // the fewest launches over the output channels (each one all of the
    // tile's pixels and bn / nsplit channels), then the most rows per tile,
    // then the most stages (>= 2 where possible), whose buffers and weights
    // fit the shared memory and whose two accumulator sets fit the tensor
    // memory
    int nsplit = 0, bn = 0, rows = 0, nstages = 0, ncols = 32;
    size_t smem = 0;
    for (int sp : {1, 2, 4}) {
        const int b = a.bn / sp;
        if (a.bn % sp || b % 16) continue;
        int nc = 32;
        while (nc < b) nc <<= 1;
        for (int r : {4, 2, 1}) {
            if (2 * r * nc > 512) continue;
            for (int s2 = kWsMaxStages; s2 >= 1; --s2) {
                const size_t by = static_cast<size_t>(ws_smem_bytes(cb_total, s2, r, b, a.k_pad)) + 1024;   // + base alignment
                if (by + sizeof(WsSmem) <= 227 * 1024 && (s2 >= 2 || r == 1)) {
                    rows = r;
                    nstages = s2;
                    smem = by;
                    break;
                }
            }
            if (rows) break;
        }
        if (rows) {
            nsplit = sp;
            bn = b;
            ncols = nc;
            break;
        }
    }
    if (!nsplit) return false;
    const int cb_a = single ? cb_total : a.c0 / 8;
    const __nv_bfloat16* src_a = single ? a.x0 : a.up_scratch;
    const __nv_bfloat16* src_b = single ? a.x0 : a.x1;
    if ((reinterpret_cast<uintptr_t>(src_a) | reinterpret_cast<uintptr_t>(src_b)) & 15u) return false;
    if (cudaFuncSetAttribute(k_conv_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_conv_ws, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv_ws, kWsThreads, smem);
    if (sms <= 0 || per_sm <= 0) {
        cudaGetLastError();
        return false;
    }
    // stacked taps (one MMA per input row and horizontal tap covers the
    // three vertical taps, N = 3 bn): 16 or 32 output channels and an even
    // number of rows per tile, whose R + 4 slots fit a set of 256 columns
    const int stack = ((bn == 32 || bn == 16) && (rows == 4 || rows == 2)) ? 1 : 0;
    // resident CTAs whose accumulator sets fit the SM's 512 tensor-memory
    // columns together, so that no CTA's allocation waits for another to finish
    int stack_cols = 32;
    while (stack_cols < (rows + 4) * bn) stack_cols <<= 1;
    per_sm = std::min(per_sm, 512 / (2 * (stack ? stack_cols : rows * ncols)));
    if (concat)
        k_upsample2<<<grid_for(a.g.npix * (a.c0s / 8), 256), 256, 0, st>>>(a.x0, a.up_scratch, a.g, a.c0s);
    const int64_t tiles = static_cast<int64_t>(a.g.n) * ((a.g.h + rows - 1) / rows) * ((a.g.w + kBM - 1) / kBM);
    const int grid = static_cast<int>(std::min<int64_t>(tiles, static_cast<int64_t>(sms) * per_sm));
    const int cbs_a = a.c0s / 8, cbs_b = concat ? a.c1s / 8 : cbs_a;
    ConvArgs part = a;
    part.bn = bn;
    for (int k = 0; k < nsplit; ++k)
        k_conv_ws<<<grid, kWsThreads, smem, st>>>(part, src_a, src_b, cb_a, cbs_a, cbs_b, static_cast<int>(tiles),
                                                  nstages, rows, k * bn, stack, err_flag);
    return true;
}

}  // namespace

cudaError_t launch_conv(int mode, const ConvArgs& a, int wgrad_splits, int* err_flag, cudaStream_t st) {
    if (mode == kFwd && try_conv_ws(a, err_flag, st)) return cudaGetLastError();
    const size_t smem = conv_smem_bytes(a.bn);
    const size_t hsmem = conv_halo_smem_bytes(a.cin8, a.bn);
    // the neighbourhood kernel for wide rows of single-source inputs; the
    // upsample + skip-concatenation layers stay on the gather (measured: their
    // large neighbourhoods leave one or two CTAs per SM and the two sources
    // split the fill's warps)
    if (mode == kFwd && a.g.w >= kHaloMinW && a.c1 == 0 && a.cin8 % 16 == 0 && a.cin8 <= 256 && a.n_tiles == 1 &&
        hsmem <= 227 * 1024) {
        cudaFuncSetAttribute(k_conv_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(hsmem));
        const int64_t tiles = static_cast<int64_t>(a.g.n) * a.g.h * ((a.g.w + kBM - 1) / kBM);
        k_conv_halo<<<static_cast<unsigned>(tiles), kThreads, hsmem, st>>>(a, err_flag);
    } else if (mode == kFwd) {
        cudaFuncSetAttribute(k_conv<kFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        const dim3 grid(static_cast<unsigned>((a.g.npix + kBM - 1) / kBM), static_cast<unsigned>(a.n_tiles));
        k_conv<kFwd><<<grid, kThreads, smem, st>>>(a, err_flag);
    } else if (mode == kDgrad) {
        cudaFuncSetAttribute(k_conv<kDgrad>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        const dim3 grid(static_cast<unsigned>((a.g.npix + kBM - 1) / kBM), static_cast<unsigned>(a.n_tiles));
        k_conv<kDgrad><<<grid, kThreads, smem, st>>>(a, err_flag);
    } else {
        cudaFuncSetAttribute(k_conv<kWgrad>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        const dim3 grid(static_cast<unsigned>(a.n_tiles), static_cast<unsigned>(std::max(1, wgrad_splits)));
        k_conv<kWgrad><<<grid, kThreads, smem, st>>>(a, err_flag);
    }
    return cudaGetLastError();
}

cudaError_t launch_wait_probe(uint32_t limit, int* err_flag, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(limit, err_flag);
    return cudaGetLastError();
}
void launch_pool_fwd(const __nv_bfloat16* x, __nv_bfloat16* y, const Geo& lo, int c8, cudaStream_t st) {
    k_pool_fwd<<<grid_for(lo.npix * (c8 / 8), 256), 256, 0, st>>>(x, y, lo, c8);
}
void launch_pool_bwd(const __nv_bfloat16* x, const float* dy, float* dx, const Geo& lo, int c8, cudaStream_t st) {
    k_pool_bwd<<<grid_for(lo.npix * c8, 256), 256, 0, st>>>(x, dy, dx, lo, c8);
}
void launch_pack(const float* rad, const float* aov, __nv_bfloat16* x, int w, int h, int wp, int hp, int64_t img_off,
                 cudaStream_t st) {
    k_pack<<<grid_for(static_cast<int64_t>(wp) * hp, 256), 256, 0, st>>>(
        reinterpret_cast<const float4*>(rad), aov, x, static_cast<int64_t>(w) * h, w, h, wp, hp, img_off);
}
void launch_unpack(const float* y, const float* aov, float* out, int w, int h, int wp, int64_t img_off,
                   cudaStream_t st) {
    k_unpack<<<grid_for(static_cast<int64_t>(w) * h, 256), 256, 0, st>>>(y, aov, reinterpret_cast<float4*>(out), w,
                                                                           h, wp, img_off);
}
void launch_l1(const float* y, const float* tgt, const float* aov, float* dy, int w, int h, int wp, int64_t img_off,
               float inv_count, double* loss, cudaStream_t st) {
    k_l1<<<grid_for(static_cast<int64_t>(w) * h, 256), 256, 0, st>>>(y, reinterpret_cast<const float4*>(tgt), aov, dy,
                                                                        w, h, wp, img_off, inv_count, loss);
}
void launch_bias_grad(const float* dy, const __nv_bfloat16* y, bool relu, const Geo& g, int cout, int cout8, float* db,
                      cudaStream_t st) {
    const dim3 grid(static_cast<unsigned>(std::min<int64_t>(64, (g.npix + 255) / 256)), static_cast<unsigned>(cout));
    k_bias_grad<<<grid, 256, 0, st>>>(dy, y, relu ? 1 : 0, g, cout, cout8, db);
}
void launch_refresh(const LayerShape& L, const float* w32, __nv_bfloat16* w16, __nv_bfloat16* wt16, cudaStream_t st) {
    k_refresh<<<grid_for(static_cast<int64_t>(L.cout) * 9 * L.cin8, 256), 256, 0, st>>>(w32, w16, wt16, L);
}
void launch_adam(const LayerShape& L, float* w32, const float* gw, float* mw, float* vw, __nv_bfloat16* w16,
                 __nv_bfloat16* wt16, float* b32, const float* gb, float* mb, float* vb, float lr, int t,
                 cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, static_cast<float>(t)), c2 = 1.0f - powf(b2, static_cast<float>(t));
    k_adam_w<<<grid_for(static_cast<int64_t>(L.cout) * 9 * L.cin8, 256), 256, 0, st>>>(w32, gw, mw, vw, w16, wt16, L,
                                                                                     lr, b1, b2, eps, c1, c2);
    k_adam_b<<<(L.cout + 127) / 128, 128, 0, st>>>(b32, gb, mb, vb, L.cout, lr, b1, b2, eps, c1, c2);
}

}  // namespace dn
}  // namespace ohao
