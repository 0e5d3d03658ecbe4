// radix_sort.cuh -- stable LSD radix sort of (uint32 key, uint32 value)
// pairs with 4-bit digits, for element counts held in device memory.
//
// One pass = tile histogram -> one-block digit-major exclusive scan ->
// stable scatter. A tile is 256 threads x 8 consecutive items; each thread
// ranks its items with 16 packed 4-bit counters, and a block scan of the
// counters (two digits per 32-bit word) gives each item's rank inside the
// tile. Launch shapes depend only on the capacity, so a sequence of passes
// can be captured in a CUDA graph and replayed for any count <= capacity.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ohao {
namespace rsort {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

inline uint32_t tiles_for(uint32_t cap) { return (cap + kTile - 1) / kTile; }

__global__ void __launch_bounds__(kThreads) k_hist(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ count,
                                                   int shift, uint32_t num_tiles, uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[16];
    const uint32_t n = *count;
    if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const uint32_t idx = base + j;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 15u], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 16) hist[threadIdx.x * num_tiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ data, uint32_t m) {
    __shared__ uint32_t s[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < m) sum += data[b0 + i];
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t v = (threadIdx.x >= static_cast<uint32_t>(off)) ? s[threadIdx.x - off] : 0u;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = s[threadIdx.x] - sum;
    for (uint32_t i = 0; i < per; ++i) {
        if (b0 + i < m) {
            const uint32_t v = data[b0 + i];
            data[b0 + i] = run;
            run += v;
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(const uint32_t* __restrict__ keys_in,
                                                      const uint32_t* __restrict__ vals_in,
                                                      const uint32_t* __restrict__ count, int shift, uint32_t num_tiles,
                                                      const uint32_t* __restrict__ offs, uint32_t* __restrict__ keys_out,
                                                      uint32_t* __restrict__ vals_out) {
    const uint32_t n = *count;
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t k[kItems], v[kItems], dg[kItems], rank[kItems];
    uint64_t packed = 0;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const uint32_t idx = base + j;
        if (idx < n) {
            k[j] = keys_in[idx];
            v[j] = vals_in[idx];
            dg[j] = (k[j] >> shift) & 15u;
            rank[j] = static_cast<uint32_t>((packed >> (4 * dg[j])) & 0xFu);
            packed += 1ull << (4 * dg[j]);
        } else {
            dg[j] = 16u;
            k[j] = v[j] = rank[j] = 0u;
        }
    }
    uint32_t w[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        w[q] = static_cast<uint32_t>((packed >> (8 * q)) & 0xFu) |
               (static_cast<uint32_t>((packed >> (8 * q + 4)) & 0xFu) << 16);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        uint32_t x = w[q];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if (lane >= off) x += y;
        }
        inc[q] = x;
    }
    __shared__ uint32_t wsum[kThreads / 32][8];
    if (lane == 31) {
#pragma unroll
        for (int q = 0; q < 8; ++q) wsum[warp][q] = inc[q];
    }
    __syncthreads();
    uint32_t wpre[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        uint32_t acc = 0;
        for (int ww = 0; ww < warp; ++ww) acc += wsum[ww][q];
        wpre[q] = acc + inc[q] - w[q];
    }
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        if (dg[j] >= 16u) continue;
        const uint32_t d = dg[j];
        uint32_t word = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (static_cast<uint32_t>(q) == (d >> 1)) word = wpre[q];
        const uint32_t pre = (d & 1u) ? (word >> 16) : (word & 0xFFFFu);
        const uint32_t pos = offs[d * num_tiles + blockIdx.x] + pre + rank[j];
        keys_out[pos] = k[j];
        vals_out[pos] = v[j];
    }
}

// Sorts keys/vals (count in device memory, <= capacity) on the low `bits`
// bits (a multiple of 4). Even pass counts leave the result in keysA/valsA.
inline void sort_pairs(uint32_t* keysA, uint32_t* valsA, uint32_t* keysB, uint32_t* valsB, uint32_t* hist,
                       const uint32_t* count, uint32_t capacity, int bits, cudaStream_t st) {
    const uint32_t tiles = tiles_for(capacity);
    uint32_t *ki = keysA, *vi = valsA, *ko = keysB, *vo = valsB;
    for (int shift = 0; shift < bits; shift += 4) {
        k_hist<<<tiles, kThreads, 0, st>>>(ki, count, shift, tiles, hist);
        k_scan<<<1, 1024, 0, st>>>(hist, 16 * tiles);
        k_scatter<<<tiles, kThreads, 0, st>>>(ki, vi, count, shift, tiles, hist, ko, vo);
        uint32_t* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
}

}  // namespace rsort
}  // namespace ohao
