// bvh_build.cu -- device LBVH builder producing the 8-wide quantized BVH.
//
// Replaces the driver build behind RTAccelerationStructure::createBLAS /
// buildTLAS (rt_acceleration_structure.cpp:205-300, 419-530). Integer work is
// exact and the float work (centroids, box unions, half areas) uses fixed
// operation order, so the output is bit-identical to a host build of the
// same algorithm:
//   1. centroid bounds (two-pass min/max reduction);
//   2. 30-bit Morton codes;
//   3. stable LSD radix sort of (code, index), 8 passes of 4 bits; each pass
//      is tile histogram -> one-block digit-major scan -> stable scatter;
//   4. Karras binary radix tree (one thread per internal node);
//   5. bottom-up pass with per-node arrival counters: box union, half area,
//      greedy 8-wide collapse, wide-subtree node count and height;
//   6. top-down layout, one launch per wide level, with child-block and leaf
//      offsets derived from subtree counts (independent of thread order);
//   7. 8-bit outward-rounded child boxes on a power-of-two grid per axis.
#include "bvh_internal.hpp"

#include <cstdio>
#include <mutex>
#include <vector>

namespace ohao {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

struct Box6 {
    float lo[3], hi[3];
};

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_cbounds_partial(const Box6* __restrict__ prims, uint32_t n, float* __restrict__ partial) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Box6 b = prims[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c = (b.lo[k] + b.hi[k]) * 0.5f;
            mn[k] = fminf(mn[k], c);
            mx[k] = fmaxf(mx[k], c);
        }
    }
    __shared__ float s[6][256];
#pragma unroll
    for (int k = 0; k < 3; ++k) { s[k][threadIdx.x] = mn[k]; s[3 + k][threadIdx.x] = mx[k]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fminf(s[k][threadIdx.x], s[k][threadIdx.x + w]);
                s[3 + k][threadIdx.x] = fmaxf(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + w]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) partial[blockIdx.x * 6 + k] = s[k][0];
}

__global__ void k_cbounds_final(const float* __restrict__ partial, int nb, float* __restrict__ out) {
    __shared__ float s[6][256];
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        for (int k = 0; k < 3; ++k) {
            v[k] = fminf(v[k], partial[i * 6 + k]);
            v[3 + k] = fmaxf(v[3 + k], partial[i * 6 + 3 + k]);
        }
    for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fminf(s[k][threadIdx.x], s[k][threadIdx.x + w]);
                s[3 + k][threadIdx.x] = fmaxf(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) out[k] = s[k][0];
}

__global__ void k_morton(const Box6* __restrict__ prims, uint32_t n, const float* __restrict__ cb,
                         uint32_t* __restrict__ codes, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Box6 b = prims[i];
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ext = cb[3 + k] - cb[k];
        const float scale = ext > 0.0f ? 1024.0f / ext : 0.0f;
        const float c = (b.lo[k] + b.hi[k]) * 0.5f;
        float f = (c - cb[k]) * scale;
        f = fminf(fmaxf(f, 0.0f), 1023.0f);
        q[k] = static_cast<uint32_t>(f);
    }
    codes[i] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    vals[i] = i;
}

// ---- stable LSD radix sort, 4-bit digits ----
__global__ void __launch_bounds__(kSortThreads) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                          uint32_t num_tiles, uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[16];
    if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile + threadIdx.x * kSortItems;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + j;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 15u], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 16) hist[threadIdx.x * num_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of m entries by one block of 1024 threads
__global__ void __launch_bounds__(1024) k_scan_excl(uint32_t* __restrict__ data, uint32_t m) {
    __shared__ uint32_t s[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < m) sum += data[b0 + i];
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = (threadIdx.x >= static_cast<uint32_t>(off)) ? s[threadIdx.x - off] : 0u;
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

__global__ void __launch_bounds__(kSortThreads) k_rs_scatter(const uint32_t* __restrict__ keys_in,
                                                             const uint32_t* __restrict__ vals_in, uint32_t n, int shift,
                                                             uint32_t num_tiles, const uint32_t* __restrict__ offs,
                                                             uint32_t* __restrict__ keys_out,
                                                             uint32_t* __restrict__ vals_out) {
    const uint32_t base = blockIdx.x * kSortTile + threadIdx.x * kSortItems;
    uint32_t k[kSortItems], v[kSortItems], dg[kSortItems], rank[kSortItems];
    uint64_t packed = 0;   // 16 x 4-bit per-thread digit counts
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
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
    // expand to 8 words of two 16-bit fields and block-exclusive-scan them
    uint32_t w[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        w[q] = static_cast<uint32_t>((packed >> (8 * q)) & 0xFu) | (static_cast<uint32_t>((packed >> (8 * q + 4)) & 0xFu) << 16);
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
    __shared__ uint32_t wsum[kSortThreads / 32][8];
    if (lane == 31)
#pragma unroll
        for (int q = 0; q < 8; ++q) wsum[warp][q] = inc[q];
    __syncthreads();
    uint32_t wpre[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        uint32_t acc = 0;
        for (int ww = 0; ww < warp; ++ww) acc += wsum[ww][q];
        wpre[q] = acc + inc[q] - w[q];
    }
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
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

// ---- Karras tree ----
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ codes, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
}

__global__ void k_karras(const uint32_t* __restrict__ codes, uint32_t n32, uint32_t* __restrict__ left,
                         uint32_t* __restrict__ right, uint32_t* __restrict__ first, uint32_t* __restrict__ last,
                         uint32_t* __restrict__ parent) {
    const int64_t n = n32;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (kdelta(codes, n, i, i + 1) - kdelta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(codes, n, i, i - d);
    int64_t lmax = 2;
    while (kdelta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t s = lmax / 2; s >= 1; s /= 2)
        if (kdelta(codes, n, i, i + (l + s) * d) > dmin) l += s;
    const int64_t j = i + l * d;
    const int dnode = kdelta(codes, n, i, j);
    int64_t s = 0, div = 2;
    while (true) {
        const int64_t step = (l + div - 1) / div;
        if (kdelta(codes, n, i, i + (s + step) * d) > dnode) s += step;
        if (step <= 1) break;
        div *= 2;
    }
    const int64_t gamma = i + s * d + min(d, 0);
    const int64_t lo = min(i, j), hi = max(i, j);
    const uint32_t lc = (lo == gamma) ? static_cast<uint32_t>(n - 1 + gamma) : static_cast<uint32_t>(gamma);
    const uint32_t rc = (hi == gamma + 1) ? static_cast<uint32_t>(n - 1 + gamma + 1) : static_cast<uint32_t>(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = static_cast<uint32_t>(lo);
    last[i] = static_cast<uint32_t>(hi);
    parent[lc] = static_cast<uint32_t>(i);
    parent[rc] = static_cast<uint32_t>(i);
}

struct TreeView {
    uint32_t n;
    const uint32_t* left;
    const uint32_t* right;
    const uint32_t* first;
    const uint32_t* last;
    Box6* box;      // 2n-1
    float* sa;      // 2n-1
};

__device__ __forceinline__ float half_area(const Box6& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}
__device__ __forceinline__ bool is_internal(uint32_t id, uint32_t n) { return id < n - 1; }
__device__ __forceinline__ uint32_t prims_of(const TreeView& t, uint32_t id) {
    if (id >= t.n - 1) return 1u;
    return __ldcg(t.last + id) - __ldcg(t.first + id) + 1u;
}
__device__ __forceinline__ uint32_t first_of(const TreeView& t, uint32_t id) {
    if (id >= t.n - 1) return id - (t.n - 1);
    return __ldcg(t.first + id);
}
__device__ __forceinline__ bool is_internal_wide(const TreeView& t, uint32_t id) {
    return is_internal(id, t.n) && prims_of(t, id) > 3u;
}

// greedy collapse (largest half-area internal member opened first; smallest
// id on ties)
__device__ int collapse(const TreeView& t, uint32_t x, uint32_t member[8]) {
    if (!is_internal(x, t.n)) { member[0] = x; return 1; }
    int cnt = 2;
    member[0] = __ldcg(t.left + x);
    member[1] = __ldcg(t.right + x);
    while (cnt < 8) {
        int best = -1;
        float bsa = 0.0f;
        uint32_t bid = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t m = member[k];
            if (!is_internal(m, t.n)) continue;
            const float sm = __ldcg(t.sa + m);
            if (best < 0 || sm > bsa || (sm == bsa && m < bid)) { best = k; bsa = sm; bid = m; }
        }
        if (best < 0) break;
        const uint32_t m = member[best];
        member[best] = __ldcg(t.left + m);
        member[cnt++] = __ldcg(t.right + m);
    }
    return cnt;
}

__device__ __forceinline__ Box6 ldcg_box(const Box6* p) {
    Box6 b;
    const float* f = reinterpret_cast<const float*>(p);
#pragma unroll
    for (int k = 0; k < 3; ++k) { b.lo[k] = __ldcg(f + k); b.hi[k] = __ldcg(f + 3 + k); }
    return b;
}

__global__ void k_bottom_up(TreeView t, const Box6* __restrict__ prims, const uint32_t* __restrict__ order,
                            const uint32_t* __restrict__ parent, uint32_t* __restrict__ arrive,
                            uint32_t* __restrict__ wcount, uint32_t* __restrict__ wheight) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = t.n;
    if (i >= n) return;
    const uint32_t leaf = n - 1 + i;
    const Box6 b = prims[order[i]];
    t.box[leaf] = b;
    t.sa[leaf] = half_area(b);
    if (n < 2) return;
    uint32_t x = parent[leaf];
    while (true) {
        __threadfence();
        if (atomicAdd(arrive + x, 1u) == 0u) return;
        __threadfence();
        const Box6 lb = ldcg_box(t.box + __ldcg(t.left + x));
        const Box6 rb = ldcg_box(t.box + __ldcg(t.right + x));
        Box6 u;
#pragma unroll
        for (int k = 0; k < 3; ++k) { u.lo[k] = fminf(lb.lo[k], rb.lo[k]); u.hi[k] = fmaxf(lb.hi[k], rb.hi[k]); }
        t.box[x] = u;
        __stcg(t.sa + x, half_area(u));
        __threadfence();
        uint32_t member[8];
        const int cnt = collapse(t, x, member);
        uint32_t wc = 1, h = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t m = member[k];
            if (is_internal_wide(t, m)) {
                wc += __ldcg(wcount + m);
                h = max(h, __ldcg(wheight + m));
            }
        }
        __stcg(wcount + x, wc);
        __stcg(wheight + x, h + 1);
        if (x == 0) return;
        x = parent[x];
    }
}

struct Item {
    uint32_t bin, widx, below, tbase;
};

__device__ int axis_exponent(float lo, float hi) {
    const double d = static_cast<double>(hi) - static_cast<double>(lo);
    if (!(d > 0.0)) return -100;
    int ex;
    const double m = frexp(d / 255.0, &ex);
    const int e = (m == 0.5) ? ex - 1 : ex;
    return max(e, -100);
}

__global__ void k_layout_level(TreeView t, const uint32_t* __restrict__ order, const uint32_t* __restrict__ wcount,
                               const Item* __restrict__ cur, const uint32_t* __restrict__ cur_count,
                               Item* __restrict__ next, uint32_t* __restrict__ next_count, uint4* __restrict__ nodes,
                               uint32_t* __restrict__ prim_order) {
    const uint32_t count = *cur_count;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
        const Item it = cur[idx];
        uint32_t member[8];
        const int cnt = collapse(t, it.bin, member);
        const Box6 nb = t.box[it.bin];
        uint8_t bytes[80];
#pragma unroll
        for (int q = 0; q < 80; ++q) bytes[q] = 0;
        int e[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            e[a] = axis_exponent(nb.lo[a], nb.hi[a]);
            while (true) {
                bool ok = true;
                for (int k = 0; k < cnt && ok; ++k) {
                    const Box6 cb = t.box[member[k]];
                    const double qh = ceil(ldexp(static_cast<double>(cb.hi[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                    if (qh > 255.0) ok = false;
                }
                if (ok) break;
                e[a] += 1;
            }
            bytes[12 + a] = static_cast<uint8_t>(static_cast<int8_t>(e[a]));
            for (int k = 0; k < cnt; ++k) {
                const Box6 cb = t.box[member[k]];
                const double ql = floor(ldexp(static_cast<double>(cb.lo[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                const double qh = ceil(ldexp(static_cast<double>(cb.hi[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                bytes[32 + a * 8 + k] = static_cast<uint8_t>(fmax(0.0, ql));
                bytes[56 + a * 8 + k] = static_cast<uint8_t>(fmin(255.0, qh));
            }
            for (int k = cnt; k < 8; ++k) {   // unused slot: the inverted box 255..0, which no ray enters
                bytes[32 + a * 8 + k] = 0xFFu;
                bytes[56 + a * 8 + k] = 0u;
            }
        }
        uint32_t nint = 0, nleaf = 0;
        for (int k = 0; k < cnt; ++k) {
            if (is_internal_wide(t, member[k])) nint++;
            else nleaf += prims_of(t, member[k]);
        }
        uint32_t imask = 0, rank = 0, loff = 0;
        uint32_t sub_below = it.below + nint, sub_tri = it.tbase + nleaf;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t m = member[k];
            if (is_internal_wide(t, m)) {
                imask |= 1u << k;
                bytes[24 + k] = static_cast<uint8_t>(0x80u | rank);
                const uint32_t slot = atomicAdd(next_count, 1u);
                next[slot] = Item{m, it.below + rank, sub_below, sub_tri};
                sub_below += wcount[m] - 1;
                sub_tri += prims_of(t, m);
                rank++;
            } else {
                const uint32_t c = prims_of(t, m), f = first_of(t, m);
                bytes[24 + k] = static_cast<uint8_t>((c << 5) | loff);
                for (uint32_t q = 0; q < c; ++q) prim_order[it.tbase + loff + q] = order[f + q];
                loff += c;
            }
        }
        bytes[15] = static_cast<uint8_t>(imask);
        uint32_t words[20];
#pragma unroll
        for (int q = 0; q < 20; ++q)
            words[q] = static_cast<uint32_t>(bytes[4 * q]) | (static_cast<uint32_t>(bytes[4 * q + 1]) << 8) |
                       (static_cast<uint32_t>(bytes[4 * q + 2]) << 16) | (static_cast<uint32_t>(bytes[4 * q + 3]) << 24);
        words[0] = __float_as_uint(nb.lo[0]);
        words[1] = __float_as_uint(nb.lo[1]);
        words[2] = __float_as_uint(nb.lo[2]);
        words[4] = it.below;
        words[5] = it.tbase;
        uint4* dst = nodes + static_cast<size_t>(it.widx) * 5;
#pragma unroll
        for (int q = 0; q < 5; ++q) dst[q] = make_uint4(words[4 * q], words[4 * q + 1], words[4 * q + 2], words[4 * q + 3]);
    }
}

__global__ void k_clear_u32(uint32_t* p, size_t n) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
        p[i] = 0u;
}

inline unsigned grid_for(size_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

#define BVH_CHECK(x)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            err = std::string("CUDA error in BVH build: ") + cudaGetErrorString(e_) + " at " #x; \
            return OHAO_ERR_CUDA;                                                             \
        }                                                                                     \
    } while (0)

namespace {
// Scratch layout of one build; with base == nullptr it only measures.
struct BuildLayout {
    float* partial;
    float* cb;
    uint32_t *keysA, *valsA, *keysB, *valsB, *hist;
    uint32_t *left, *right, *first, *last, *parent, *arrive;
    Box6* boxes;
    float* sa;
    uint32_t *wcount, *wheight;
    Item *frontA, *frontB;
    uint32_t* counts;
    size_t bytes;

    BuildLayout(char* base, uint32_t n) {
        size_t off = 0;
        auto take = [&](size_t count, size_t elem) {
            char* r = base ? base + off : nullptr;
            off += (count * elem + 255) & ~size_t(255);
            return r;
        };
        const size_t nn = n ? n : 1;
        const size_t tiles = (nn + kSortTile - 1) / kSortTile;
        partial = reinterpret_cast<float*>(take(1024 * 6, 4));
        cb = reinterpret_cast<float*>(take(8, 4));
        keysA = reinterpret_cast<uint32_t*>(take(nn, 4));
        valsA = reinterpret_cast<uint32_t*>(take(nn, 4));
        keysB = reinterpret_cast<uint32_t*>(take(nn, 4));
        valsB = reinterpret_cast<uint32_t*>(take(nn, 4));
        hist = reinterpret_cast<uint32_t*>(take(16 * tiles, 4));
        left = reinterpret_cast<uint32_t*>(take(nn, 4));
        right = reinterpret_cast<uint32_t*>(take(nn, 4));
        first = reinterpret_cast<uint32_t*>(take(nn, 4));
        last = reinterpret_cast<uint32_t*>(take(nn, 4));
        parent = reinterpret_cast<uint32_t*>(take(2 * nn, 4));
        arrive = reinterpret_cast<uint32_t*>(take(nn, 4));
        boxes = reinterpret_cast<Box6*>(take(2 * nn, sizeof(Box6)));
        sa = reinterpret_cast<float*>(take(2 * nn, 4));
        wcount = reinterpret_cast<uint32_t*>(take(nn, 4));
        wheight = reinterpret_cast<uint32_t*>(take(nn, 4));
        frontA = reinterpret_cast<Item*>(take(nn, sizeof(Item)));
        frontB = reinterpret_cast<Item*>(take(nn, sizeof(Item)));
        counts = reinterpret_cast<uint32_t*>(take(64, 4));
        bytes = off;
    }
};
}  // namespace

size_t bvh_build_scratch_bytes(uint32_t n) { return BuildLayout(nullptr, n).bytes; }

ohao_status bvh_build(const float* d_boxes, uint32_t n, void* d_scratch, size_t scratch_bytes, uint4* d_nodes,
                      uint32_t* d_prim_order, float* d_root_box, BvhBuildInfo* info, cudaStream_t st, std::string& err) {
    info->nnodes = 0;
    info->height = 0;
    if (n == 0) return OHAO_OK;
    if (scratch_bytes < bvh_build_scratch_bytes(n)) {
        err = "BVH build scratch too small";
        return OHAO_ERR_INVALID_ARG;
    }
    const Box6* prims = reinterpret_cast<const Box6*>(d_boxes);
    const size_t tiles = (static_cast<size_t>(n) + kSortTile - 1) / kSortTile;
    const BuildLayout L(static_cast<char*>(d_scratch), n);
    float* partial = L.partial;
    float* cb = L.cb;
    uint32_t *keysA = L.keysA, *valsA = L.valsA, *keysB = L.keysB, *valsB = L.valsB, *hist = L.hist;
    uint32_t *left = L.left, *right = L.right, *first = L.first, *last = L.last, *parent = L.parent;
    uint32_t* arrive = L.arrive;
    Box6* boxes = L.boxes;
    float* sa = L.sa;
    uint32_t *wcount = L.wcount, *wheight = L.wheight;
    Item *frontA = L.frontA, *frontB = L.frontB;
    uint32_t* counts = L.counts;

    const int nb_part = static_cast<int>(std::min<size_t>(1024, grid_for(n, 256)));
    k_cbounds_partial<<<nb_part, 256, 0, st>>>(prims, n, partial);
    k_cbounds_final<<<1, 256, 0, st>>>(partial, nb_part, cb);
    k_morton<<<grid_for(n, 256), 256, 0, st>>>(prims, n, cb, keysA, valsA);
    BVH_CHECK(cudaGetLastError());
    uint32_t *kin = keysA, *vin = valsA, *kout = keysB, *vout = valsB;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = pass * 4;
        k_rs_hist<<<static_cast<unsigned>(tiles), kSortThreads, 0, st>>>(kin, n, shift, static_cast<uint32_t>(tiles), hist);
        k_scan_excl<<<1, 1024, 0, st>>>(hist, static_cast<uint32_t>(16 * tiles));
        k_rs_scatter<<<static_cast<unsigned>(tiles), kSortThreads, 0, st>>>(kin, vin, n, shift,
                                                                            static_cast<uint32_t>(tiles), hist, kout, vout);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    BVH_CHECK(cudaGetLastError());
    // kin = sorted codes, vin = order
    TreeView tv{n, left, right, first, last, boxes, sa};
    if (n >= 2) {
        k_karras<<<grid_for(n - 1, 256), 256, 0, st>>>(kin, n, left, right, first, last, parent);
        k_clear_u32<<<256, 256, 0, st>>>(arrive, n);
    }
    k_bottom_up<<<grid_for(n, 256), 256, 0, st>>>(tv, prims, vin, parent, arrive, wcount, wheight);
    BVH_CHECK(cudaGetLastError());
    uint32_t hinfo[2] = {1u, 1u};
    if (n >= 2) {
        BVH_CHECK(cudaMemcpyAsync(&hinfo[0], wcount, 4, cudaMemcpyDeviceToHost, st));
        BVH_CHECK(cudaMemcpyAsync(&hinfo[1], wheight, 4, cudaMemcpyDeviceToHost, st));
    }
    BVH_CHECK(cudaMemcpyAsync(d_root_box, n >= 2 ? reinterpret_cast<const float*>(boxes)
                                                  : reinterpret_cast<const float*>(boxes + (n - 1)),
                              24, cudaMemcpyDeviceToDevice, st));
    BVH_CHECK(cudaStreamSynchronize(st));
    const uint32_t total = hinfo[0], height = hinfo[1];
    info->nnodes = total;
    info->height = height;
    // top-down layout
    const Item root{n >= 2 ? 0u : (n - 1), 0u, 1u, 0u};
    BVH_CHECK(cudaMemcpyAsync(frontA, &root, sizeof(Item), cudaMemcpyHostToDevice, st));
    BVH_CHECK(cudaMemsetAsync(counts, 0, 64 * sizeof(uint32_t), st));
    const uint32_t one = 1u;
    BVH_CHECK(cudaMemcpyAsync(counts, &one, 4, cudaMemcpyHostToDevice, st));
    Item *cur = frontA, *nxt = frontB;
    for (uint32_t lvl = 0; lvl < height; ++lvl) {
        uint32_t* cc = counts + (lvl % 32);
        uint32_t* nc = counts + ((lvl + 1) % 32);
        BVH_CHECK(cudaMemsetAsync(nc, 0, 4, st));
        k_layout_level<<<152 * 4, 128, 0, st>>>(tv, vin, wcount, cur, cc, nxt, nc, d_nodes, d_prim_order);
        std::swap(cur, nxt);
    }
    BVH_CHECK(cudaGetLastError());
    BVH_CHECK(cudaStreamSynchronize(st));
    return OHAO_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free build (ohao_bvh_build_noalloc)
//
// For callers that must not allocate device memory themselves: a host that
// hands the renderer a fixed memory budget and keeps the rest of the GPU for
// its own pool, or a per-frame rebuild of a small animated mesh where
// cudaMalloc/cudaFree (which synchronise the device) would stall the other
// streams. The build's scratch is one file-scope device array sized for
// OHAO_BVH_NOALLOC_MAX_PRIMS primitives; every GPU that loads this library
// holds it (about 9.2 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace {
constexpr uint32_t kNoAllocMaxPrims = OHAO_BVH_NOALLOC_MAX_PRIMS;
// 140 bytes per primitive covers the sort, tree, box and frontier arrays;
// 64 KB covers the fixed-size parts and the 256-byte alignment of each array.
constexpr size_t kNoAllocScratchBytes = 140ull * kNoAllocMaxPrims + 64ull * 1024ull;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

}  // namespace ohao

extern "C" ohao_status ohao_bvh_build_noalloc(const float* d_boxes, uint32_t n, void* d_nodes, uint32_t* d_prim_order,
                                              float* d_root_box, uint32_t* out_nnodes, uint32_t* out_height,
                                              ohao_stream stream) {
    using namespace ohao;
    if (!out_nnodes || !out_height || (n && (!d_boxes || !d_nodes || !d_prim_order || !d_root_box)))
        return OHAO_ERR_INVALID_ARG;
    if (n > kNoAllocMaxPrims) {
        std::fprintf(stderr, "[ohao] ohao_bvh_build_noalloc: %u primitives exceed the fixed capacity of %u\n", n,
                     kNoAllocMaxPrims);
        return OHAO_ERR_TOO_LARGE;
    }
    if (bvh_build_scratch_bytes(n) > kNoAllocScratchBytes) return OHAO_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return OHAO_ERR_CUDA;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return OHAO_ERR_UNSUPPORTED;
    void* scratch = nullptr;
    {
        // First call on a device: resolve the device address of the array
        // (the host-side symbol is only a stand-in), with that device current.
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return OHAO_ERR_CUDA;
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    BvhBuildInfo info{};
    std::string err;
    const ohao_status s = bvh_build(d_boxes, n, scratch, kNoAllocScratchBytes, static_cast<uint4*>(d_nodes),
                                    d_prim_order, d_root_box, &info, reinterpret_cast<cudaStream_t>(stream), err);
    if (s != OHAO_OK) {
        std::fprintf(stderr, "[ohao] ohao_bvh_build_noalloc: %s\n", err.c_str());
        return s;
    }
    *out_nnodes = info.nnodes;
    *out_height = info.height;
    return OHAO_OK;
}
