// wavefront.cu -- wavefront path integrator and the batch trace call.
//
// One wave holds up to `capacity` paths, numbered sample-major
// (slot = k*npix + rank - wave_begin, rank = the pixel's place in 8x4-tile
// order, see rank_pixel), in structure-of-arrays state. Each of
// the 1 + 2*max_bounces iterations runs:
//   extend  closest-hit traversal for the ray queue;
//   shade   closest-hit/miss shading and the estimator step; emits the next
//           ray and up to two shadow queries per path; queues are compacted
//           with one atomic per warp (ballot + popc prefix);
//   shadow  any-hit traversal; visible queries add their contribution.
// finalize applies the firefly clamp and folds the wave's samples into the
// progressive (mean, count) accumulator in sample order per pixel, the
// reference's own-pixel running mean (pt_raygen.rgen:1144-1186).
// Every kernel is a grid-stride loop over a device-side count, so the launch
// sequence is fixed and does not read counts back to the host.
#include "pt_path.cuh"
#include "pt_fetch.cuh"
#include "radix_sort.cuh"

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

namespace ohao {

namespace {

// Path state by slot p, in 32-byte pairs of 16-byte records, so that a
// path read out of queue order (after binning) touches one DRAM sector per
// pair instead of one per field:
//   ray[2p] = origin, ray[2p+1] = (direction, last pdf)
//   tr[2p]  = throughput, tr[2p+1] = radiance
//   hm[2p]  = (rng, dim, flags, hit instance), hm[2p+1] = hit (t, u, v, prim bits)
// flags = phase | bounce<<2 | delta<<10 | shL<<11 | shE<<12.
struct Soa {
    float4* ray;
    float4* tr;
    uint4* hm;
    float4* fhP;
    float4* fhN;
    float4* fhA;
    float4* sh_org;
    float4* shL;         // dir, tmax
    float4* shLc;        // contribution
    float4* shE;
    float4* shEc;
    uint32_t* q_ray[2];
    uint32_t* q_sh;
    uint32_t* counts;    // [0],[1] ray queue counts, [2] shadow count, [3] done count, [4] work claimed
    // persistent pool only: slot -> (global pixel, sample), running mean, finished-path queue
    uint32_t* pix;
    uint32_t* smp;
    float4* acc;
    uint32_t* q_done;
    // persistent pool only: ray-queue reordering (keys/values ping-pong, histogram)
    uint32_t *skA, *svA, *skB, *svB, *shist;
};

// Persistent multi-view pool: per-call view table in device memory.
constexpr uint32_t kMaxViews = 1024;
constexpr uint32_t kIdle = 0xFFFFFFFFu;
constexpr int kCtrChunks = 7;                    // Soa::counts: pool chunks run in this render
constexpr uint64_t kMaxChunks = 1u << 20;       // bound on pool chunks per render
constexpr int kErrQueueTimeout = 4;              // error-flag bit: the work queue did not drain

struct PView {
    ViewParams vp;
    float* accum;
    float* path_out;
    float* aov;
    uint32_t history;
    uint32_t pix_begin;
    uint32_t npix;
    uint32_t pad;
};

struct LaunchBlock {
    uint32_t nviews;
    uint32_t total_pix;
    uint32_t spp;
    uint32_t max_chunks;      // bound on this render's chunks (a generous multiple of the work's own bound)
    float box_lo[4];          // scene bounds for the ray-reordering key
    float box_scale[4];       // 128 / extent per axis
    PView views[kMaxViews];
};

__device__ __forceinline__ uint32_t find_view(const LaunchBlock* lb, uint32_t g) {
    uint32_t lo = 0, hi = lb->nviews - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (lb->views[mid].pix_begin <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr uint32_t kFlagDelta = 1u << 10, kFlagShL = 1u << 11, kFlagShE = 1u << 12;

__device__ __forceinline__ float4 f4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float4 ld_hit(const Soa& s, uint32_t p) {
    const uint4 h = s.hm[2 * p + 1];
    return make_float4(__uint_as_float(h.x), __uint_as_float(h.y), __uint_as_float(h.z), __uint_as_float(h.w));
}
// the hit record and its instance, as extend writes them
__device__ __forceinline__ void st_hit(const Soa& s, uint32_t p, const Hit& h) {
    s.hm[2 * p + 1] = make_uint4(__float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v), h.prim);
    s.hm[2 * p].w = h.inst;
}

// The first-hit record (fhP, fhN, fhAlb) is written by the primary step and
// read only while the specular chain runs (the diffuse chain starts from it),
// so it moves through memory only then: with_first_hit on the store after a
// primary step, and on the load when the path is in its specular chain.
__device__ __forceinline__ void store_state(const Soa& s, uint32_t p, const PathState& ps, uint32_t extra_flags,
                                            bool with_first_hit) {
    // the hit instance (w) is the next extend's to write
    s.hm[2 * p] = make_uint4(ps.rng, ps.dim, ps.phase | (ps.bounce << 2) | (ps.delta ? kFlagDelta : 0u) | extra_flags, 0u);
    s.ray[2 * p] = f4(ps.ro, 0.0f);
    s.ray[2 * p + 1] = f4(ps.rd, ps.last_pdf);
    s.tr[2 * p] = f4(ps.thr, 0.0f);
    s.tr[2 * p + 1] = f4(ps.rad, 0.0f);
    if (with_first_hit) {
        s.fhP[p] = f4(ps.fhP, 0.0f);
        s.fhN[p] = f4(ps.fhN, 0.0f);
        s.fhA[p] = f4(ps.fhAlb, 0.0f);
    }
}
__device__ __forceinline__ void load_state(const Soa& s, uint32_t p, PathState& ps) {
    const uint4 m = s.hm[2 * p];
    ps.rng = m.x;
    ps.dim = m.y;
    const uint32_t f = m.z;
    ps.phase = f & 3u;
    ps.bounce = (f >> 2) & 0xFFu;
    ps.delta = (f & kFlagDelta) != 0u;
    const float4 ro = s.ray[2 * p], rd = s.ray[2 * p + 1];
    ps.ro = ld3(ro);
    ps.rd = ld3(rd);
    ps.last_pdf = rd.w;
    ps.thr = ld3(s.tr[2 * p]);
    ps.rad = ld3(s.tr[2 * p + 1]);
    if (ps.phase == kPhaseSpec) {
        ps.fhP = ld3(s.fhP[p]);
        ps.fhN = ld3(s.fhN[p]);
        ps.fhAlb = ld3(s.fhA[p]);
    } else {
        ps.fhP = ps.fhN = ps.fhAlb = v3s(0.0f);
    }
}

// Pixel of work rank j in a w x h view. Waves and the pool's work queue take
// pixels in rank order; ranks run over 8x4 tiles in row-major tile order (a
// warp's 32 consecutive paths cover one tile, so its primary rays and first
// hits are compact), then the pixels right of and below the whole tiles, row
// by row. Every output is written at the pixel's own index py * w + px.
__device__ __forceinline__ void rank_pixel(uint32_t j, uint32_t w, uint32_t h, uint32_t& px, uint32_t& py) {
    const uint32_t tw = w / 8u, th = h / 4u, nt = tw * th * 32u;
    if (j < nt) {
        const uint32_t t = j >> 5, r = j & 31u;
        px = (t % tw) * 8u + (r & 7u);
        py = (t / tw) * 4u + (r >> 3);
        return;
    }
    j -= nt;
    const uint32_t rw = w - tw * 8u, rh = th * 4u;
    if (j < rw * rh) {
        px = tw * 8u + j % rw;
        py = j / rw;
        return;
    }
    j -= rw * rh;
    px = j % w;
    py = rh + j / w;
}

// warp-aggregated queue append; returns the slot or ~0u
__device__ __forceinline__ uint32_t warp_push(uint32_t* counter, bool pred) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, pred);
    if (m == 0u) return 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(m)));
    base = __shfl_sync(act, base, leader);
    if (!pred) return 0xFFFFFFFFu;
    return base + static_cast<uint32_t>(__popc(m & ((1u << lane) - 1u)));
}

__global__ void k_generate(ViewParams vp, PathParams pp, uint32_t w0, uint32_t n, uint32_t npix, Soa s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) s.counts[0] = n;
    if (i >= n) return;
    const uint32_t lin = w0 + i;
    const uint32_t k = lin / npix, p = vp.pix_base + (lin - k * npix);   // npix: the lane's pixels
    uint32_t px, py;
    rank_pixel(p, vp.width, vp.height, px, py);
    PathState ps;
    path_start(vp, pp, px, py, pp.sample_base + k, ps);
    store_state(s, i, ps, 0u, false);
    s.q_ray[0][i] = i;
}

// Profiling counters (rays, nodes, triangles) summed over the warp first: one
// atomic per warp and counter, so the counting kernels run at the speed of
// the plain ones they stand in for when timed. Call with the whole warp.
__device__ __forceinline__ void add_stats(unsigned long long* dst, uint32_t rays, const TravCount& tc) {
    uint32_t v[3] = {rays, tc.nodes, tc.tris};
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], off);
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k)
            if (v[k]) atomicAdd(dst + k, static_cast<unsigned long long>(v[k]));
}

// stats (profiling only): [0] rays, [1] nodes, [2] triangles
// kLevels: 1 = flat BVH, 2 = two-level (one kernel per scene kind).
// Registers capped for 8 resident blocks per SM on flat scenes (64
// registers), 5 on two-level ones. On flat scenes the first
// kShStackEntries stack entries of each ray live in shared memory.
constexpr int kShStackEntries = 8;
template <bool kStats, int kLevels, bool kAlpha>
__global__ void __launch_bounds__(128, kLevels == 1 ? 8 : 5) k_extend(DScene sc, Soa s, int cur, int* err,
                                                                       unsigned long long* stats) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    constexpr int kSh = kLevels == 1 ? kShStackEntries : 0;
    __shared__ uint2 s_stack[kSh > 0 ? kSh * kShStride : 1];
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const float4 ro = s.ray[2 * p], rd = s.ray[2 * p + 1];
        const Hit h = scene_closest<kStats, kLevels, kAlpha, kSh>(sc, ld3(ro), ld3(rd), 0.001f, 10000.0f, tc, e,
                                                                  s_stack + threadIdx.x);
        st_hit(s, p, h);
        nr++;
    }
    if (e) atomicOr(err, 1);
    if (kStats) add_stats(stats + 0, nr, tc);
}

// kPool: slot -> (pixel, sample) comes from the pool arrays and the view
// table; finished paths are queued for regeneration. Otherwise a slot is
// the sample-major index inside the wave [w0, w0 + n) of one view.
// Registers capped for 8 resident blocks per SM: the step is latency-bound
// (scene and state loads, 21% of issue slots at 128 registers and 4 blocks),
// and 32 warps hide more of it than the spills cost (sphere_1m: 376 -> 402
// Msamples/s; 10 or 12 blocks gain under 1% more).
template <bool kPool, bool kTex, bool kMis, int kPhase>
__global__ void __launch_bounds__(128, 8) k_shade(DScene sc, PathParams pp, ViewParams vp_plain, uint32_t w0,
                                               uint32_t npix_plain, Soa s, int cur, float* aov_plain, uint32_t aov_k,
                                               const LaunchBlock* lb) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    uint32_t* qn = s.q_ray[cur ^ 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        uint32_t k, pix;
        const ViewParams* vpp;
        float* aov;
        if (kPool) {
            const uint32_t g = s.pix[p];
            const PView& pv = lb->views[find_view(lb, g)];
            k = s.smp[p];
            pix = g - pv.pix_begin;
            vpp = &pv.vp;
            aov = pv.aov;
        } else {
            const uint32_t lin = w0 + p;
            k = lin / npix_plain;
            pix = vp_plain.pix_base + (lin - k * npix_plain);
            vpp = &vp_plain;
            aov = aov_plain;
        }
        const ViewParams& vp = *vpp;
        uint32_t px, py;
        rank_pixel(pix, vp.width, vp.height, px, py);
        pix = py * vp.width + px;
        PathState ps;
        load_state(s, p, ps);
        const float4 hv = ld_hit(s, p);
        Hit h;
        h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_uint(hv.w); h.inst = s.hm[2 * p].w;
        const bool primary = ps.phase == kPhasePrimary;
        ShadowReq qL, qE;
        AovOut ao;
        const bool want_aov = aov != nullptr && primary && k == aov_k;
        const bool more = path_step<kTex, kMis, kPhase>(sc, pp, vp, px, py, pp.sample_base + k, ps, h, qL, qE,
                                                        want_aov ? &ao : nullptr);
        uint32_t extra = 0;
        if (qL.valid) {
            extra |= kFlagShL;
            s.shL[p] = f4(qL.dir, qL.tmax);
            s.shLc[p] = f4(qL.contrib, 0.0f);
            s.sh_org[p] = f4(qL.org, 0.0f);
        }
        if (qE.valid) {
            extra |= kFlagShE;
            s.shE[p] = f4(qE.dir, qE.tmax);
            s.shEc[p] = f4(qE.contrib, 0.0f);
            s.sh_org[p] = f4(qE.org, 0.0f);
        }
        store_state(s, p, ps, extra, primary && ps.phase == kPhaseSpec);
        if (want_aov) {
            float4* a = reinterpret_cast<float4*>(aov + static_cast<size_t>(pix) * OHAO_PT_AOV_FLOATS);
            a[0] = make_float4(ao.albedo.x, ao.albedo.y, ao.albedo.z, ao.normal.x);
            a[1] = make_float4(ao.normal.y, ao.normal.z, ao.depth, ao.hit);
            a[2] = make_float4(ao.rough, ao.metal, 0.0f, 0.0f);
        }
        const uint32_t slot = warp_push(s.counts + (cur ^ 1), more);
        if (slot != 0xFFFFFFFFu) qn[slot] = p;
        const uint32_t sslot = warp_push(s.counts + 2, extra != 0u);
        if (sslot != 0xFFFFFFFFu) s.q_sh[sslot] = p;
        if (kPool) {
            const uint32_t dslot = warp_push(s.counts + 3, !more);
            if (dslot != 0xFFFFFFFFu) s.q_done[dslot] = p;
        }
    }
}

// The shading step for the scene's features (bindless textures, emitter MIS)
// and its queue (phase 1: every path at its camera ray, the first step of a
// per-view wave; 2: every path in a chain, its later steps; 0: mixed, the
// pool).
template <bool kPool, int kPhase>
void launch_shade(const DScene& sc, const PathParams& pp, const ViewParams& vp, uint32_t w0, uint32_t npix, const Soa& s,
                  int cur, float* aov, uint32_t aov_k, const LaunchBlock* lb, cudaStream_t st);

// Pool ray reordering: 24-bit key = direction octant (3 bits, most
// significant) + Morton code of the origin on a 128^3 grid over the scene box.
__device__ __forceinline__ uint32_t spread7(uint32_t v) {
    v &= 0x7Fu;
    v = (v | (v << 8)) & 0x0000F00Fu;
    v = (v | (v << 4)) & 0x000C30C3u;
    v = (v | (v << 2)) & 0x00249249u;
    return v;
}

__global__ void k_ray_keys(const LaunchBlock* lb, Soa s, int cur) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const float4 o = s.ray[2 * p], d = s.ray[2 * p + 1];
        const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
        // a point 1/8 of the scene box along the ray: groups primary rays of
        // one camera by image region and secondary rays by origin and direction
        const float fx = (o.x - lb->box_lo[0]) * lb->box_scale[0] + d.x * 16.0f;
        const float fy = (o.y - lb->box_lo[1]) * lb->box_scale[1] + d.y * 16.0f;
        const float fz = (o.z - lb->box_lo[2]) * lb->box_scale[2] + d.z * 16.0f;
        const uint32_t ix = static_cast<uint32_t>(fminf(fmaxf(fx, 0.0f), 127.0f));
        const uint32_t iy = static_cast<uint32_t>(fminf(fmaxf(fy, 0.0f), 127.0f));
        const uint32_t iz = static_cast<uint32_t>(fminf(fmaxf(fz, 0.0f), 127.0f));
        s.skA[i] = (oct << 21) | (spread7(ix) << 2) | (spread7(iy) << 1) | spread7(iz);
        s.svA[i] = p;
    }
}

// Ray-queue binning: a counting sort of queue `cur` into at most kBinsMax bins of a
// small key, so that a warp's lanes take the same branches (material key,
// before shading) or walk similar parts of the BVH (ray key, before a
// bounce's traversal). Not stable -- the order inside a bin follows the
// atomics -- which changes nothing but the order paths are processed in:
// every path's result is its own. Two kernels: keys + block histograms,
// then the scatter (each block scans the bin counts itself and reserves one
// range per bin and block tile).
constexpr int kBinsMax = 512;
constexpr int kBinTile = 1024;   // entries per block tile of the scatter (8 per thread)

// Material key (OHAO_PT_FLAG_SORT_MATERIAL): bit 5 miss, bits 4-3 the
// path's phase (primary, specular chain, diffuse chain), then for hits bit
// 2 metallic >= 0.5, bit 1 roughness >= 0.5, bit 0 a textured material.
// Ray key (OHAO_PT_FLAG_SORT_RAYS): direction octant (bits 8-6) and the
// origin's quarter of the scene box per axis (bits 5-0).
template <int kMode>
__device__ __forceinline__ uint32_t bin_key(const DScene& sc, const Soa& s, uint32_t p) {
    if (kMode == 0) {
        const uint4 m = s.hm[2 * p];
        const uint32_t phase = m.z & 3u;
        const uint32_t prim = s.hm[2 * p + 1].w;
        if (prim == 0xFFFFFFFFu) return 32u | (phase << 3);
        const DInst& in = sc.inst[m.w];
        const uint32_t mid = __ldg(sc.mat_ids + (__ldg(&in.custom) & 0xFFFFFFu) + prim);
        const float4 m0 = __ldg(sc.mats + mid * 3), m1 = __ldg(sc.mats + mid * 3 + 1), m2 = __ldg(sc.mats + mid * 3 + 2);
        const bool tex = (__float_as_uint(m0.w) & __float_as_uint(m1.z) & __float_as_uint(m1.w) &
                          __float_as_uint(m2.x)) != 0xFFFFFFFFu;
        return (phase << 3) | (m1.y >= 0.5f ? 4u : 0u) | (m1.x >= 0.5f ? 2u : 0u) | (tex ? 1u : 0u);
    } else {
        const float4 o = s.ray[2 * p], d = s.ray[2 * p + 1];
        const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
        auto quarter = [&](float v, int a) {
            const float f = (v - sc.box_lo[a]) * sc.box_inv[a];
            return static_cast<uint32_t>(fminf(fmaxf(f, 0.0f), 3.0f));
        };
        return (oct << 6) | (quarter(o.x, 0) << 4) | (quarter(o.y, 1) << 2) | quarter(o.z, 2);
    }
}

// h[key] += 1 for every active lane, one shared-memory atomic per distinct
// key of the warp (the keys are few, so per-lane atomics would serialise on
// the same words); returns the lane's slot among the entries it added.
__device__ __forceinline__ uint32_t warp_bin_add(uint32_t* h, uint32_t key) {
    const uint32_t peers = __match_any_sync(__activemask(), key);
    const int leader = __ffs(peers) - 1;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0u;
    if (static_cast<int>(lane) == leader) base = atomicAdd(&h[key], static_cast<uint32_t>(__popc(peers)));
    base = __shfl_sync(peers, base, leader);
    return base + static_cast<uint32_t>(__popc(peers & ((1u << lane) - 1u)));
}

// Bins of each key: 6-bit material keys, 9-bit ray keys.
template <int kMode> constexpr int kBinsOf = kMode == 0 ? 64 : 512;

template <int kMode>
__global__ void __launch_bounds__(128) k_bin_count(DScene sc, Soa s, int cur, uint32_t* bins) {
    constexpr int kB = kBinsOf<kMode>;
    __shared__ uint32_t h[kB];
    for (int b = threadIdx.x; b < kB; b += blockDim.x) h[b] = 0u;
    __syncthreads();
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const uint32_t key = bin_key<kMode>(sc, s, p);
        s.skA[i] = key;
        s.svA[i] = p;
        warp_bin_add(h, key);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kB; b += blockDim.x)
        if (h[b]) atomicAdd(&bins[b], h[b]);
}

// Scatter of the keyed entries into queue `cur` in bin order. Every block
// takes the bins' exclusive prefix from the counts itself (warp 0: kB / 32
// consecutive bins per lane, then a shuffle scan), and reserves each block
// tile's range of a bin with one atomic on that bin's cursor (zero at entry).
template <int kMode>
__global__ void __launch_bounds__(128) k_bin_scatter(Soa s, int cur, const uint32_t* bins, uint32_t* cursors) {
    constexpr int kB = kBinsOf<kMode>;
    constexpr int kPerLane = kB / 32;
    __shared__ uint32_t base[kB], tc[kB], tb[kB];
    const uint32_t count = s.counts[cur];
    if (blockIdx.x * kBinTile >= count) return;   // uniform per block
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        uint32_t v[kPerLane], sum = 0u;
#pragma unroll
        for (int j = 0; j < kPerLane; ++j) {
            v[j] = bins[lane * kPerLane + j];
            sum += v[j];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= off) incl += x;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int j = 0; j < kPerLane; ++j) {
            base[lane * kPerLane + j] = run;
            run += v[j];
        }
    }
    uint32_t* q = s.q_ray[cur];
    constexpr int kPer = kBinTile / 128;
    for (uint32_t t0 = blockIdx.x * kBinTile; t0 < count; t0 += gridDim.x * kBinTile) {   // uniform per block
        for (int b = threadIdx.x; b < kB; b += blockDim.x) tc[b] = 0u;
        __syncthreads();
        uint32_t key[kPer], rank[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = t0 + j * 128 + threadIdx.x;
            key[j] = 0u;
            rank[j] = 0u;
            if (i < count) {
                key[j] = s.skA[i];
                rank[j] = warp_bin_add(tc, key[j]);
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < kB; b += blockDim.x)
            if (tc[b]) tb[b] = base[b] + atomicAdd(&cursors[b], tc[b]);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = t0 + j * 128 + threadIdx.x;
            if (i < count) q[tb[key[j]] + rank[j]] = s.svA[i];
        }
        __syncthreads();
    }
}

__global__ void k_copy_queue(Soa s, int cur) {
    const uint32_t count = s.counts[cur];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        s.q_ray[cur][i] = s.svA[i];
}

// Pool: every slot starts idle and queued for regeneration.
__global__ void k_pool_init(Soa s, uint32_t cap) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        s.pix[i] = kIdle;
        s.q_done[i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s.counts[0] = 0;
        s.counts[1] = 0;
        s.counts[3] = cap;
        s.counts[4] = 0;
        s.counts[kCtrChunks] = 0;
    }
}

// End of one pool chunk inside the render's CUDA graph: the graph's while
// loop runs another chunk until the work queue is drained (no path in
// flight, nothing left to claim), and gives up after the render's chunk bound with
// the queue-timeout error bit. No host round trip between chunks.
__global__ void k_pool_continue(cudaGraphConditionalHandle loop, const LaunchBlock* lb, Soa s, int* err) {
    const uint32_t pending = s.counts[0], done = s.counts[3], claimed = s.counts[4];
    const bool drained = pending == 0 && done == 0 && claimed >= lb->total_pix;
    const uint32_t chunks = ++s.counts[kCtrChunks];
    bool more = !drained;
    if (more && chunks >= lb->max_chunks) {
        atomicOr(err, kErrQueueTimeout);
        more = false;
    }
    cudaGraphSetConditional(loop, more ? 1u : 0u);
}

// Pool regeneration (after the shadow pass of an iteration): a finished
// path is folded into its slot's running mean in sample order; the slot
// then starts the pixel's next sample, or writes the pixel and claims the
// next pixel of the work queue (one atomic per warp). New primary rays are
// appended to the ray queue of the coming iteration.
__global__ void __launch_bounds__(128) k_regen(PathParams pp, const LaunchBlock* lb, Soa s, int cur) {
    const uint32_t count = s.counts[3];
    uint32_t* q = s.q_ray[cur];
    const uint32_t total = lb->total_pix, spp = lb->spp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = s.q_done[i];
        uint32_t g = s.pix[p];
        uint32_t k = s.smp[p];
        float4 acc = s.acc[p];
        bool start = false;
        if (g != kIdle) {
            const PView& pv = lb->views[find_view(lb, g)];
            uint32_t px, py;
            rank_pixel(g - pv.pix_begin, pv.vp.width, pv.vp.height, px, py);
            const uint32_t pix = py * pv.vp.width + px;
            const V3 L = firefly(pp, ld3(s.tr[2 * p + 1]));
            if (pv.path_out)
                reinterpret_cast<float4*>(pv.path_out)[static_cast<size_t>(k) * pv.npix + pix] = f4(L, 0.0f);
            if (pv.history + k == 0) {
                acc = make_float4(L.x, L.y, L.z, 1.0f);
            } else {
                const float cnt = acc.w + 1.0f;
                acc.x = (acc.x * acc.w + L.x) / cnt;
                acc.y = (acc.y * acc.w + L.y) / cnt;
                acc.z = (acc.z * acc.w + L.z) / cnt;
                acc.w = cnt;
            }
            k++;
            if (k < spp) {
                start = true;
            } else {
                reinterpret_cast<float4*>(pv.accum)[pix] = acc;
                g = kIdle;
            }
        }
        const uint32_t claim = warp_push(s.counts + 4, g == kIdle);
        if (g == kIdle && claim < total) {
            g = claim;
            k = 0;
            const PView& pv = lb->views[find_view(lb, g)];
            uint32_t px, py;
            rank_pixel(g - pv.pix_begin, pv.vp.width, pv.vp.height, px, py);
            acc = pv.history > 0 ? reinterpret_cast<const float4*>(pv.accum)[py * pv.vp.width + px]
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            start = true;
        }
        if (start) {
            const PView& pv = lb->views[find_view(lb, g)];
            uint32_t px, py;
            rank_pixel(g - pv.pix_begin, pv.vp.width, pv.vp.height, px, py);
            PathState ps;
            path_start(pv.vp, pp, px, py, pp.sample_base + k, ps);
            store_state(s, p, ps, 0u, false);
        } else {
            g = kIdle;
        }
        s.pix[p] = g;
        s.smp[p] = k;
        s.acc[p] = acc;
        const uint32_t slot = warp_push(s.counts + cur, start);
        if (slot != 0xFFFFFFFFu) q[slot] = p;
    }
}

// stats (profiling only): [3] shadow rays, [4] nodes, [5] triangles
template <bool kStats, int kLevels, bool kAlpha>
__global__ void __launch_bounds__(128, kLevels == 1 ? 8 : 5) k_shadow(DScene sc, Soa s, int* err,
                                                                       unsigned long long* stats) {
    const uint32_t count = s.counts[2];
    constexpr int kSh = 0;   // a shared-memory stack measured slower for shadow rays (less L1 for nodes)
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = s.q_sh[i];
        const uint32_t f = s.hm[2 * p].z;
        const V3 org = ld3(s.sh_org[p]);
        V3 rad = ld3(s.tr[2 * p + 1]);
        if (f & kFlagShL) {
            const float4 d = s.shL[p];
            nr++;
            if (!scene_occluded<kStats, kLevels, kAlpha, kSh>(sc, org, ld3(d), 0.001f, d.w, tc, e, nullptr))
                rad = rad + ld3(s.shLc[p]);
        }
        if (f & kFlagShE) {
            const float4 d = s.shE[p];
            nr++;
            if (!scene_occluded<kStats, kLevels, kAlpha, kSh>(sc, org, ld3(d), 0.001f, d.w, tc, e, nullptr))
                rad = rad + ld3(s.shEc[p]);
        }
        s.tr[2 * p + 1] = f4(rad, 0.0f);
        s.hm[2 * p].z = f & ~(kFlagShL | kFlagShE);
    }
    if (e) atomicOr(err, 1);
    if (kStats) add_stats(stats + 3, nr, tc);
}

// Pool extend / shadow with persistent warps (flat or two-level scenes). A lane
// whose ray finished takes the next one from the queue while the other lanes
// carry on: once at least `refill` lanes of a warp are idle, one atomic on the
// queue's fetch counter claims rays for all of them. A warp therefore does
// not wait for its longest ray before taking more work -- in instanced scenes
// per-ray step counts vary by orders of magnitude. Results equal those of
// k_extend / k_shadow (see pt_fetch.cuh); the shadow rays of one path run in
// one lane, light ray first, so their contributions add in the same order.
constexpr int kCtrExtendFetch = 5, kCtrShadowFetch = 6;   // fetch counters in Soa::counts

struct WarpFetch {
    bool drained = false;
    // Claims up to one queue index per idle lane; returns this lane's index
    // (>= count: none). Call with the whole warp.
    __device__ __forceinline__ uint32_t claim(bool idle_lane, uint32_t* ctr, uint32_t count, int refill) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, idle_lane);
        const uint32_t nidle = __popc(idle);
        if (drained || static_cast<int>(nidle) < refill) return 0xFFFFFFFFu;
        const uint32_t lane = threadIdx.x & 31u;
        uint32_t b = 0u;
        if (lane == 0u) b = atomicAdd(ctr, nidle);
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (b >= count || count - b <= nidle) drained = true;
        if (!idle_lane) return 0xFFFFFFFFu;
        const uint32_t i = b + __popc(idle & ((1u << lane) - 1u));
        return i < count ? i : 0xFFFFFFFFu;
    }
};

template <bool kStats, int kLevels, bool kAlpha>
__global__ void __launch_bounds__(128) k_extend_fetch(DScene sc, Soa s, int cur, int refill, int* err,
                                                      unsigned long long* stats) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    uint32_t st_node[kStackSize];
    float st_t[kStackSize];
    Walk w;
    RayPre r;
    uint32_t p = 0u;
    bool active = false;
    WarpFetch wf;
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    while (true) {
        const uint32_t i = wf.claim(!active, s.counts + kCtrExtendFetch, count, refill);
        if (i != 0xFFFFFFFFu) {
            p = q[i];
            r = ray_pre(ld3(s.ray[2 * p]), ld3(s.ray[2 * p + 1]));
            walk_begin<kLevels>(sc, w, r);
            active = true;
            nr++;
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
            if (wf.drained) break;
            continue;
        }
        if (active && walk_step<kLevels, kStats, kAlpha>(sc, w, r, 0.001f, 10000.0f, st_node, st_t, e, &tc)) {
            st_hit(s, p, w.best);
            active = false;
        }
    }
    if (e) atomicOr(err, 1);
    if (kStats) add_stats(stats + 0, nr, tc);
}

// Closest hit, flat BVH, one ray per lane with refill: a warp's lanes take
// one traversal step (closest_step: a node with its triangle leaves, or a
// pop) per loop turn, and a lane whose ray is done takes the next queue
// entry once `refill` lanes are idle -- so a warp no longer waits for its
// longest ray -- while each ray's steps stay those of scene_closest (same
// hits, same visit counts).
template <bool kStats, bool kAlpha>
__global__ void __launch_bounds__(128, 8) k_extend_refill(DScene sc, Soa s, int cur, int refill, int* err,
                                                          unsigned long long* stats) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    __shared__ uint2 s_stack[kShStackEntries * kShStride];
    TravStack<kShStackEntries> stk;
    stk.sh = s_stack + threadIdx.x;
    const int lim = stack_limit(sc);
    RayPre r;
    Hit best;
    uint32_t node = 0u, p = 0u;
    float node_tn = 0.0f;
    int sp = 0;
    bool active = false;
    WarpFetch wf;
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    while (true) {
        const uint32_t i = wf.claim(!active, s.counts + kCtrExtendFetch, count, refill);
        if (i != 0xFFFFFFFFu) {
            p = q[i];
            r = ray_pre(ld3(s.ray[2 * p]), ld3(s.ray[2 * p + 1]));
            best.t = 0.0f; best.u = 0.0f; best.v = 0.0f;
            best.inst = 0xFFFFFFFFu; best.prim = 0xFFFFFFFFu;
            node = 0u;
            node_tn = -INFINITY;
            sp = 0;
            active = sc.nnodes > 0 && lim > 0;
            if (!active) st_hit(s, p, best);   // no geometry: a miss without a walk
            nr++;
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
            if (wf.drained) break;
            continue;
        }
        if (active && closest_step<kStats, kAlpha>(sc, sc.nodes, sc.tris, r, 0.001f, 10000.0f, best, 0xFFFFFFFFu, stk,
                                                   0, lim, tc, e, sp, node, node_tn)) {
            st_hit(s, p, best);
            active = false;
        }
    }
    if (e) atomicOr(err, 1);
    if (kStats) add_stats(stats + 0, nr, tc);
}

// Starts shadow ray `which` (0 light, 1 environment) of path p; a ray with
// tmax <= tmin is unoccluded without a walk (as in scene_occluded).
template <int kLevels>
__device__ __forceinline__ void start_shadow(const DScene& sc, const Soa& s, uint32_t p, int which, Probe& w,
                                             RayPre& r) {
    const float4 d = which == 0 ? s.shL[p] : s.shE[p];
    r = ray_pre(ld3(s.sh_org[p]), ld3(d));
    probe_begin<kLevels>(sc, w, r);
    if (!(d.w > 0.001f)) w.have_node = false;   // the next step ends the walk unoccluded
}

template <bool kStats, int kLevels, bool kAlpha>
__global__ void __launch_bounds__(128) k_shadow_fetch(DScene sc, Soa s, int refill, int* err,
                                                      unsigned long long* stats) {
    const uint32_t count = s.counts[2];
    uint32_t st_node[kStackSize];
    Probe w;
    RayPre r;
    float tmax = 0.0f;
    uint32_t p = 0u, f = 0u;
    int which = 0;
    bool visL = false;
    bool active = false;
    WarpFetch wf;
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    while (true) {
        const uint32_t i = wf.claim(!active, s.counts + kCtrShadowFetch, count, refill);
        if (i != 0xFFFFFFFFu) {
            p = s.q_sh[i];
            f = s.hm[2 * p].z;
            which = (f & kFlagShL) ? 0 : 1;
            start_shadow<kLevels>(sc, s, p, which, w, r);
            tmax = which == 0 ? s.shL[p].w : s.shE[p].w;
            visL = false;
            active = true;
            nr++;
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
            if (wf.drained) break;
            continue;
        }
        if (active && probe_step<kLevels, kStats, kAlpha>(sc, w, r, 0.001f, tmax, st_node, e, &tc)) {
            if (which == 0) visL = !w.hit;
            if (which == 0 && (f & kFlagShE)) {
                which = 1;
                start_shadow<kLevels>(sc, s, p, 1, w, r);
                tmax = s.shE[p].w;
                nr++;
            } else {
                const bool visE = which == 1 && !w.hit;
                V3 rad = ld3(s.tr[2 * p + 1]);
                if (visL) rad = rad + ld3(s.shLc[p]);
                if (visE) rad = rad + ld3(s.shEc[p]);
                s.tr[2 * p + 1] = f4(rad, 0.0f);
                s.hm[2 * p].z = f & ~(kFlagShL | kFlagShE);
                active = false;
            }
        }
    }
    if (e) atomicOr(err, 1);
    if (kStats) add_stats(stats + 3, nr, tc);
}

// p: the pixel's work rank (slots are rank-major); outputs at its index.
// One wave of a lane: npix = the lane's pixel count, ranks from vp.pix_base.
__global__ void k_finalize(PathParams pp, uint32_t w0, uint32_t n, ViewParams vp, uint32_t npix, Soa s,
                           float* accum, uint32_t history, float* path_out) {
    const uint32_t width = vp.width, height = vp.height;
    const uint32_t view_npix = width * height;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const uint64_t lo = w0, hi = static_cast<uint64_t>(w0) + n;   // [lo, hi)
        uint64_t k0 = (lo > p) ? (lo - p + npix - 1) / npix : 0;
        if (k0 * npix + p >= hi) continue;
        const uint64_t k1 = (hi - 1 - p) / npix;
        uint32_t px, py;
        rank_pixel(vp.pix_base + p, width, height, px, py);
        const uint32_t pidx = py * width + px;
        float4 acc = reinterpret_cast<float4*>(accum)[pidx];
        for (uint64_t k = k0; k <= k1; ++k) {
            const uint32_t slot = static_cast<uint32_t>(k * npix + p - lo);
            const V3 L = firefly(pp, ld3(s.tr[2 * slot + 1]));
            if (path_out) reinterpret_cast<float4*>(path_out)[k * view_npix + pidx] = f4(L, 0.0f);
            if (history + k == 0) {
                acc = make_float4(L.x, L.y, L.z, 1.0f);
            } else {
                const float cnt = acc.w + 1.0f;
                acc.x = (acc.x * acc.w + L.x) / cnt;
                acc.y = (acc.y * acc.w + L.y) / cnt;
                acc.z = (acc.z * acc.w + L.z) / cnt;
                acc.w = cnt;
            }
        }
        reinterpret_cast<float4*>(accum)[pidx] = acc;
    }
}

__global__ void __launch_bounds__(128) k_trace(DScene sc, const float* __restrict__ rays, uint32_t n,
                                               uint32_t* __restrict__ hits, int any, uint32_t* __restrict__ stats,
                                               int* err) {
    int e = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(rays)[2 * i];
        const float4 b = reinterpret_cast<const float4*>(rays)[2 * i + 1];
        TravCount tc{0, 0};
        uint32_t* h = hits + static_cast<size_t>(i) * 5;
        if (any) {
            const bool occ = stats ? scene_occluded<true, 0, true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e)
                                   : scene_occluded<false, 0, true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e);
            h[0] = occ ? 1u : 0u; h[1] = 0u; h[2] = 0u; h[3] = 0xFFFFFFFFu; h[4] = 0xFFFFFFFFu;
        } else {
            const Hit r = stats ? scene_closest<true, 0, true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e)
                                : scene_closest<false, 0, true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e);
            if (r.prim != 0xFFFFFFFFu) {
                h[0] = __float_as_uint(r.t); h[1] = __float_as_uint(r.u); h[2] = __float_as_uint(r.v);
                h[3] = r.inst; h[4] = r.prim;
            } else {
                h[0] = 0u; h[1] = 0u; h[2] = 0u; h[3] = 0xFFFFFFFFu; h[4] = 0xFFFFFFFFu;
            }
        }
        if (stats) { stats[2 * i] = tc.nodes; stats[2 * i + 1] = tc.tris; }
    }
    if (e) atomicOr(err, 1);
}

// Carves 256-byte aligned arrays out of one scratch block; with a null base
// it only measures (off = bytes needed).
struct Carve {
    char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t count) {
        const size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        T* r = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += bytes;
        return r;
    }
};

Soa carve_soa_at(Carve& c, uint32_t cap) {
    Soa s;
    s.ray = c.take<float4>(2 * static_cast<size_t>(cap));
    s.tr = c.take<float4>(2 * static_cast<size_t>(cap));
    s.hm = c.take<uint4>(2 * static_cast<size_t>(cap));
    s.fhP = c.take<float4>(cap);
    s.fhN = c.take<float4>(cap);
    s.fhA = c.take<float4>(cap);

    s.sh_org = c.take<float4>(cap);
    s.shL = c.take<float4>(cap);
    s.shLc = c.take<float4>(cap);
    s.shE = c.take<float4>(cap);
    s.shEc = c.take<float4>(cap);
    s.q_ray[0] = c.take<uint32_t>(cap);
    s.q_ray[1] = c.take<uint32_t>(cap);
    s.q_sh = c.take<uint32_t>(cap);
    s.counts = c.take<uint32_t>(64);
    s.pix = c.take<uint32_t>(cap);
    s.smp = c.take<uint32_t>(cap);
    s.acc = c.take<float4>(cap);
    s.q_done = c.take<uint32_t>(cap);
    s.skA = c.take<uint32_t>(cap);
    s.svA = c.take<uint32_t>(cap);
    s.skB = c.take<uint32_t>(cap);
    s.svB = c.take<uint32_t>(cap);
    // radix-sort tile histograms, or the binning's counts and cursors
    s.shist = c.take<uint32_t>(std::max<size_t>(16 * static_cast<size_t>(rsort::tiles_for(cap)), 2 * static_cast<size_t>(kBinsMax)));
    return s;
}

Soa carve_soa(void* base, uint32_t cap) {
    Carve c{static_cast<char*>(base)};
    return carve_soa_at(c, cap);
}

int g_num_sms = 0;
constexpr int kTraversalWaves = 4;
int g_blocks_extend[2] = {0, 0}, g_blocks_shadow[2] = {0, 0};   // [flat, two-level]
int g_blocks_shade = 0, g_blocks_trace = 0;
int g_blocks_fetch[4] = {0, 0, 0, 0};   // persistent-warp extend [flat, two-level], shadow [flat, two-level]
int g_blocks_refill = 0;                // k_extend_refill: one wave of resident blocks

void init_launch_shapes() {
    if (g_num_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend<false, 1, false>, 128, 0);
    g_blocks_extend[0] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend<false, 2, false>, 128, 0);
    g_blocks_extend[1] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade<false, false, false, 2>, 128, 0);
    g_blocks_shade = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shadow<false, 1, false>, 128, 0);
    g_blocks_shadow[0] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shadow<false, 2, false>, 128, 0);
    g_blocks_shadow[1] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace, 128, 0);
    g_blocks_trace = std::max(1, b) * g_num_sms;
    // traversal grids: 4 waves of resident blocks over the grid-stride ray
    // loop, so blocks that drew short rays are replaced by new ones while
    // long rays finish (+5% on sphere_1m against one wave)
    for (int k = 0; k < 2; ++k) {
        g_blocks_extend[k] *= kTraversalWaves;
        g_blocks_shadow[k] *= kTraversalWaves;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend_fetch<false, 1, false>, 128, 0);
    g_blocks_fetch[0] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend_fetch<false, 2, false>, 128, 0);
    g_blocks_fetch[1] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shadow_fetch<false, 1, false>, 128, 0);
    g_blocks_fetch[2] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shadow_fetch<false, 2, false>, 128, 0);
    g_blocks_fetch[3] = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend_refill<false, false>, 128, 0);
    g_blocks_refill = std::max(1, b) * g_num_sms;
}

template <bool kPool, int kPhase>
void launch_shade(const DScene& sc, const PathParams& pp, const ViewParams& vp, uint32_t w0, uint32_t npix, const Soa& s,
                  int cur, float* aov, uint32_t aov_k, const LaunchBlock* lb, cudaStream_t st) {
    const dim3 g(g_blocks_shade), b(128);
    if (sc.emitter_mis) {
        if (sc.ntex) k_shade<kPool, true, true, kPhase><<<g, b, 0, st>>>(sc, pp, vp, w0, npix, s, cur, aov, aov_k, lb);
        else k_shade<kPool, false, true, kPhase><<<g, b, 0, st>>>(sc, pp, vp, w0, npix, s, cur, aov, aov_k, lb);
    } else {
        if (sc.ntex) k_shade<kPool, true, false, kPhase><<<g, b, 0, st>>>(sc, pp, vp, w0, npix, s, cur, aov, aov_k, lb);
        else k_shade<kPool, false, false, kPhase><<<g, b, 0, st>>>(sc, pp, vp, w0, npix, s, cur, aov, aov_k, lb);
    }
}

// Kernel selection: statistics on/off x flat / two-level x alpha test
// compiled in or not (opaque rays keep the traversal at its register count).
#define OHAO_LAUNCH_TRAVERSAL(KERNEL, GRID, ...)                                                       \
    do {                                                                                               \
        const int lv = sc.two_level ? 2 : 1;                                                           \
        const bool al = sc.alpha_test != 0;                                                            \
        if (stats) {                                                                                   \
            if (lv == 2) { if (al) KERNEL<true, 2, true><<<GRID[1], 128, 0, st>>>(__VA_ARGS__);         \
                           else KERNEL<true, 2, false><<<GRID[1], 128, 0, st>>>(__VA_ARGS__); }        \
            else { if (al) KERNEL<true, 1, true><<<GRID[0], 128, 0, st>>>(__VA_ARGS__);                 \
                   else KERNEL<true, 1, false><<<GRID[0], 128, 0, st>>>(__VA_ARGS__); }                \
        } else {                                                                                       \
            if (lv == 2) { if (al) KERNEL<false, 2, true><<<GRID[1], 128, 0, st>>>(__VA_ARGS__);        \
                           else KERNEL<false, 2, false><<<GRID[1], 128, 0, st>>>(__VA_ARGS__); }       \
            else { if (al) KERNEL<false, 1, true><<<GRID[0], 128, 0, st>>>(__VA_ARGS__);                \
                   else KERNEL<false, 1, false><<<GRID[0], 128, 0, st>>>(__VA_ARGS__); }               \
        }                                                                                              \
    } while (0)

// persistent-warp closest-hit / any-hit kernels (the caller zeroes the
// fetch counters first)
// Persistent warps over the closest-hit queue: on a flat BVH one step is a
// node with its triangle leaves (k_extend_refill), on a two-level one a
// node, one triangle, an instance entry or a pop (k_extend_fetch).
void launch_extend_fetch(const DScene& sc, const Soa& s, int cur, int refill, int* d_err, unsigned long long* stats,
                         cudaStream_t st) {
    if (!sc.two_level) {
        const bool al = sc.alpha_test != 0;
        if (stats) {
            if (al) k_extend_refill<true, true><<<g_blocks_refill, 128, 0, st>>>(sc, s, cur, refill, d_err, stats);
            else k_extend_refill<true, false><<<g_blocks_refill, 128, 0, st>>>(sc, s, cur, refill, d_err, stats);
        } else {
            if (al) k_extend_refill<false, true><<<g_blocks_refill, 128, 0, st>>>(sc, s, cur, refill, d_err, stats);
            else k_extend_refill<false, false><<<g_blocks_refill, 128, 0, st>>>(sc, s, cur, refill, d_err, stats);
        }
        return;
    }
    OHAO_LAUNCH_TRAVERSAL(k_extend_fetch, g_blocks_fetch, sc, s, cur, refill, d_err, stats);
}
void launch_shadow(const DScene& sc, const Soa& s, int* d_err, unsigned long long* stats, cudaStream_t st);
// Persistent warps over the shadow queue on a two-level BVH; on a flat one
// the one-ray-per-thread any-hit kernel (its walks are short and alike:
// persistent warps measured 10% slower on sphere_1m).
void launch_shadow_fetch(const DScene& sc, const Soa& s, int refill, int* d_err, unsigned long long* stats,
                         cudaStream_t st) {
    if (!sc.two_level) {
        launch_shadow(sc, s, d_err, stats, st);
        return;
    }
    OHAO_LAUNCH_TRAVERSAL(k_shadow_fetch, (g_blocks_fetch + 2), sc, s, refill, d_err, stats);
}
// one-ray-per-thread closest-hit / any-hit kernels
void launch_extend(const DScene& sc, const Soa& s, int cur, int* d_err, unsigned long long* stats, cudaStream_t st) {
    OHAO_LAUNCH_TRAVERSAL(k_extend, g_blocks_extend, sc, s, cur, d_err, stats);
}
void launch_shadow(const DScene& sc, const Soa& s, int* d_err, unsigned long long* stats, cudaStream_t st) {
    OHAO_LAUNCH_TRAVERSAL(k_shadow, g_blocks_shadow, sc, s, d_err, stats);
}

constexpr uint32_t kFlagSortMaterial = OHAO_PT_FLAG_SORT_MATERIAL;
constexpr uint32_t kFlagSortRays = OHAO_PT_FLAG_SORT_RAYS;

constexpr int kBinLaunches = 2;   // kernels bin_queue launches

// Bins ray queue `cur` by the key of kMode (0 material, 1 ray); the bin
// counts and cursors live in the first 2 * kBinsOf<kMode> words of s.shist.
template <int kMode>
void bin_queue(const DScene& sc, const Soa& s, int cur, uint32_t cap, cudaStream_t st) {
    constexpr int kB = kBinsOf<kMode>;
    uint32_t* bins = s.shist;
    uint32_t* cursors = s.shist + kB;
    cudaMemsetAsync(bins, 0, 2 * kB * sizeof(uint32_t), st);
    k_bin_count<kMode><<<g_blocks_shade, 128, 0, st>>>(sc, s, cur, bins);
    const uint32_t tiles = (cap + kBinTile - 1) / kBinTile;
    k_bin_scatter<kMode><<<std::min<uint32_t>(tiles, static_cast<uint32_t>(g_num_sms) * 8u), 128, 0, st>>>(
        s, cur, bins, cursors);
}

// Profile-mode CUDA events around each section of a render, by kind (0
// extend, 1 shade, 2 shadow, 3 other) with the kernel launches inside it.
struct EvTimer {
    struct Sect {
        cudaEvent_t a, b;
        int launches;
    };
    bool on;
    cudaStream_t st;
    std::vector<Sect> ev[4];
    void begin(int kind, cudaEvent_t& a) {
        if (!on) return;
        cudaEventCreate(&a);
        cudaEventRecord(a, st);
        (void)kind;
    }
    void end(int kind, cudaEvent_t a, int launches = 1) {
        if (!on) return;
        cudaEvent_t b;
        cudaEventCreate(&b);
        cudaEventRecord(b, st);
        ev[kind].push_back({a, b, launches});
    }
    void collect(ProfileAcc* p) {
        if (!on || !p) return;
        cudaStreamSynchronize(st);
        for (int k = 0; k < 4; ++k) {
            for (auto& e : ev[k]) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e.a, e.b);
                if (k == 0) { p->extend_ms += ms; p->extend_launches += e.launches; }
                if (k == 1) { p->shade_ms += ms; p->shade_launches += e.launches; }
                if (k == 2) { p->shadow_ms += ms; p->shadow_launches += e.launches; }
                if (k == 3) { p->other_ms += ms; p->other_launches += e.launches; }
                cudaEventDestroy(e.a);
                cudaEventDestroy(e.b);
            }
            ev[k].clear();
        }
    }
};

}  // namespace


size_t wavefront_scratch_bytes(uint32_t cap) {
    Carve c{nullptr};
    carve_soa_at(c, cap);
    return c.off;
}

uint32_t wavefront_default_capacity() { return 1u << 21; }

size_t wavefront_lanes_scratch_bytes(uint32_t capacity) {
    Carve c{nullptr};
    for (int l = 0; l < kWaveLanes; ++l) carve_soa_at(c, capacity / kWaveLanes);
    return c.off;
}

ohao_status wavefront_render(const DScene& sc, const RenderView& view, const PathParams& pp, uint32_t spp,
                             void* scratch, size_t scratch_bytes, uint32_t capacity, cudaStream_t st, bool profile,
                             ProfileAcc* prof, int* d_err, std::string& err, const WaveStreams* ws) {
    init_launch_shapes();
    const uint32_t npix = view.vp.width * view.vp.height;
    // kWaveLanes lanes (a view of >= 64 pixels per lane, one ray per thread
    // in traversal, not profiled): the pixel ranks are split at multiples of
    // 32 (whole 8x4 tiles) and each slice renders all its samples on its own
    // stream with its share of the scratch, beside the others; the slices
    // share no pixel, so each pixel's samples still fold in order within one
    // lane. Persistent-warp traversal keeps one lane: its grids fill the GPU
    // by themselves, and two of them side by side measured 3% slower on the
    // instanced scene.
    const bool fetch = pp.refill > 0 && sc.nnodes > 0;
    const int lanes_unprofiled = (ws && ws->main[1] && !fetch && npix >= 64u * kWaveLanes) ? kWaveLanes : 1;
    const int nl = profile ? 1 : lanes_unprofiled;
    if (profile) prof->lanes = std::max<uint32_t>(prof->lanes, static_cast<uint32_t>(lanes_unprofiled));
    const uint32_t wcap = capacity / static_cast<uint32_t>(nl);
    if (scratch_bytes < (nl > 1 ? wavefront_lanes_scratch_bytes(capacity) : wavefront_scratch_bytes(capacity))) {
        err = "wavefront scratch too small";
        return OHAO_ERR_INVALID_ARG;
    }
    Soa lane_soa[kWaveLanes];
    uint32_t pix_base[kWaveLanes + 1], pix_count[kWaveLanes];
    {
        Carve c{static_cast<char*>(scratch)};
        for (int l = 0; l < nl; ++l) {
            lane_soa[l] = carve_soa_at(c, wcap);
            pix_base[l] = static_cast<uint32_t>(static_cast<uint64_t>(npix) * l / nl) & ~31u;
        }
        pix_base[nl] = npix;
        for (int l = 0; l < nl; ++l) pix_count[l] = pix_base[l + 1] - pix_base[l];
    }
    unsigned long long* dstats = reinterpret_cast<unsigned long long*>(lane_soa[0].counts + 16);
    if (profile) cudaMemsetAsync(dstats, 0, 8 * sizeof(unsigned long long), st);
    const uint32_t niters = 1 + 2 * pp.max_bounces;
    EvTimer tm{profile, st, {}};
    cudaEvent_t t_all0 = nullptr, t_all1 = nullptr;
    if (profile) {
        cudaEventCreate(&t_all0);
        cudaEventCreate(&t_all1);
        cudaEventRecord(t_all0, st);
    }
    // Shadow rays of step k and closest-hit rays of step k + 1 are
    // independent (different path fields, different queues and fetch
    // counters), so with an auxiliary stream the shadow kernel runs beside
    // the next extend and is joined before the next binning and shading: the
    // small queues of a frame's last steps then share the GPU instead of
    // running one after the other. Profiled renders stay serial (their
    // per-kernel timers are on one stream).
    cudaStream_t main_st[kWaveLanes], sh_st[kWaveLanes];
    bool overlap[kWaveLanes] = {};
    cudaEvent_t ev_shaded[kWaveLanes] = {}, ev_shadowed[kWaveLanes] = {}, ev_join[kWaveLanes] = {}, ev_fork = nullptr;
    for (int l = 0; l < nl; ++l) {
        main_st[l] = l == 0 ? st : ws->main[l];
        const cudaStream_t aux = ws ? ws->aux[l] : nullptr;
        overlap[l] = aux != nullptr && !profile;
        if (overlap[l]) {
            sh_st[l] = aux;
            cudaEventCreateWithFlags(&ev_shaded[l], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ev_shadowed[l], cudaEventDisableTiming);
        } else {
            sh_st[l] = main_st[l];
        }
    }
    if (nl > 1) {   // the other lanes start after the caller's work on st
        cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
        cudaEventRecord(ev_fork, st);
        for (int l = 1; l < nl; ++l) {
            cudaEventCreateWithFlags(&ev_join[l], cudaEventDisableTiming);
            cudaStreamWaitEvent(main_st[l], ev_fork, 0);
        }
    }
    // one wave of lane l: paths [w0, w0 + n) of the lane's (sample, pixel) space
    auto run_wave = [&](int l, uint64_t w0, uint32_t n) {
        const Soa& s = lane_soa[l];
        const cudaStream_t ms = main_st[l], ss = sh_st[l];
        ViewParams vp = view.vp;
        vp.pix_base = pix_base[l];
        const uint32_t pn = pix_count[l];
        cudaEvent_t a;
        tm.begin(3, a);
        k_generate<<<(n + 255) / 256, 256, 0, ms>>>(vp, pp, static_cast<uint32_t>(w0), n, pn, s);
        tm.end(3, a);
        int cur = 0;
        for (uint32_t it = 0; it < niters; ++it) {
            if (it > 0 && (pp.flags & kFlagSortRays)) {   // bounce rays grouped by direction and origin
                tm.begin(3, a);
                bin_queue<1>(sc, s, cur, wcap, ms);
                tm.end(3, a, kBinLaunches);
            }
            if (fetch) cudaMemsetAsync(s.counts + kCtrExtendFetch, 0, 4, ms);
            tm.begin(0, a);
            if (fetch) launch_extend_fetch(sc, s, cur, static_cast<int>(pp.refill), d_err, profile ? dstats : nullptr, ms);
            else launch_extend(sc, s, cur, d_err, profile ? dstats : nullptr, ms);
            tm.end(0, a);
            if (overlap[l] && it > 0) cudaStreamWaitEvent(ms, ev_shadowed[l], 0);   // step it - 1's shadow rays done
            if (pp.flags & kFlagSortMaterial) {
                tm.begin(3, a);
                bin_queue<0>(sc, s, cur, wcap, ms);
                tm.end(3, a, kBinLaunches);
            }
            cudaMemsetAsync(s.counts + (cur ^ 1), 0, 4, ms);
            cudaMemsetAsync(s.counts + 2, 0, 4, ms);
            tm.begin(1, a);
            if (it == 0)   // the wave's camera rays: every path at its first step
                launch_shade<false, 1>(sc, pp, vp, static_cast<uint32_t>(w0), pn, s, cur, view.aov, spp - 1, nullptr, ms);
            else
                launch_shade<false, 2>(sc, pp, vp, static_cast<uint32_t>(w0), pn, s, cur, view.aov, spp - 1, nullptr, ms);
            tm.end(1, a);
            if (overlap[l]) {
                cudaEventRecord(ev_shaded[l], ms);
                cudaStreamWaitEvent(ss, ev_shaded[l], 0);
            }
            tm.begin(2, a);
            if (fetch) cudaMemsetAsync(s.counts + kCtrShadowFetch, 0, 4, ss);
            if (fetch) launch_shadow_fetch(sc, s, static_cast<int>(pp.refill), d_err, profile ? dstats : nullptr, ss);
            else launch_shadow(sc, s, d_err, profile ? dstats : nullptr, ss);
            tm.end(2, a);
            if (overlap[l]) cudaEventRecord(ev_shadowed[l], ss);
            cur ^= 1;
        }
        if (overlap[l]) cudaStreamWaitEvent(ms, ev_shadowed[l], 0);   // the wave's last shadow rays
        if (view.accum_ready) cudaStreamWaitEvent(ms, view.accum_ready, 0);   // the history upload has landed
        tm.begin(3, a);
        k_finalize<<<std::max(1u, std::min(4096u, (pn + 255) / 256)), 256, 0, ms>>>(
            pp, static_cast<uint32_t>(w0), n, vp, pn, s, view.accum, view.history, view.path_out);
        tm.end(3, a);
    };
    uint64_t lane_total[kWaveLanes], most = 0;
    for (int l = 0; l < nl; ++l) {
        lane_total[l] = static_cast<uint64_t>(pix_count[l]) * spp;
        most = std::max(most, lane_total[l]);
    }
    for (uint64_t w0 = 0; w0 < most; w0 += wcap)
        for (int l = 0; l < nl; ++l)
            if (w0 < lane_total[l])
                run_wave(l, w0, static_cast<uint32_t>(std::min<uint64_t>(wcap, lane_total[l] - w0)));
    for (int l = 1; l < nl; ++l) {   // the caller's stream continues after every lane
        cudaEventRecord(ev_join[l], main_st[l]);
        cudaStreamWaitEvent(st, ev_join[l], 0);
    }
    for (int l = 0; l < nl; ++l) {   // released once their pending records complete
        if (ev_shaded[l]) cudaEventDestroy(ev_shaded[l]);
        if (ev_shadowed[l]) cudaEventDestroy(ev_shadowed[l]);
        if (ev_join[l]) cudaEventDestroy(ev_join[l]);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("wavefront launch failed: ") + cudaGetErrorString(e);
        return OHAO_ERR_CUDA;
    }
    if (profile) {
        cudaEventRecord(t_all1, st);
        tm.collect(prof);
        float ms = 0;
        cudaEventElapsedTime(&ms, t_all0, t_all1);
        prof->total_ms += ms;
        unsigned long long hs[8];
        cudaMemcpy(hs, dstats, sizeof(hs), cudaMemcpyDeviceToHost);
        prof->rays_closest += hs[0];
        prof->nodes_closest += hs[1];
        prof->tris_closest += hs[2];
        prof->rays_shadow += hs[3];
        prof->nodes_shadow += hs[4];
        prof->tris_shadow += hs[5];
        cudaEventDestroy(t_all0);
        cudaEventDestroy(t_all1);
    }
    return OHAO_OK;
}

ohao_status trace_rays(const DScene& sc, const float* rays, uint32_t n, uint32_t* hits, int any_hit, uint32_t* stats,
                       cudaStream_t st, int* d_err, std::string& err) {
    init_launch_shapes();
    if (n == 0) return OHAO_OK;
    k_trace<<<g_blocks_trace, 128, 0, st>>>(sc, rays, n, hits, any_hit, stats, d_err);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("trace launch failed: ") + cudaGetErrorString(e);
        return OHAO_ERR_CUDA;
    }
    return OHAO_OK;
}

// ---------------------------------------------------------------------------
// Persistent multi-view pool
//
// One call renders all its views from one work queue of pixels (views
// concatenated). A pool of `cap` path slots stays full: each iteration runs
// regenerate -> extend -> shade -> shadow, where regenerate folds finished
// paths into their pixel's running mean (samples of a pixel stay in one slot,
// in sample order, so the result equals the per-view wavefront bit for bit)
// and refills idle slots from the queue. A render is one CUDA graph launch:
// a conditional while node whose body is a chunk of kChunk iterations and a
// one-thread kernel that decides on the device whether another chunk is
// needed (no host round trip). Where the driver refuses conditional nodes,
// one chunk per graph is replayed from the host, which reads four counters
// between chunks. The autotuner picks the pool shape.
// ---------------------------------------------------------------------------
namespace {
constexpr int kChunk = 8;                       // iterations per graph replay (even)
struct PoolVariant {
    uint32_t cap;
    bool reorder;
    int refill;          // persistent-warp traversal refilled at >= refill idle lanes (0: one ray per thread)
    const char* name;
};
const PoolVariant kPool[] = {
    {1u << 20, true, 0, "pool_1M_sorted_chunk8"},          {1u << 21, true, 0, "pool_2M_sorted_chunk8"},
    {1u << 22, true, 0, "pool_4M_sorted_chunk8"},          {1u << 21, false, 0, "pool_2M_unsorted_chunk8"},
    {1u << 22, false, 0, "pool_4M_unsorted_chunk8"},       {1u << 21, true, 4, "pool_2M_sorted_fetch4_chunk8"},
    {1u << 22, false, 4, "pool_4M_unsorted_fetch4_chunk8"}, {1u << 22, false, 8, "pool_4M_unsorted_fetch8_chunk8"},
};
constexpr int kNumPool = sizeof(kPool) / sizeof(kPool[0]);
constexpr int kDefaultPool = 1;
}  // namespace

struct PersistentState {
    // a chunk's shadow rays run on aux beside the next step's closest-hit rays
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_shaded = nullptr, ev_shadowed = nullptr;
    LaunchBlock* d_lb = nullptr;
    LaunchBlock* h_lb = nullptr;                // pinned staging
    uint32_t* h_counts = nullptr;               // pinned readback
    void* pool = nullptr;
    size_t pool_bytes = 0;
    uint32_t cap = 0;
    int variant = -1;
    cudaGraphExec_t graph = nullptr;
    bool graph_whole = false;                   // the graph holds the whole render (device while loop)
    DScene graph_scene{};
    PathParams graph_pp{};
    int* graph_err = nullptr;
    int graph_variant = -1;
};

PersistentState* persistent_create() {
    auto* s = new PersistentState();
    if (cudaMalloc(&s->d_lb, sizeof(LaunchBlock)) != cudaSuccess ||
        cudaMallocHost(&s->h_lb, sizeof(LaunchBlock)) != cudaSuccess ||
        cudaMallocHost(&s->h_counts, 64) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_shaded, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_shadowed, cudaEventDisableTiming) != cudaSuccess) {
        persistent_destroy(s);
        return nullptr;
    }
    return s;
}

void persistent_destroy(PersistentState* s) {
    if (!s) return;
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->pool) cudaFree(s->pool);
    if (s->d_lb) cudaFree(s->d_lb);
    if (s->h_lb) cudaFreeHost(s->h_lb);
    if (s->h_counts) cudaFreeHost(s->h_counts);
    if (s->ev_shaded) cudaEventDestroy(s->ev_shaded);
    if (s->ev_shadowed) cudaEventDestroy(s->ev_shadowed);
    if (s->aux) cudaStreamDestroy(s->aux);
    delete s;
}

uint32_t persistent_max_views() { return kMaxViews; }

const char* persistent_variant_name(const PersistentState* s) {
    return s && s->variant >= 0 ? kPool[s->variant].name : "default";
}

const char* persistent_variant_at(uint32_t i) { return i < static_cast<uint32_t>(kNumPool) ? kPool[i].name : nullptr; }

bool persistent_select(PersistentState* s, const char* name) {
    for (int v = 0; v < kNumPool; ++v) {
        if (std::strcmp(kPool[v].name, name) == 0) {
            s->variant = v;
            return true;
        }
    }
    return false;
}

namespace {

ohao_status stage_views(PersistentState* s, const RenderView* views, uint32_t n, uint32_t spp, uint32_t max_bounces,
                        const float* box, cudaStream_t st, std::string& err) {
    if (n == 0 || n > kMaxViews) {
        err = "persistent render: view count outside [1, 1024]";
        return OHAO_ERR_INVALID_ARG;
    }
    cudaStreamSynchronize(st);   // the pinned staging block may still be in flight
    LaunchBlock& lb = *s->h_lb;
    lb.nviews = n;
    lb.spp = spp;
    for (int a = 0; a < 3; ++a) {
        const float ext = box[3 + a] - box[a];
        lb.box_lo[a] = box[a];
        lb.box_scale[a] = ext > 0.0f ? 128.0f / ext : 0.0f;
    }
    uint64_t off = 0;
    for (uint32_t v = 0; v < n; ++v) {
        PView& pv = lb.views[v];
        pv.vp = views[v].vp;
        pv.accum = views[v].accum;
        pv.path_out = views[v].path_out;
        pv.aov = views[v].aov;
        pv.history = views[v].history;
        pv.pix_begin = static_cast<uint32_t>(off);
        pv.npix = views[v].vp.width * views[v].vp.height;
        off += pv.npix;
    }
    if (off >= (1ull << 31)) {
        err = "persistent render: more than 2^31 pixels in one call";
        return OHAO_ERR_INVALID_ARG;
    }
    lb.total_pix = static_cast<uint32_t>(off);
    // While the work queue is not exhausted every slot of the smallest pool
    // (2^20) advances one step per iteration, and a path takes at most
    // 1 + 2 max_bounces steps plus its regeneration: a bound on the
    // iterations, then on the chunks, taken four times over.
    {
        const uint64_t steps = 2ull + 2ull * max_bounces + 1ull;
        const uint64_t iters = (off * spp * steps + (1ull << 20) - 1) / (1ull << 20) + steps + 2;
        const uint64_t chunks = 4 * ((iters + kChunk - 1) / kChunk + 2);
        lb.max_chunks = static_cast<uint32_t>(std::min<uint64_t>(chunks, kMaxChunks));
    }
    const size_t bytes = offsetof(LaunchBlock, views) + sizeof(PView) * n;
    if (cudaMemcpyAsync(s->d_lb, s->h_lb, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        err = "persistent render: view table upload failed";
        return OHAO_ERR_CUDA;
    }
    return OHAO_OK;
}

constexpr int kCtrNewBegin = 8;   // Soa::counts: queue index of the first camera ray regenerated this step

// One chunk of pool steps. With persistent-warp traversal and no ray
// reordering, and an auxiliary stream, each step's shadow rays run on aux
// beside the next step's closest-hit rays of the paths that continue; after
// the join, regeneration appends new camera rays to the queue and a second
// extend claims just those (its fetch counter starts at their first index),
// so a regenerated path still traces in the step it was started. Otherwise
// the steps run serially: regeneration, extend, shading, shadow rays.
void enqueue_chunk(const DScene& sc, const PathParams& pp, const LaunchBlock* lb, const Soa& s, uint32_t cap,
                   const PoolVariant& pv, int* d_err, cudaStream_t st, cudaStream_t aux, cudaEvent_t ev_shaded,
                   cudaEvent_t ev_shadowed) {
    const bool fetch = pv.refill > 0 && sc.nnodes > 0;
    if (aux && fetch && !pv.reorder) {
        for (int it = 0; it < kChunk; ++it) {
            const int cur = it & 1;
            cudaMemsetAsync(s.counts + kCtrExtendFetch, 0, 4, st);
            launch_extend_fetch(sc, s, cur, pv.refill, d_err, nullptr, st);    // continuing rays
            if (it > 0) cudaStreamWaitEvent(st, ev_shadowed, 0);                // the last step's shadow rays
            cudaMemcpyAsync(s.counts + kCtrNewBegin, s.counts + cur, 4, cudaMemcpyDeviceToDevice, st);
            k_regen<<<g_blocks_shade, 128, 0, st>>>(pp, lb, s, cur);
            cudaMemcpyAsync(s.counts + kCtrExtendFetch, s.counts + kCtrNewBegin, 4, cudaMemcpyDeviceToDevice, st);
            launch_extend_fetch(sc, s, cur, pv.refill, d_err, nullptr, st);    // the new camera rays
            if (pp.flags & kFlagSortMaterial) bin_queue<0>(sc, s, cur, cap, st);
            cudaMemsetAsync(s.counts + (cur ^ 1), 0, 4, st);
            cudaMemsetAsync(s.counts + 2, 0, 8, st);   // shadow and done counts
            launch_shade<true, 0>(sc, pp, ViewParams{}, 0u, 1u, s, cur, nullptr, 0u, lb, st);
            cudaEventRecord(ev_shaded, st);
            cudaStreamWaitEvent(aux, ev_shaded, 0);
            cudaMemsetAsync(s.counts + kCtrShadowFetch, 0, 4, aux);
            launch_shadow_fetch(sc, s, pv.refill, d_err, nullptr, aux);
            cudaEventRecord(ev_shadowed, aux);
        }
        cudaStreamWaitEvent(st, ev_shadowed, 0);   // the chunk ends with its shadow rays done
        return;
    }
    for (int it = 0; it < kChunk; ++it) {
        const int cur = it & 1;
        k_regen<<<g_blocks_shade, 128, 0, st>>>(pp, lb, s, cur);
        if (pv.reorder) {
            k_ray_keys<<<g_blocks_shade, 128, 0, st>>>(lb, s, cur);
            rsort::sort_pairs(s.skA, s.svA, s.skB, s.svB, s.shist, s.counts + cur, cap, 24, st);
            k_copy_queue<<<g_blocks_shade, 128, 0, st>>>(s, cur);
        }
        if (fetch) {
            cudaMemsetAsync(s.counts + kCtrExtendFetch, 0, 8, st);   // both fetch counters
            launch_extend_fetch(sc, s, cur, pv.refill, d_err, nullptr, st);
        } else {
            launch_extend(sc, s, cur, d_err, nullptr, st);
        }
        if (pp.flags & kFlagSortMaterial) bin_queue<0>(sc, s, cur, cap, st);
        cudaMemsetAsync(s.counts + (cur ^ 1), 0, 4, st);
        cudaMemsetAsync(s.counts + 2, 0, 8, st);   // shadow and done counts
        launch_shade<true, 0>(sc, pp, ViewParams{}, 0u, 1u, s, cur, nullptr, 0u, lb, st);
        if (fetch) {
            launch_shadow_fetch(sc, s, pv.refill, d_err, nullptr, st);
        } else {
            launch_shadow(sc, s, d_err, nullptr, st);
        }
    }
}

ohao_status run_pool(PersistentState* s, int variant, const DScene& sc, const PathParams& pp, cudaStream_t st,
                     int* d_err, bool use_graph, std::string& err) {
    init_launch_shapes();
    const uint32_t cap = kPool[variant].cap;
    const size_t need = wavefront_scratch_bytes(cap);
    if (s->pool_bytes < need) {
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
        if (s->pool) cudaFree(s->pool);
        s->pool = nullptr;
        s->pool_bytes = 0;
        if (cudaMalloc(&s->pool, need) != cudaSuccess) {
            err = "persistent render: pool allocation failed";
            return OHAO_ERR_OOM;
        }
        s->pool_bytes = need;
    }
    const Soa soa = carve_soa(s->pool, cap);
    k_pool_init<<<g_blocks_shade, 128, 0, st>>>(soa, cap);
    if (use_graph) {
        const bool stale = !s->graph || s->graph_variant != variant || s->graph_err != d_err ||
                           std::memcmp(&s->graph_scene, &sc, sizeof(DScene)) != 0 ||
                           std::memcmp(&s->graph_pp, &pp, sizeof(PathParams)) != 0;
        if (stale) {
            if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
            cudaStream_t cap_st;
            if (cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking) != cudaSuccess) {
                err = "persistent: capture stream";
                return OHAO_ERR_CUDA;
            }
            // The whole render as one graph: a conditional while node whose
            // body is one chunk followed by k_pool_continue.
            s->graph_whole = false;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaGraphCreate(&g, 0);
            cudaGraphConditionalHandle loop{};
            if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&loop, g, 1u, cudaGraphCondAssignDefault);
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = loop;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node = nullptr;
            if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
            if (e == cudaSuccess) {
                cudaGraph_t body = cp.conditional.phGraph_out[0];
                e = cudaStreamBeginCaptureToGraph(cap_st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    enqueue_chunk(sc, pp, s->d_lb, soa, cap, kPool[variant], d_err, cap_st, s->aux, s->ev_shaded,
                                  s->ev_shadowed);
                    k_pool_continue<<<1, 1, 0, cap_st>>>(loop, s->d_lb, soa, d_err);
                    cudaGraph_t captured = nullptr;
                    e = cudaStreamEndCapture(cap_st, &captured);
                }
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&s->graph, g, 0);
            if (e == cudaSuccess) {
                s->graph_whole = true;
            } else {
                // fall back to one chunk per graph, replayed from the host
                cudaGetLastError();
                s->graph = nullptr;
                if (g) { cudaGraphDestroy(g); g = nullptr; }
                cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal);
                enqueue_chunk(sc, pp, s->d_lb, soa, cap, kPool[variant], d_err, cap_st, s->aux, s->ev_shaded,
                              s->ev_shadowed);
                e = cudaStreamEndCapture(cap_st, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&s->graph, g, 0);
            }
            if (g) cudaGraphDestroy(g);
            cudaStreamDestroy(cap_st);
            if (e != cudaSuccess) {
                s->graph = nullptr;
                err = std::string("persistent graph: ") + cudaGetErrorString(e);
                return OHAO_ERR_CUDA;
            }
            s->graph_variant = variant;
            s->graph_err = d_err;
            s->graph_scene = sc;
            s->graph_pp = pp;
        }
        if (s->graph_whole) {   // one launch renders every view; completion is stream-ordered
            const cudaError_t e = cudaGraphLaunch(s->graph, st);
            if (e != cudaSuccess) { err = std::string("persistent graph launch: ") + cudaGetErrorString(e); return OHAO_ERR_CUDA; }
            return OHAO_OK;
        }
    }
    for (uint64_t chunk = 0;; ++chunk) {
        if (chunk >= s->h_lb->max_chunks) {
            err = "persistent render: work queue did not drain within the iteration bound";
            return OHAO_ERR_TIMEOUT;
        }
        if (use_graph) {
            const cudaError_t e = cudaGraphLaunch(s->graph, st);
            if (e != cudaSuccess) { err = std::string("persistent graph launch: ") + cudaGetErrorString(e); return OHAO_ERR_CUDA; }
        } else {
            enqueue_chunk(sc, pp, s->d_lb, soa, cap, kPool[variant], d_err, st, s->aux, s->ev_shaded, s->ev_shadowed);
        }
        cudaMemcpyAsync(s->h_counts, soa.counts, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { err = std::string("persistent render: ") + cudaGetErrorString(e); return OHAO_ERR_CUDA; }
        const uint32_t pending = s->h_counts[0], done = s->h_counts[3], claimed = s->h_counts[4];
        if (pending == 0 && done == 0 && claimed >= s->h_lb->total_pix) break;
    }
    return OHAO_OK;
}

}  // namespace

ohao_status persistent_render(PersistentState* s, const DScene& sc, const RenderView* views, uint32_t n,
                              const PathParams& pp, uint32_t spp, const float* scene_box, cudaStream_t st, int* d_err,
                              bool profile, ProfileAcc* prof, std::string& err) {
    ohao_status r = stage_views(s, views, n, spp, pp.max_bounces, scene_box, st, err);
    if (r != OHAO_OK) return r;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profile) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
    }
    r = run_pool(s, s->variant >= 0 ? s->variant : kDefaultPool, sc, pp, st, d_err, true, err);
    if (profile && prof) {
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        prof->other_ms += ms;
        prof->total_ms += ms;
        prof->other_launches += 1;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return r;
}

ohao_status persistent_autotune(PersistentState* s, const DScene& sc, const RenderView* views, uint32_t n,
                                const PathParams& pp, uint32_t spp, const float* scene_box, cudaStream_t st, int* d_err,
                                float* best_ms, std::string& err) {
    ohao_status r = stage_views(s, views, n, spp, pp.max_bounces, scene_box, st, err);
    if (r != OHAO_OK) return r;
    float best = 1e30f;
    int bi = kDefaultPool;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int v = 0; v < kNumPool; ++v) {
        cudaEventRecord(e0, st);
        r = run_pool(s, v, sc, pp, st, d_err, false, err);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        if (r != OHAO_OK) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; bi = v; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r != OHAO_OK) return r;
    s->variant = bi;
    if (best_ms) *best_ms = best;
    return OHAO_OK;
}

}  // namespace ohao
