// wavefront.cu -- wavefront path integrator and the batch trace call.
//
// One wave holds up to `capacity` paths, numbered sample-major
// (slot = k*npix + pixel - wave_begin), in structure-of-arrays state. Each of
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

#include <algorithm>
#include <vector>

namespace ohao {

namespace {

struct Soa {
    uint32_t* rng;
    uint32_t* dim;
    uint32_t* flags;     // phase | bounce<<2 | delta<<10 | shL<<11 | shE<<12
    float4* ro;          // origin
    float4* rd;          // dir, w = last pdf
    float4* thr;
    float4* rad;
    float4* fhP;
    float4* fhN;
    float4* fhA;
    float4* hit;         // t, u, v, prim bits
    uint32_t* hit_inst;
    float4* sh_org;
    float4* shL;         // dir, tmax
    float4* shLc;        // contribution
    float4* shE;
    float4* shEc;
    uint32_t* q_ray[2];
    uint32_t* q_sh;
    uint32_t* counts;    // [0],[1] ray queue counts, [2] shadow count
};

constexpr uint32_t kFlagDelta = 1u << 10, kFlagShL = 1u << 11, kFlagShE = 1u << 12;

__device__ __forceinline__ float4 f4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

__device__ __forceinline__ void store_state(const Soa& s, uint32_t p, const PathState& ps, uint32_t extra_flags) {
    s.rng[p] = ps.rng;
    s.dim[p] = ps.dim;
    s.flags[p] = ps.phase | (ps.bounce << 2) | (ps.delta ? kFlagDelta : 0u) | extra_flags;
    s.ro[p] = f4(ps.ro, 0.0f);
    s.rd[p] = f4(ps.rd, ps.last_pdf);
    s.thr[p] = f4(ps.thr, 0.0f);
    s.rad[p] = f4(ps.rad, 0.0f);
    s.fhP[p] = f4(ps.fhP, 0.0f);
    s.fhN[p] = f4(ps.fhN, 0.0f);
    s.fhA[p] = f4(ps.fhAlb, 0.0f);
}
__device__ __forceinline__ void load_state(const Soa& s, uint32_t p, PathState& ps) {
    ps.rng = s.rng[p];
    ps.dim = s.dim[p];
    const uint32_t f = s.flags[p];
    ps.phase = f & 3u;
    ps.bounce = (f >> 2) & 0xFFu;
    ps.delta = (f & kFlagDelta) != 0u;
    const float4 ro = s.ro[p], rd = s.rd[p];
    ps.ro = ld3(ro);
    ps.rd = ld3(rd);
    ps.last_pdf = rd.w;
    ps.thr = ld3(s.thr[p]);
    ps.rad = ld3(s.rad[p]);
    ps.fhP = ld3(s.fhP[p]);
    ps.fhN = ld3(s.fhN[p]);
    ps.fhAlb = ld3(s.fhA[p]);
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
    const uint32_t k = lin / npix, p = lin - k * npix;
    const uint32_t px = p % vp.width, py = p / vp.width;
    PathState ps;
    path_start(vp, pp, px, py, pp.sample_base + k, ps);
    store_state(s, i, ps, 0u);
    s.q_ray[0][i] = i;
}

// stats (profiling only): [0] rays, [1] nodes, [2] triangles
template <bool kStats>
__global__ void __launch_bounds__(128) k_extend(DScene sc, Soa s, int cur, int* err, unsigned long long* stats) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const float4 ro = s.ro[p], rd = s.rd[p];
        const Hit h = scene_closest<kStats>(sc, ld3(ro), ld3(rd), 0.001f, 10000.0f, tc, e);
        s.hit[p] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        s.hit_inst[p] = h.inst;
        nr++;
    }
    if (e) atomicOr(err, 1);
    if (kStats && nr) {
        atomicAdd(stats + 0, static_cast<unsigned long long>(nr));
        atomicAdd(stats + 1, static_cast<unsigned long long>(tc.nodes));
        atomicAdd(stats + 2, static_cast<unsigned long long>(tc.tris));
    }
}

__global__ void __launch_bounds__(128) k_shade(DScene sc, PathParams pp, ViewParams vp, uint32_t w0, uint32_t npix,
                                               Soa s, int cur, float* aov, uint32_t aov_k) {
    const uint32_t count = s.counts[cur];
    const uint32_t* q = s.q_ray[cur];
    uint32_t* qn = s.q_ray[cur ^ 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const uint32_t lin = w0 + p;
        const uint32_t k = lin / npix, pix = lin - k * npix;
        const uint32_t px = pix % vp.width, py = pix / vp.width;
        PathState ps;
        load_state(s, p, ps);
        const float4 hv = s.hit[p];
        Hit h;
        h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_uint(hv.w); h.inst = s.hit_inst[p];
        const bool primary = ps.phase == kPhasePrimary;
        ShadowReq qL, qE;
        AovOut ao;
        const bool want_aov = aov != nullptr && primary && k == aov_k;
        const bool more = path_step(sc, pp, vp, px, py, pp.sample_base + k, ps, h, qL, qE, want_aov ? &ao : nullptr);
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
        store_state(s, p, ps, extra);
        if (want_aov) {
            float* a = aov + static_cast<size_t>(pix) * 8;
            a[0] = ao.albedo.x; a[1] = ao.albedo.y; a[2] = ao.albedo.z;
            a[3] = ao.normal.x; a[4] = ao.normal.y; a[5] = ao.normal.z;
            a[6] = ao.depth; a[7] = ao.hit;
        }
        const uint32_t slot = warp_push(s.counts + (cur ^ 1), more);
        if (slot != 0xFFFFFFFFu) qn[slot] = p;
        const uint32_t sslot = warp_push(s.counts + 2, extra != 0u);
        if (sslot != 0xFFFFFFFFu) s.q_sh[sslot] = p;
    }
}

// stats (profiling only): [3] shadow rays, [4] nodes, [5] triangles
template <bool kStats>
__global__ void __launch_bounds__(128) k_shadow(DScene sc, Soa s, int* err, unsigned long long* stats) {
    const uint32_t count = s.counts[2];
    int e = 0;
    TravCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = s.q_sh[i];
        const uint32_t f = s.flags[p];
        const V3 org = ld3(s.sh_org[p]);
        V3 rad = ld3(s.rad[p]);
        if (f & kFlagShL) {
            const float4 d = s.shL[p];
            nr++;
            if (!scene_occluded<kStats>(sc, org, ld3(d), 0.001f, d.w, tc, e)) rad = rad + ld3(s.shLc[p]);
        }
        if (f & kFlagShE) {
            const float4 d = s.shE[p];
            nr++;
            if (!scene_occluded<kStats>(sc, org, ld3(d), 0.001f, d.w, tc, e)) rad = rad + ld3(s.shEc[p]);
        }
        s.rad[p] = f4(rad, 0.0f);
        s.flags[p] = f & ~(kFlagShL | kFlagShE);
    }
    if (e) atomicOr(err, 1);
    if (kStats && nr) {
        atomicAdd(stats + 3, static_cast<unsigned long long>(nr));
        atomicAdd(stats + 4, static_cast<unsigned long long>(tc.nodes));
        atomicAdd(stats + 5, static_cast<unsigned long long>(tc.tris));
    }
}

__global__ void k_finalize(PathParams pp, uint32_t w0, uint32_t n, uint32_t npix, Soa s, float* accum,
                           uint32_t history, float* path_out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const uint64_t lo = w0, hi = static_cast<uint64_t>(w0) + n;   // [lo, hi)
        uint64_t k0 = (lo > p) ? (lo - p + npix - 1) / npix : 0;
        if (k0 * npix + p >= hi) continue;
        const uint64_t k1 = (hi - 1 - p) / npix;
        float4 acc = reinterpret_cast<float4*>(accum)[p];
        for (uint64_t k = k0; k <= k1; ++k) {
            const uint32_t slot = static_cast<uint32_t>(k * npix + p - lo);
            const V3 L = firefly(pp, ld3(s.rad[slot]));
            if (path_out) reinterpret_cast<float4*>(path_out)[k * npix + p] = f4(L, 0.0f);
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
        reinterpret_cast<float4*>(accum)[p] = acc;
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
            const bool occ = stats ? scene_occluded<true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e)
                                   : scene_occluded<false>(sc, ld3(a), ld3(b), a.w, b.w, tc, e);
            h[0] = occ ? 1u : 0u; h[1] = 0u; h[2] = 0u; h[3] = 0xFFFFFFFFu; h[4] = 0xFFFFFFFFu;
        } else {
            const Hit r = stats ? scene_closest<true>(sc, ld3(a), ld3(b), a.w, b.w, tc, e)
                                : scene_closest<false>(sc, ld3(a), ld3(b), a.w, b.w, tc, e);
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
    s.rng = c.take<uint32_t>(cap);
    s.dim = c.take<uint32_t>(cap);
    s.flags = c.take<uint32_t>(cap);
    s.ro = c.take<float4>(cap);
    s.rd = c.take<float4>(cap);
    s.thr = c.take<float4>(cap);
    s.rad = c.take<float4>(cap);
    s.fhP = c.take<float4>(cap);
    s.fhN = c.take<float4>(cap);
    s.fhA = c.take<float4>(cap);
    s.hit = c.take<float4>(cap);
    s.hit_inst = c.take<uint32_t>(cap);
    s.sh_org = c.take<float4>(cap);
    s.shL = c.take<float4>(cap);
    s.shLc = c.take<float4>(cap);
    s.shE = c.take<float4>(cap);
    s.shEc = c.take<float4>(cap);
    s.q_ray[0] = c.take<uint32_t>(cap);
    s.q_ray[1] = c.take<uint32_t>(cap);
    s.q_sh = c.take<uint32_t>(cap);
    s.counts = c.take<uint32_t>(64);
    return s;
}

Soa carve_soa(void* base, uint32_t cap) {
    Carve c{static_cast<char*>(base)};
    return carve_soa_at(c, cap);
}

int g_num_sms = 0;
int g_blocks_extend = 0, g_blocks_shade = 0, g_blocks_shadow = 0, g_blocks_trace = 0;

void init_launch_shapes() {
    if (g_num_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_extend<false>, 128, 0);
    g_blocks_extend = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade, 128, 0);
    g_blocks_shade = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shadow<false>, 128, 0);
    g_blocks_shadow = std::max(1, b) * g_num_sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace, 128, 0);
    g_blocks_trace = std::max(1, b) * g_num_sms;
}

struct EvTimer {
    bool on;
    cudaStream_t st;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[4];
    void begin(int kind, cudaEvent_t& a) {
        if (!on) return;
        cudaEventCreate(&a);
        cudaEventRecord(a, st);
        (void)kind;
    }
    void end(int kind, cudaEvent_t a) {
        if (!on) return;
        cudaEvent_t b;
        cudaEventCreate(&b);
        cudaEventRecord(b, st);
        ev[kind].push_back({a, b});
    }
    void collect(ProfileAcc* p) {
        if (!on || !p) return;
        cudaStreamSynchronize(st);
        for (int k = 0; k < 4; ++k) {
            for (auto& e : ev[k]) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e.first, e.second);
                if (k == 0) { p->extend_ms += ms; p->extend_launches++; }
                if (k == 1) { p->shade_ms += ms; p->shade_launches++; }
                if (k == 2) { p->shadow_ms += ms; p->shadow_launches++; }
                if (k == 3) { p->other_ms += ms; p->other_launches++; }
                cudaEventDestroy(e.first);
                cudaEventDestroy(e.second);
            }
            ev[k].clear();
        }
    }
};

}  // namespace

void upload_sobol_table(const uint32_t* dirs128) { cudaMemcpyToSymbol(c_sobol_dirs, dirs128, 128 * sizeof(uint32_t)); }

size_t wavefront_scratch_bytes(uint32_t cap) {
    Carve c{nullptr};
    carve_soa_at(c, cap);
    return c.off;
}

uint32_t wavefront_default_capacity() { return 1u << 21; }

ohao_status wavefront_render(const DScene& sc, const RenderView& view, const PathParams& pp, uint32_t spp,
                             void* scratch, size_t scratch_bytes, uint32_t capacity, cudaStream_t st, bool profile,
                             ProfileAcc* prof, int* d_err, std::string& err) {
    init_launch_shapes();
    if (scratch_bytes < wavefront_scratch_bytes(capacity)) {
        err = "wavefront scratch too small";
        return OHAO_ERR_INVALID_ARG;
    }
    const uint32_t npix = view.vp.width * view.vp.height;
    const uint64_t total = static_cast<uint64_t>(npix) * spp;
    Soa s = carve_soa(scratch, capacity);
    unsigned long long* dstats = reinterpret_cast<unsigned long long*>(s.counts + 16);
    if (profile) cudaMemsetAsync(dstats, 0, 8 * sizeof(unsigned long long), st);
    const uint32_t niters = 1 + 2 * pp.max_bounces;
    EvTimer tm{profile, st, {}};
    cudaEvent_t t_all0 = nullptr, t_all1 = nullptr;
    if (profile) {
        cudaEventCreate(&t_all0);
        cudaEventCreate(&t_all1);
        cudaEventRecord(t_all0, st);
    }
    for (uint64_t w0 = 0; w0 < total; w0 += capacity) {
        const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(capacity, total - w0));
        cudaEvent_t a;
        tm.begin(3, a);
        k_generate<<<(n + 255) / 256, 256, 0, st>>>(view.vp, pp, static_cast<uint32_t>(w0), n, npix, s);
        tm.end(3, a);
        int cur = 0;
        for (uint32_t it = 0; it < niters; ++it) {
            tm.begin(0, a);
            if (profile) k_extend<true><<<g_blocks_extend, 128, 0, st>>>(sc, s, cur, d_err, dstats);
            else k_extend<false><<<g_blocks_extend, 128, 0, st>>>(sc, s, cur, d_err, nullptr);
            tm.end(0, a);
            cudaMemsetAsync(s.counts + (cur ^ 1), 0, 4, st);
            cudaMemsetAsync(s.counts + 2, 0, 4, st);
            tm.begin(1, a);
            k_shade<<<g_blocks_shade, 128, 0, st>>>(sc, pp, view.vp, static_cast<uint32_t>(w0), npix, s, cur, view.aov,
                                                    spp - 1);
            tm.end(1, a);
            tm.begin(2, a);
            if (profile) k_shadow<true><<<g_blocks_shadow, 128, 0, st>>>(sc, s, d_err, dstats);
            else k_shadow<false><<<g_blocks_shadow, 128, 0, st>>>(sc, s, d_err, nullptr);
            tm.end(2, a);
            cur ^= 1;
        }
        tm.begin(3, a);
        k_finalize<<<std::max(1u, std::min(4096u, (npix + 255) / 256)), 256, 0, st>>>(
            pp, static_cast<uint32_t>(w0), n, npix, s, view.accum, view.history, view.path_out);
        tm.end(3, a);
    }
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

}  // namespace ohao
