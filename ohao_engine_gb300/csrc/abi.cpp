// abi.cpp -- host side of the C ABI (C++20): scene storage, acceleration
// structure builds and render orchestration around the CUDA kernels.
//
// Mirrors the reference's host objects: the input setters of PathTracer
// (ohao/render/rt/path_tracer.hpp:124-194), RTAccelerationStructure's
// createBLAS / addInstance / buildTLAS (rt_acceleration_structure.hpp:73-107),
// updateRTMaterialParams (ohao/gpu/vulkan/rt_build.cpp:313-389) and
// EnvCDF::build (ohao/render/rt/env_cdf.cpp:13-61). Errors are status codes
// plus a per-context message, never exceptions (the reference's
// [[nodiscard]] bool + std::cerr convention, path_tracer.cpp:92-120).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ohao_pt.h"
#include "bvh_internal.hpp"
#include "env_guide.hpp"
#include "pt_types.hpp"

namespace {

using namespace ohao;

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= n && p) return cudaSuccess;
        release();
        if (bytes == 0) bytes = 256;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) { p = nullptr; return e; }
        n = bytes;
        return cudaSuccess;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct BvhDev {
    DevBuf nodes, prims;   // prims: tri records (48 B) or TLAS instance ids
    uint32_t nnodes = 0, nprims = 0, height = 0;
    float root_box[6] = {0, 0, 0, 0, 0, 0};
};

struct BlasDesc {
    uint32_t first_index, index_count;
    uint32_t flags = 0;        // OHAO_BLAS_FLAG_*
};

}  // namespace

struct ohao_pt_ctx {
    int device = 0;
    uint64_t flatten_limit = 1ull << 25;
    std::string last_error;
    // geometry
    DevBuf pos, normals, uvs, indices, mat_ids, mats, lights, env, marg, cond, albedo_map;
    DevBuf guide_marg, guide_cond;   // env_guide.hpp tables; has_guide when both are current
    bool has_guide = false;
    uint32_t guide_mm = 0, guide_mc = 0;
    uint32_t nverts = 0, ntris = 0, nmats = 0, nlights = 0;
    uint32_t max_mat_id = 0;              // largest per-triangle material id
    uint32_t env_w = 0, env_h = 0;
    bool has_env = false, has_cdf = false;
    float env_intensity = 1.0f;
    uint32_t map_w = 0, map_h = 0;
    // bindless textures: RGBA8 texels of every texture back to back, and per
    // texture (first texel, width, height, 0)
    DevBuf tex_texels, tex_info;
    uint32_t ntex = 0;
    // material texture indices the renders need, from the host copy of the
    // table, summarised when the table changes: the largest bindless index
    // other than diffuse 0 (or -1), whether diffuse index 0 occurs
    std::vector<float> mats_host;
    int64_t mat_max_tex = -1;
    bool mat_uses_diffuse0 = false;
    // acceleration structure
    std::vector<BlasDesc> blas;
    std::vector<ohao_pt_instance> instances;
    bool built = false, two_level = false;
    BvhDev flat;                          // flat BVH or TLAS
    std::vector<BvhDev> blas_bvh;
    DevBuf blas_nodes_all, blas_tris_all, blas_desc, inst_dev;
    // scratch
    DevBuf scratch, build_scratch, err_flag;
    DevBuf adj_scratch, adj_grads;        // backward: view table, loss cell; per-pixel loss gradients
    std::vector<DevBuf*> host_accum_bufs, host_display_bufs, host_target_bufs;
    DevBuf host_grad_bufs[2];             // ohao_pt_adjoint_host: map and roughness gradients
    ohao_pt_profile profile{};
    // emitter MIS: the emissive-triangle table (pt_types.hpp DScene::emis_*),
    // built by the first render with OHAO_PT_FLAG_EMITTER_MIS after a build
    // or a change of the materials' emission
    DevBuf emis_tri, emis_cdf, emis_rank, emis_inst;
    uint32_t nemis = 0;
    bool emis_dirty = true;
    ohao::PersistentState* persistent = nullptr;
    // ohao_pt_render_host: history uploads run on their own stream, so that
    // they overlap the render up to its first read of the accumulator
    cudaStream_t upload_stream = nullptr;
    // per-view wavefront (created on first use): the streams of the pixel
    // lanes after the first, and each lane's stream for its shadow rays
    ohao::WaveStreams wave{};
    std::vector<cudaEvent_t> upload_after, upload_done;   // per view: stream order in, upload landed
    ~ohao_pt_ctx() {
        if (persistent) ohao::persistent_destroy(persistent);
        for (cudaEvent_t e : upload_after) cudaEventDestroy(e);
        for (cudaEvent_t e : upload_done) cudaEventDestroy(e);
        if (upload_stream) cudaStreamDestroy(upload_stream);
        for (int l = 0; l < ohao::kWaveLanes; ++l) {
            if (wave.main[l]) cudaStreamDestroy(wave.main[l]);
            if (wave.aux[l]) cudaStreamDestroy(wave.aux[l]);
        }
        for (auto* b : host_accum_bufs) delete b;
        for (auto* b : host_display_bufs) delete b;
        for (auto* b : host_target_bufs) delete b;
    }
};

namespace ohao {
// aov.cu: mean first-hit features over nsamp camera samples per pixel
cudaError_t launch_aov_mean(const DScene& sc, const PathParams& pp, const ViewParams& vp, uint32_t nsamp, float* out,
                            int* err, cudaStream_t st);
}  // namespace ohao

namespace {

ohao_status fail(ohao_pt_ctx* c, ohao_status s, const std::string& msg) {
    if (c) c->last_error = msg;
    return s;
}

ohao_status cuda_fail(ohao_pt_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? OHAO_ERR_OOM : OHAO_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr, what)                                       \
    do {                                                     \
        cudaError_t e_ = (expr);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

ohao_status upload(ohao_pt_ctx* ctx, DevBuf& b, const void* src, size_t bytes, const char* what) {
    CK(b.ensure(bytes), what);
    if (bytes) CK(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice), what);
    return OHAO_OK;
}

// True when the row-major 3x4 transform is finite and its 3x3 part has a
// non-zero, finite determinant (computed in double, as instance_matrices does).
bool instance_invertible(const float x[12]) {
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(x[k])) return false;
    const double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
    const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    return det != 0.0 && std::isfinite(det);
}

void instance_matrices(const float x[12], float w2o[12], float nrm[9]) {
    const double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    const double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    const double det = a * A + b * B + c * C;
    const double inv[9] = {A / det, D / det, G / det, B / det, E / det, H / det, C / det, F / det, I / det};
    const double t[3] = {x[3], x[7], x[11]};
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) w2o[r * 4 + k] = static_cast<float>(inv[r * 3 + k]);
        w2o[r * 4 + 3] = static_cast<float>(-(inv[r * 3 + 0] * t[0] + inv[r * 3 + 1] * t[1] + inv[r * 3 + 2] * t[2]));
    }
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) nrm[r * 3 + k] = static_cast<float>(inv[k * 3 + r]);
}


ohao_status build_one(ohao_pt_ctx* ctx, const float* d_boxes, uint32_t n, BvhDev& out, cudaStream_t st) {
    std::string err;
    const size_t need = ohao::bvh_build_scratch_bytes(n);
    CK(ctx->build_scratch.ensure(need), "BVH scratch");
    CK(out.nodes.ensure(static_cast<size_t>(std::max(n, 1u)) * 80), "BVH nodes");
    DevBuf order_tmp;
    CK(order_tmp.ensure(static_cast<size_t>(std::max(n, 1u)) * 4), "BVH order");
    DevBuf rb;
    CK(rb.ensure(32), "BVH root box");
    ohao::BvhBuildInfo info{};
    const ohao_status s = ohao::bvh_build(d_boxes, n, ctx->build_scratch.p, ctx->build_scratch.n, out.nodes.as<uint4>(),
                                          order_tmp.as<uint32_t>(), rb.as<float>(), &info, st, err);
    if (s != OHAO_OK) return fail(ctx, s, err);
    out.nnodes = info.nnodes;
    out.height = info.height;
    out.nprims = n;
    if (n) CK(cudaMemcpy(out.root_box, rb.p, 24, cudaMemcpyDeviceToHost), "BVH root box");
    // keep the order in prims temporarily (caller gathers records)
    std::swap(out.prims.p, order_tmp.p);
    std::swap(out.prims.n, order_tmp.n);
    return OHAO_OK;
}

constexpr uint32_t kStackEntries = 64;   // the traversal stack of every ray (pt_traverse.cuh kStackSize)

// The per-ray stack limit of a render: settings.trace_stack_limit in
// [1, 64], 0 = all 64.
uint32_t stack_limit_of(const ohao_pt_settings* st) {
    return (st->trace_stack_limit == 0u || st->trace_stack_limit > kStackEntries) ? kStackEntries
                                                                                  : st->trace_stack_limit;
}

ohao::DScene make_scene(const ohao_pt_ctx* c) {
    ohao::DScene s{};
    s.nodes = c->flat.nodes.as<uint4>();
    s.nnodes = c->flat.nnodes;
    s.two_level = c->two_level ? 1 : 0;
    if (c->two_level) {
        s.tris = nullptr;
        s.tlas_inst = c->flat.prims.as<uint32_t>();
    } else {
        s.tris = c->flat.prims.as<float4>();
        s.tlas_inst = nullptr;
    }
    s.blas = c->blas_desc.as<ohao::DBlas>();
    s.blas_nodes = c->blas_nodes_all.as<uint4>();
    s.blas_tris = c->blas_tris_all.as<float4>();
    s.inst = c->inst_dev.as<ohao::DInst>();
    s.indices = c->indices.as<uint32_t>();
    s.normals = c->normals.as<float4>();
    s.uvs = c->uvs.as<float2>();
    s.mat_ids = c->mat_ids.as<uint32_t>();
    s.mats = c->mats.as<float4>();
    s.lights = c->lights.as<float4>();
    s.nlights = c->nlights;
    s.env = c->env.as<float4>();
    s.env_w = c->env_w;
    s.env_h = c->env_h;
    s.marg = c->marg.as<float>();
    s.cond = c->cond.as<float>();
    s.guide_marg = c->has_guide ? c->guide_marg.as<uint16_t>() : nullptr;
    s.guide_cond = c->has_guide ? c->guide_cond.as<uint16_t>() : nullptr;
    s.guide_mm = c->guide_mm;
    s.guide_mc = c->guide_mc;
    s.env_intensity = c->env_intensity;
    s.has_env = c->has_env ? 1 : 0;
    s.has_cdf = c->has_cdf ? 1 : 0;
    s.albedo_map = c->albedo_map.as<float>();
    s.map_w = c->map_w;
    s.map_h = c->map_h;
    s.stack_limit = kStackEntries;
    s.tex = c->tex_texels.as<uchar4>();
    s.tex_info = c->tex_info.as<uint4>();
    s.ntex = c->ntex;
    s.alpha_test = 0;
    for (int a = 0; a < 3; ++a) {
        const float ext = c->flat.root_box[3 + a] - c->flat.root_box[a];
        s.box_lo[a] = c->flat.root_box[a];
        s.box_inv[a] = ext > 0.0f ? 4.0f / ext : 0.0f;
    }
    return s;
}

ohao_status check_device_error(ohao_pt_ctx* ctx, cudaStream_t st) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, ctx->err_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st), "error flag");
    CK(cudaStreamSynchronize(st), "stream sync");
    if (flag) {
        cudaMemsetAsync(ctx->err_flag.p, 0, sizeof(int), st);
        if (flag & 4)   // the persistent pool's device loop gave up
            return fail(ctx, OHAO_ERR_TIMEOUT, "persistent render: the work queue did not drain within the chunk bound");
        return fail(ctx, OHAO_ERR_DEVICE_CHECK, "traversal stack limit exceeded on the device");
    }
    return OHAO_OK;
}

}  // namespace

extern "C" {

const char* ohao_pt_version(void) { return "ohao-gb300-pt 0.1 (sm_103a)"; }

ohao_status ohao_pt_create(const ohao_pt_desc* desc, ohao_pt_ctx** out) {
    if (!out) return OHAO_ERR_INVALID_ARG;
    *out = nullptr;
    auto* ctx = new (std::nothrow) ohao_pt_ctx();
    if (!ctx) return OHAO_ERR_OOM;
    if (desc) {
        ctx->device = desc->device;
        if (desc->flatten_limit) ctx->flatten_limit = desc->flatten_limit;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        delete ctx;
        return OHAO_ERR_CUDA;
    }
    e = ctx->err_flag.ensure(256);
    if (e == cudaSuccess) e = cudaMemset(ctx->err_flag.p, 0, 256);
    if (e != cudaSuccess) {
        delete ctx;
        return OHAO_ERR_CUDA;
    }
    *out = ctx;
    return OHAO_OK;
}

void ohao_pt_destroy(ohao_pt_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    delete ctx;
}

const char* ohao_pt_last_error(const ohao_pt_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

ohao_status ohao_pt_set_geometry(ohao_pt_ctx* ctx, const float* pos, uint32_t pos_stride_bytes, uint32_t nverts,
                                 const float* normal4, const float* uv2, const uint32_t* indices, uint32_t ntris,
                                 const uint32_t* mat_ids) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    if ((nverts && (!pos || !normal4)) || (ntris && (!indices || !mat_ids)) || pos_stride_bytes < 12)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "set_geometry: null array or stride < 12");
    for (size_t i = 0; i < static_cast<size_t>(ntris) * 3; ++i)
        if (indices[i] >= nverts) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_geometry: index out of range");
    // a failed upload below leaves buffers reallocated or released: nothing
    // renders from them until the next successful set_geometry + build
    ctx->built = false;
    ctx->nverts = ctx->ntris = 0;
    // positions are stored packed (12 B per vertex) whatever the caller's stride
    std::vector<float> packed(static_cast<size_t>(nverts) * 3);
    const auto* pb = reinterpret_cast<const uint8_t*>(pos);
    for (uint32_t i = 0; i < nverts; ++i) std::memcpy(&packed[3 * static_cast<size_t>(i)], pb + static_cast<size_t>(i) * pos_stride_bytes, 12);
    std::vector<float> uvz;
    if (!uv2) uvz.assign(static_cast<size_t>(nverts) * 2, 0.0f);
    ohao_status s;
    if ((s = upload(ctx, ctx->pos, packed.data(), packed.size() * 4, "positions")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->normals, normal4, static_cast<size_t>(nverts) * 16, "normals")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->uvs, uv2 ? uv2 : uvz.data(), static_cast<size_t>(nverts) * 8, "uvs")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->indices, indices, static_cast<size_t>(ntris) * 12, "indices")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->mat_ids, mat_ids, static_cast<size_t>(ntris) * 4, "material ids")) != OHAO_OK) return s;
    ctx->max_mat_id = 0;
    for (uint32_t t = 0; t < ntris; ++t) ctx->max_mat_id = std::max(ctx->max_mat_id, mat_ids[t]);
    ctx->nverts = nverts;
    ctx->ntris = ntris;
    ctx->built = false;
    return OHAO_OK;
}

ohao_status ohao_pt_set_geometry_device(ohao_pt_ctx* ctx, const float* d_pos, uint32_t pos_stride_bytes,
                                        uint32_t nverts, const float* d_normal4, const float* d_uv2,
                                        const uint32_t* d_indices, uint32_t ntris, const uint32_t* d_mat_ids,
                                        ohao_stream stream) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    if ((nverts && (!d_pos || !d_normal4)) || (ntris && (!d_indices || !d_mat_ids)) || pos_stride_bytes < 12 ||
        pos_stride_bytes % 4 != 0)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "set_geometry_device: null array or stride < 12 (or not 4-byte aligned)");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    ctx->built = false;
    ctx->nverts = ctx->ntris = 0;
    const size_t nv = nverts, nt = ntris;
    CK(ctx->pos.ensure(nv * 12), "positions");
    CK(ctx->normals.ensure(nv * 16), "normals");
    CK(ctx->uvs.ensure(nv * 8), "uvs");
    CK(ctx->indices.ensure(nt * 12), "indices");
    CK(ctx->mat_ids.ensure(nt * 4), "material ids");
    if (nv) {
        // positions packed to 12 B per vertex whatever the caller's stride
        CK(cudaMemcpy2DAsync(ctx->pos.p, 12, d_pos, pos_stride_bytes, 12, nv, cudaMemcpyDeviceToDevice, st), "positions");
        CK(cudaMemcpyAsync(ctx->normals.p, d_normal4, nv * 16, cudaMemcpyDeviceToDevice, st), "normals");
        if (d_uv2) CK(cudaMemcpyAsync(ctx->uvs.p, d_uv2, nv * 8, cudaMemcpyDeviceToDevice, st), "uvs");
        else CK(cudaMemsetAsync(ctx->uvs.p, 0, nv * 8, st), "uvs");
    }
    uint32_t maxes[2] = {0, 0};
    if (nt) {
        CK(cudaMemcpyAsync(ctx->indices.p, d_indices, nt * 12, cudaMemcpyDeviceToDevice, st), "indices");
        CK(cudaMemcpyAsync(ctx->mat_ids.p, d_mat_ids, nt * 4, cudaMemcpyDeviceToDevice, st), "material ids");
        DevBuf m;
        CK(m.ensure(8), "range check");
        CK(cudaMemsetAsync(m.p, 0, 8, st), "range check");
        ohao::launch_max_u32(ctx->indices.as<uint32_t>(), nt * 3, m.as<uint32_t>(), st);
        ohao::launch_max_u32(ctx->mat_ids.as<uint32_t>(), nt, m.as<uint32_t>() + 1, st);
        CK(cudaGetLastError(), "range check");
        CK(cudaMemcpyAsync(maxes, m.p, 8, cudaMemcpyDeviceToHost, st), "range check");
    }
    CK(cudaStreamSynchronize(st), "set_geometry_device");
    if (nt && maxes[0] >= nverts) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_geometry_device: index out of range");
    ctx->max_mat_id = maxes[1];
    ctx->nverts = nverts;
    ctx->ntris = ntris;
    return OHAO_OK;
}

ohao_status ohao_pt_create_blas(ohao_pt_ctx* ctx, uint32_t first_index, uint32_t index_count, uint32_t* out_blas) {
    if (!ctx || !out_blas) return OHAO_ERR_INVALID_ARG;
    *out_blas = 0xFFFFFFFFu;   // INVALID_BLAS
    if (index_count % 3 != 0 || static_cast<uint64_t>(first_index) + index_count > static_cast<uint64_t>(ctx->ntris) * 3)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "create_blas: index range outside the geometry");
    ctx->blas.push_back({first_index, index_count, 0u});
    *out_blas = static_cast<uint32_t>(ctx->blas.size() - 1);
    ctx->built = false;
    return OHAO_OK;
}

ohao_status ohao_pt_set_instances(ohao_pt_ctx* ctx, const ohao_pt_instance* inst, uint32_t n) {
    if (!ctx || (n && !inst)) return OHAO_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i)
        if (inst[i].blas >= ctx->blas.size()) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_instances: unknown BLAS handle");
    ctx->instances.assign(inst, inst + n);
    ctx->built = false;
    return OHAO_OK;
}

int32_t ohao_pt_is_two_level(const ohao_pt_ctx* ctx) { return ctx && ctx->two_level ? 1 : 0; }

ohao_status ohao_pt_build(ohao_pt_ctx* ctx, ohao_stream stream) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    ctx->built = false;   // a build that fails part way leaves no usable structure
    ctx->emis_dirty = true;
    // BLAS ranges were checked when created; geometry set since may be smaller
    for (const auto& b : ctx->blas)
        if (static_cast<uint64_t>(b.first_index) + b.index_count > static_cast<uint64_t>(ctx->ntris) * 3)
            return fail(ctx, OHAO_ERR_INVALID_ARG, "build: a BLAS index range lies outside the current geometry");
    // An instance whose 3x3 part is singular (zero scale, often used to hide
    // an instance) or not finite has no world-to-object transform: it is
    // treated as masked out, in the flat and the two-level build alike.
    std::vector<ohao_pt_instance> insts = ctx->instances;
    for (auto& in : insts)
        if (!instance_invertible(in.transform)) in.mask = 0;
    const uint32_t ninst = static_cast<uint32_t>(insts.size());
    // per-instance device records
    std::vector<ohao::DInst> di(std::max(ninst, 1u));
    for (uint32_t i = 0; i < ninst; ++i) {
        instance_matrices(insts[i].transform, di[i].w2o, di[i].nrm);
        di[i].custom = insts[i].custom_index;
        di[i].blas = insts[i].blas;
        di[i].mask = insts[i].mask & 0xFFu;
        if (ctx->blas[insts[i].blas].flags & OHAO_BLAS_FLAG_NO_OPAQUE) di[i].mask |= ohao::kInstNoOpaque;
    }
    ohao_status s = upload(ctx, ctx->inst_dev, di.data(), di.size() * sizeof(ohao::DInst), "instances");
    if (s != OHAO_OK) return s;
    uint64_t total = 0;
    for (const auto& in : insts)
        if (in.mask & 0xFFu) total += ctx->blas[in.blas].index_count / 3;
    for (const auto& in : insts) {
        const uint64_t last = static_cast<uint64_t>(in.custom_index & 0xFFFFFFu) + ctx->blas[in.blas].index_count / 3;
        if ((in.mask & 0xFFu) && last > ctx->ntris)
            return fail(ctx, OHAO_ERR_INVALID_ARG, "build: custom_index + primitive id exceeds the global triangle count");
    }
    if (total >= (1ull << 31) && total <= ctx->flatten_limit)
        return fail(ctx, OHAO_ERR_UNSUPPORTED, "build: more than 2^31 instanced triangles in a flat BVH");
    ctx->two_level = total > ctx->flatten_limit;
    ctx->blas_bvh.clear();
    DevBuf tv, tinst, tprim, boxes;
    if (!ctx->two_level) {
        const uint32_t n = static_cast<uint32_t>(total);
        std::vector<uint32_t> first_index, tri_off, vis;
        std::vector<float> o2w;
        uint32_t acc = 0;
        for (uint32_t i = 0; i < ninst; ++i) {
            const auto& in = insts[i];
            if (!(in.mask & 0xFFu)) continue;
            vis.push_back(i);
            first_index.push_back(ctx->blas[in.blas].first_index);
            tri_off.push_back(acc);
            acc += ctx->blas[in.blas].index_count / 3;
            o2w.insert(o2w.end(), in.transform, in.transform + 12);
        }
        DevBuf dfi, dto, do2w;
        if ((s = upload(ctx, dfi, first_index.data(), first_index.size() * 4, "build")) != OHAO_OK) return s;
        if ((s = upload(ctx, dto, tri_off.data(), tri_off.size() * 4, "build")) != OHAO_OK) return s;
        if ((s = upload(ctx, do2w, o2w.data(), o2w.size() * 4, "build")) != OHAO_OK) return s;
        CK(tv.ensure(static_cast<size_t>(std::max(n, 1u)) * 36), "build");
        CK(tinst.ensure(static_cast<size_t>(std::max(n, 1u)) * 4), "build");
        CK(tprim.ensure(static_cast<size_t>(std::max(n, 1u)) * 4), "build");
        CK(boxes.ensure(static_cast<size_t>(std::max(n, 1u)) * 24), "build");
        ohao::launch_flat_triangles(ctx->pos.as<float>(), ctx->indices.as<uint32_t>(), dfi.as<uint32_t>(),
                                    dto.as<uint32_t>(), do2w.as<float>(), static_cast<uint32_t>(vis.size()), n,
                                    tv.as<float>(), tinst.as<uint32_t>(), tprim.as<uint32_t>(), boxes.as<float>(), st);
        // map the visible-instance index back to the instance id
        if (vis.size() != ninst && n) {
            std::vector<uint32_t> h_inst(n);
            CK(cudaMemcpyAsync(h_inst.data(), tinst.p, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, st), "build");
            CK(cudaStreamSynchronize(st), "build");
            for (auto& v : h_inst) v = vis[v];
            CK(cudaMemcpy(tinst.p, h_inst.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice), "build");
        }
        if ((s = build_one(ctx, boxes.as<float>(), n, ctx->flat, st)) != OHAO_OK) return s;
        DevBuf recs;
        CK(recs.ensure(static_cast<size_t>(std::max(n, 1u)) * 48), "build");
        ohao::launch_gather_records(tv.as<float>(), tinst.as<uint32_t>(), tprim.as<uint32_t>(),
                                    ctx->flat.prims.as<uint32_t>(), n, recs.as<float4>(), st);
        CK(cudaStreamSynchronize(st), "build");
        std::swap(ctx->flat.prims.p, recs.p);
        std::swap(ctx->flat.prims.n, recs.n);
        CK(ctx->blas_desc.ensure(sizeof(ohao::DBlas)), "build");
    } else {
        // BLAS builds
        const uint32_t nb = static_cast<uint32_t>(ctx->blas.size());
        ctx->blas_bvh.resize(nb);
        std::vector<ohao::DBlas> desc(nb);
        uint64_t node_total = 0, tri_total = 0;
        for (uint32_t b = 0; b < nb; ++b) {
            const uint32_t n = ctx->blas[b].index_count / 3;
            CK(tv.ensure(static_cast<size_t>(std::max(n, 1u)) * 36), "build");
            CK(tinst.ensure(static_cast<size_t>(std::max(n, 1u)) * 4), "build");
            CK(tprim.ensure(static_cast<size_t>(std::max(n, 1u)) * 4), "build");
            CK(boxes.ensure(static_cast<size_t>(std::max(n, 1u)) * 24), "build");
            ohao::launch_blas_triangles(ctx->pos.as<float>(), ctx->indices.as<uint32_t>(), ctx->blas[b].first_index, n,
                                        tv.as<float>(), tinst.as<uint32_t>(), tprim.as<uint32_t>(), boxes.as<float>(), st);
            BvhDev& bv = ctx->blas_bvh[b];
            if ((s = build_one(ctx, boxes.as<float>(), n, bv, st)) != OHAO_OK) return s;
            DevBuf recs;
            CK(recs.ensure(static_cast<size_t>(std::max(n, 1u)) * 48), "build");
            ohao::launch_gather_records(tv.as<float>(), tinst.as<uint32_t>(), tprim.as<uint32_t>(), bv.prims.as<uint32_t>(),
                                        n, recs.as<float4>(), st);
            CK(cudaStreamSynchronize(st), "build");
            std::swap(bv.prims.p, recs.p);
            std::swap(bv.prims.n, recs.n);
            desc[b] = {static_cast<uint32_t>(node_total), static_cast<uint32_t>(tri_total), bv.nnodes, n};
            node_total += bv.nnodes;
            tri_total += n;
        }
        CK(ctx->blas_nodes_all.ensure(std::max<uint64_t>(node_total, 1) * 80), "build");
        CK(ctx->blas_tris_all.ensure(std::max<uint64_t>(tri_total, 1) * 48), "build");
        for (uint32_t b = 0; b < nb; ++b) {
            const BvhDev& bv = ctx->blas_bvh[b];
            if (bv.nnodes)
                CK(cudaMemcpyAsync(ctx->blas_nodes_all.as<char>() + static_cast<size_t>(desc[b].node_off) * 80, bv.nodes.p,
                                   static_cast<size_t>(bv.nnodes) * 80, cudaMemcpyDeviceToDevice, st), "build");
            if (bv.nprims)
                CK(cudaMemcpyAsync(ctx->blas_tris_all.as<char>() + static_cast<size_t>(desc[b].tri_off) * 48, bv.prims.p,
                                   static_cast<size_t>(bv.nprims) * 48, cudaMemcpyDeviceToDevice, st), "build");
        }
        if ((s = upload(ctx, ctx->blas_desc, desc.data(), desc.size() * sizeof(ohao::DBlas), "build")) != OHAO_OK) return s;
        // TLAS over visible instances' world boxes: min/max of every
        // transformed vertex of the instance's BLAS, on the device
        std::vector<float> xf;
        std::vector<uint32_t> span, ids;
        for (uint32_t i = 0; i < ninst; ++i) {
            const auto& in = insts[i];
            if (!(in.mask & 0xFFu) || ctx->blas_bvh[in.blas].nprims == 0) continue;
            xf.insert(xf.end(), in.transform, in.transform + 12);
            span.push_back(desc[in.blas].tri_off);
            span.push_back(desc[in.blas].ntris);
            ids.push_back(i);
        }
        const uint32_t ni = static_cast<uint32_t>(ids.size());
        DevBuf dxf, dspan, dib;
        if ((s = upload(ctx, dxf, xf.data(), xf.size() * 4, "build")) != OHAO_OK) return s;
        if ((s = upload(ctx, dspan, span.data(), span.size() * 4, "build")) != OHAO_OK) return s;
        CK(dib.ensure(static_cast<size_t>(std::max(ni, 1u)) * 24), "build");
        ohao::launch_instance_boxes(dxf.as<float>(), dspan.as<uint32_t>(), ctx->blas_tris_all.as<float4>(), ni,
                                    dib.as<float>(), st);
        if ((s = build_one(ctx, dib.as<float>(), ni, ctx->flat, st)) != OHAO_OK) return s;
        std::vector<uint32_t> order(ni);
        if (ni) CK(cudaMemcpy(order.data(), ctx->flat.prims.p, static_cast<size_t>(ni) * 4, cudaMemcpyDeviceToHost), "build");
        for (auto& v : order) v = ids[v];
        if (ni) CK(cudaMemcpy(ctx->flat.prims.p, order.data(), static_cast<size_t>(ni) * 4, cudaMemcpyHostToDevice), "build");
    }
    CK(cudaStreamSynchronize(st), "build");
    ctx->built = true;
    return OHAO_OK;
}

// Texture slots of a 48-byte material record (layout_meta.hpp:20-58):
// diffuse [3], normal [6], emissive [7], roughness-metal [8].
constexpr uint32_t kNoTex = 0xFFFFFFFFu;
constexpr uint32_t kMaxTextures = 65536u;
static bool material_indices_valid(const float* m, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i)
        for (int slot : {3, 6, 7, 8}) {
            uint32_t t;
            std::memcpy(&t, m + 12 * static_cast<size_t>(i) + slot, 4);
            if (t != kNoTex && t >= kMaxTextures) return false;
        }
    return true;
}

// Re-summarises the texture indices of the host copy of the material table
// (called when the table changes, so renders check two numbers).
static void summarise_material_textures(ohao_pt_ctx* ctx) {
    ctx->mat_max_tex = -1;
    ctx->mat_uses_diffuse0 = false;
    const size_t n = ctx->mats_host.size() / 12;
    for (size_t i = 0; i < n; ++i)
        for (int slot : {3, 6, 7, 8}) {
            uint32_t t;
            std::memcpy(&t, ctx->mats_host.data() + 12 * i + slot, 4);
            if (t == kNoTex) continue;
            if (slot == 3 && t == 0u) {
                ctx->mat_uses_diffuse0 = true;
                continue;
            }
            ctx->mat_max_tex = std::max<int64_t>(ctx->mat_max_tex, t);
        }
}

// Whether every texture index of the material table names a texture (or,
// for diffuse index 0, the tile albedo map when one is set).
static bool material_textures_bound(const ohao_pt_ctx* ctx) {
    if (ctx->mat_max_tex >= static_cast<int64_t>(ctx->ntex)) return false;
    return !ctx->mat_uses_diffuse0 || ctx->map_w > 0 || ctx->ntex > 0;
}

// Whether any material uses a bindless texture (the tile albedo map aside).
static bool material_uses_textures(const ohao_pt_ctx* ctx) {
    return ctx->mat_max_tex >= 0 || (ctx->mat_uses_diffuse0 && ctx->map_w == 0);
}

ohao_status ohao_pt_set_materials(ohao_pt_ctx* ctx, const float* m, uint32_t n) {
    if (!ctx || (n && !m)) return OHAO_ERR_INVALID_ARG;
    if (!material_indices_valid(m, n))
        return fail(ctx, OHAO_ERR_INVALID_ARG, "set_materials: a texture index is neither 0xFFFFFFFF nor below 65536");
    ohao_status s = upload(ctx, ctx->mats, m, static_cast<size_t>(n) * 48, "materials");
    ctx->emis_dirty = true;
    ctx->nmats = s == OHAO_OK ? n : 0;   // a failed upload may have released the table
    if (s == OHAO_OK) ctx->mats_host.assign(m, m + static_cast<size_t>(n) * 12);
    else ctx->mats_host.clear();
    summarise_material_textures(ctx);
    return s;
}

ohao_status ohao_pt_update_materials(ohao_pt_ctx* ctx, const float* m, uint32_t first, uint32_t n) {
    if (!ctx || (n && !m)) return OHAO_ERR_INVALID_ARG;
    if (static_cast<uint64_t>(first) + n > ctx->nmats) return fail(ctx, OHAO_ERR_INVALID_ARG, "update_materials: range outside the table");
    if (!material_indices_valid(m, n))
        return fail(ctx, OHAO_ERR_INVALID_ARG, "update_materials: a texture index is neither 0xFFFFFFFF nor below 65536");
    if (n) CK(cudaMemcpy(ctx->mats.as<char>() + static_cast<size_t>(first) * 48, m, static_cast<size_t>(n) * 48, cudaMemcpyHostToDevice), "materials");
    for (size_t i = 0; i < n && !ctx->emis_dirty; ++i) {   // the emission fields: emissive texture, slot-2 emission
        const float* o = &ctx->mats_host[(first + i) * 12];
        const float* q = m + i * 12;
        if (std::memcmp(o + 7, q + 7, 4) != 0 || std::memcmp(o + 9, q + 9, 12) != 0) ctx->emis_dirty = true;
    }
    std::copy(m, m + static_cast<size_t>(n) * 12, ctx->mats_host.begin() + static_cast<size_t>(first) * 12);
    summarise_material_textures(ctx);
    return OHAO_OK;
}

ohao_status ohao_pt_set_textures(ohao_pt_ctx* ctx, const ohao_pt_texture* tex, uint32_t n) {
    if (!ctx || (n && !tex)) return OHAO_ERR_INVALID_ARG;
    if (n > kMaxTextures) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_textures: more than 65536 textures");
    uint64_t total = 0;
    std::vector<uint32_t> info(static_cast<size_t>(std::max(n, 1u)) * 4, 0u);
    for (uint32_t i = 0; i < n; ++i) {
        if (!tex[i].rgba8 || tex[i].width == 0 || tex[i].height == 0 || tex[i].width > 65536u || tex[i].height > 65536u)
            return fail(ctx, OHAO_ERR_INVALID_ARG, "set_textures: null texels or a size outside [1, 65536]");
        info[4 * i] = static_cast<uint32_t>(total);
        info[4 * i + 1] = tex[i].width;
        info[4 * i + 2] = tex[i].height;
        total += static_cast<uint64_t>(tex[i].width) * tex[i].height;
        if (total >= (1ull << 32)) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_textures: more than 2^32 texels");
    }
    ctx->ntex = 0;   // until every upload below has succeeded
    CK(ctx->tex_texels.ensure(std::max<uint64_t>(total, 1) * 4), "textures");
    for (uint32_t i = 0; i < n; ++i)
        CK(cudaMemcpy(ctx->tex_texels.as<uint8_t>() + static_cast<size_t>(info[4 * i]) * 4, tex[i].rgba8,
                      static_cast<size_t>(tex[i].width) * tex[i].height * 4, cudaMemcpyHostToDevice), "textures");
    ohao_status s = upload(ctx, ctx->tex_info, info.data(), info.size() * 4, "texture table");
    if (s != OHAO_OK) return s;
    ctx->ntex = n;
    return OHAO_OK;
}

ohao_status ohao_pt_set_blas_flags(ohao_pt_ctx* ctx, uint32_t blas, uint32_t flags) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    if (blas >= ctx->blas.size()) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_blas_flags: unknown BLAS handle");
    if (flags & ~OHAO_BLAS_FLAG_NO_OPAQUE) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_blas_flags: unknown flag");
    ctx->blas[blas].flags = flags;
    ctx->built = false;
    return OHAO_OK;
}

ohao_status ohao_pt_set_lights(ohao_pt_ctx* ctx, const ohao_gpu_light* l, uint32_t n) {
    if (!ctx || (n && !l)) return OHAO_ERR_INVALID_ARG;
    if (n > 64) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_lights: at most 64 lights (MAX_GPU_LIGHTS)");
    ohao_status s = upload(ctx, ctx->lights, l, static_cast<size_t>(n) * 80, "lights");
    ctx->nlights = s == OHAO_OK ? n : 0;
    return s;
}

// Guide tables for the device's inverse-CDF searches (env_guide.hpp), when
// the marginal and every conditional row are non-decreasing; otherwise the
// device searches whole rows. Either way it samples the same texels.
static ohao_status build_env_guides(ohao_pt_ctx* ctx, const float* marg, const float* cond, uint32_t w, uint32_t h) {
    namespace eg = ohao_env_guide;
    if (w > eg::kMaxEntries || h > eg::kMaxEntries || !eg::monotone(marg, h)) return OHAO_OK;
    for (uint32_t y = 0; y < h; ++y)
        if (!eg::monotone(cond + static_cast<size_t>(y) * w, w)) return OHAO_OK;
    const uint32_t mm = eg::cells_for(h), mc = eg::cells_for(w);
    std::vector<uint16_t> gm(mm + 1), gc(static_cast<size_t>(h) * (mc + 1));
    eg::build(marg, h, mm, gm.data());
    for (uint32_t y = 0; y < h; ++y)
        eg::build(cond + static_cast<size_t>(y) * w, w, mc, gc.data() + static_cast<size_t>(y) * (mc + 1));
    ohao_status s = upload(ctx, ctx->guide_marg, gm.data(), gm.size() * 2, "env marginal guide");
    if (s == OHAO_OK) s = upload(ctx, ctx->guide_cond, gc.data(), gc.size() * 2, "env conditional guide");
    if (s != OHAO_OK) return s;
    ctx->guide_mm = mm;
    ctx->guide_mc = mc;
    ctx->has_guide = true;
    return OHAO_OK;
}

ohao_status ohao_pt_set_env(ohao_pt_ctx* ctx, const float* rgba, uint32_t w, uint32_t h, const float* marg,
                            const float* cond, float integral, float intensity) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    (void)integral;
    if (!rgba || w == 0 || h == 0) {
        ctx->has_env = ctx->has_cdf = ctx->has_guide = false;
        ctx->env_w = ctx->env_h = 0;
        return OHAO_OK;
    }
    ctx->has_env = ctx->has_cdf = ctx->has_guide = false;   // until every upload below has succeeded
    ctx->env_w = ctx->env_h = 0;
    ohao_status s = upload(ctx, ctx->env, rgba, static_cast<size_t>(w) * h * 16, "env");
    if (s != OHAO_OK) return s;
    if (marg && cond) {
        if ((s = upload(ctx, ctx->marg, marg, static_cast<size_t>(h) * 4, "env marginal")) != OHAO_OK) return s;
        if ((s = upload(ctx, ctx->cond, cond, static_cast<size_t>(w) * h * 4, "env conditional")) != OHAO_OK) return s;
        ctx->has_cdf = true;
        if ((s = build_env_guides(ctx, marg, cond, w, h)) != OHAO_OK) return s;
    }
    ctx->has_env = true;
    ctx->env_w = w;
    ctx->env_h = h;
    ctx->env_intensity = intensity;
    return OHAO_OK;
}

ohao_status ohao_pt_set_albedo_map(ohao_pt_ctx* ctx, const float* rgb, uint32_t w, uint32_t h) {
    if (!ctx) return OHAO_ERR_INVALID_ARG;
    if (!rgb || !w || !h) { ctx->map_w = ctx->map_h = 0; return OHAO_OK; }
    ohao_status s = upload(ctx, ctx->albedo_map, rgb, static_cast<size_t>(w) * h * 12, "albedo map");
    ctx->map_w = s == OHAO_OK ? w : 0;
    ctx->map_h = s == OHAO_OK ? h : 0;
    return s;
}

ohao_status ohao_env_cdf_build(const float* px, int32_t w, int32_t h, float* marg, float* cond, float* integral) {
    if (!px || !marg || !cond || !integral || w <= 0 || h <= 0) return OHAO_ERR_INVALID_ARG;
    std::vector<float> rowSum(static_cast<size_t>(h), 0.0f);
    const float kPi = 3.14159265358979323846f;
    for (int y = 0; y < h; ++y) {
        const float theta = kPi * (float(y) + 0.5f) / float(h);
        const float sinT = std::sin(theta);
        float acc = 0.0f;
        for (int x = 0; x < w; ++x) {
            const float* p = px + (static_cast<size_t>(y) * w + x) * 4;
            const float lw = (0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2]) * sinT;
            acc += lw;
            cond[static_cast<size_t>(y) * w + x] = acc;
        }
        if (acc > 0.0f) {
            for (int x = 0; x < w; ++x) cond[static_cast<size_t>(y) * w + x] /= acc;
        } else {
            for (int x = 0; x < w; ++x) cond[static_cast<size_t>(y) * w + x] = float(x + 1) / float(w);
        }
        rowSum[static_cast<size_t>(y)] = acc;
    }
    float total = 0.0f;
    for (int y = 0; y < h; ++y) { total += rowSum[static_cast<size_t>(y)]; marg[y] = total; }
    *integral = total;
    if (total > 0.0f) for (int y = 0; y < h; ++y) marg[y] /= total;
    else for (int y = 0; y < h; ++y) marg[y] = float(y + 1) / float(h);
    return OHAO_OK;
}

static ohao_status validate_render(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                   const ohao_pt_settings* st) {
    if (!ctx || !views || !st || n_views == 0) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: null argument");
    if (!ctx->built) return fail(ctx, OHAO_ERR_NOT_BUILT, "render before ohao_pt_build");
    if (ctx->ntris && ctx->max_mat_id >= ctx->nmats)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "render: a triangle's material id is outside the material table");
    if (!material_textures_bound(ctx))
        return fail(ctx, OHAO_ERR_INVALID_ARG, "render: a material's texture index names no texture");
    if (st->spp == 0) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: spp must be >= 1");
    if (st->max_bounces > 64) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: max_bounces > 64");
    if (st->sampler > 1) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: unknown sampler");
    if (st->mode > OHAO_PT_MODE_PERSISTENT) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: unknown mode");
    if (st->wavefront_refill > 33u) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: wavefront_refill above 33");
    for (uint32_t v = 0; v < n_views; ++v)
        if (views[v].width == 0 || views[v].height == 0 || static_cast<uint64_t>(views[v].width) * views[v].height > (1ull << 31))
            return fail(ctx, OHAO_ERR_INVALID_ARG, "render: bad view size");
    return OHAO_OK;
}

// Traversal shape of the per-view wavefront (settings.wavefront_refill; 33 =
// one ray per thread). The default (0) depends on the scene: one ray per
// thread on a flat BVH (sphere_1m: the persistent warps 1-5% slower per
// frame), persistent warps refilled at 8 idle lanes on a two-level one (the
// instanced scene: 3.5% faster per frame).
static uint32_t wavefront_refill(const ohao_pt_ctx* ctx, const ohao_pt_settings* st) {
    if (st->wavefront_refill == 0u) return ctx->two_level ? 8u : 0u;
    return st->wavefront_refill >= 33u ? 0u : st->wavefront_refill;
}

static bool any_non_opaque(const ohao_pt_ctx* ctx) {
    for (const auto& b : ctx->blas)
        if (b.flags & OHAO_BLAS_FLAG_NO_OPAQUE) return true;
    return false;
}

// Light-NEE weight of a material's emission: the luminance of its slot-2
// emission (negative channels as 0), + 1 with an emissive texture; > 0 makes
// the material's triangles emissive for emitter MIS.
static float emission_weight(const float* m) {
    uint32_t etex;
    std::memcpy(&etex, m + 7, 4);
    float l = 0.2126f * std::max(m[9], 0.0f) + 0.7152f * std::max(m[10], 0.0f) + 0.0722f * std::max(m[11], 0.0f);
    if (etex != 0xFFFFFFFFu) l = l + 1.0f;
    return l;
}

// The emissive-triangle table of emitter MIS. Entries run over the
// instances in order (visible, invertible instances of opaque BLASes only)
// and over each one's emissive triangles in order: world-space corner p0
// (the instance transform applied as the flat build applies it), edges
// p1 - p0, p2 - p0, the (instance, prim) ids, and the pdf per unit area of
// choosing a point there: (its CDF step) / area, where the CDF runs over
// area x emission_weight (in double, rounded to float, the last entry 1).
static ohao_status build_emitter_table(ohao_pt_ctx* ctx) {
    ctx->nemis = 0;
    const uint32_t nm = ctx->nmats, nt = ctx->ntris;
    std::vector<float> wmat(nm);
    bool any = false;
    for (uint32_t m = 0; m < nm; ++m) {
        wmat[m] = emission_weight(&ctx->mats_host[static_cast<size_t>(m) * 12]);
        any = any || wmat[m] > 0.0f;
    }
    if (!any || nt == 0 || ctx->instances.empty()) {
        ctx->emis_dirty = false;
        return OHAO_OK;
    }
    std::vector<uint32_t> mids(nt), idx(static_cast<size_t>(nt) * 3);
    std::vector<float> pos(static_cast<size_t>(ctx->nverts) * 3);
    CK(cudaDeviceSynchronize(), "emitter table");
    CK(cudaMemcpy(mids.data(), ctx->mat_ids.p, mids.size() * 4, cudaMemcpyDeviceToHost), "emitter table");
    CK(cudaMemcpy(idx.data(), ctx->indices.p, idx.size() * 4, cudaMemcpyDeviceToHost), "emitter table");
    CK(cudaMemcpy(pos.data(), ctx->pos.p, pos.size() * 4, cudaMemcpyDeviceToHost), "emitter table");
    std::vector<uint32_t> rank(nt);
    uint32_t cnt = 0;
    for (uint32_t g = 0; g < nt; ++g) {
        const bool em = wmat[mids[g]] > 0.0f;
        rank[g] = cnt | (em ? 0x80000000u : 0u);
        cnt += em ? 1u : 0u;
    }
    const uint32_t ninst = static_cast<uint32_t>(ctx->instances.size());
    std::vector<uint32_t> itab(static_cast<size_t>(ninst) * 2);
    std::vector<float> tri;     // 12 floats per entry
    std::vector<float> area;
    std::vector<double> acc;
    double total = 0.0;
    for (uint32_t ii = 0; ii < ninst; ++ii) {
        const ohao_pt_instance& in = ctx->instances[ii];
        const BlasDesc& b = ctx->blas[in.blas];
        const uint32_t first = in.custom_index & 0xFFFFFFu, count = b.index_count / 3;
        itab[2 * ii] = 0xFFFFFFFFu;
        itab[2 * ii + 1] = 0u;
        if (!(in.mask & 0xFFu) || !instance_invertible(in.transform) || (b.flags & OHAO_BLAS_FLAG_NO_OPAQUE) ||
            static_cast<uint64_t>(first) + count > nt)
            continue;
        itab[2 * ii] = static_cast<uint32_t>(area.size());
        itab[2 * ii + 1] = count ? (rank[first] & 0x7FFFFFFFu) : 0u;
        const float* x = in.transform;
        for (uint32_t p = 0; p < count; ++p) {
            if (!(rank[first + p] & 0x80000000u)) continue;
            float w[3][3];
            for (int k = 0; k < 3; ++k) {
                const float* v = &pos[static_cast<size_t>(idx[b.first_index + 3 * p + k]) * 3];
                for (int r = 0; r < 3; ++r)
                    w[k][r] = ((x[r * 4] * v[0] + x[r * 4 + 1] * v[1]) + x[r * 4 + 2] * v[2]) + x[r * 4 + 3];
            }
            float e1[3], e2[3];
            for (int r = 0; r < 3; ++r) {
                e1[r] = w[1][r] - w[0][r];
                e2[r] = w[2][r] - w[0][r];
            }
            const float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                        cz = e1[0] * e2[1] - e1[1] * e2[0];
            const float a = 0.5f * std::sqrt((cx * cx + cy * cy) + cz * cz);
            total += static_cast<double>(a * wmat[mids[first + p]]);
            acc.push_back(total);
            area.push_back(a);
            uint32_t ib = ii, pb = p;
            float ibf, pbf;
            std::memcpy(&ibf, &ib, 4);
            std::memcpy(&pbf, &pb, 4);
            const float e[12] = {w[0][0], w[0][1], w[0][2], 0.0f, e1[0], e1[1], e1[2], ibf, e2[0], e2[1], e2[2], pbf};
            tri.insert(tri.end(), e, e + 12);
        }
    }
    const size_t ne = area.size();
    if (ne == 0 || !(total > 0.0) || ne >= (1ull << 31)) {
        ctx->emis_dirty = false;
        return OHAO_OK;
    }
    std::vector<float> cdf(ne);
    for (size_t i = 0; i < ne; ++i) cdf[i] = static_cast<float>(acc[i] / total);
    cdf[ne - 1] = 1.0f;
    for (size_t i = 0; i < ne; ++i) {
        const float pmf = cdf[i] - (i ? cdf[i - 1] : 0.0f);
        tri[12 * i + 3] = area[i] > 0.0f ? pmf / area[i] : 0.0f;
    }
    ohao_status s;
    if ((s = upload(ctx, ctx->emis_tri, tri.data(), tri.size() * 4, "emitter table")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->emis_cdf, cdf.data(), cdf.size() * 4, "emitter table")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->emis_rank, rank.data(), rank.size() * 4, "emitter table")) != OHAO_OK) return s;
    if ((s = upload(ctx, ctx->emis_inst, itab.data(), itab.size() * 4, "emitter table")) != OHAO_OK) return s;
    ctx->nemis = static_cast<uint32_t>(ne);
    ctx->emis_dirty = false;
    return OHAO_OK;
}

// The scene as a render with these settings sees it: stack limit, alpha
// test, and the emitter-MIS table (built here when out of date).
static ohao_status render_scene(ohao_pt_ctx* ctx, const ohao_pt_settings* st, ohao::DScene& sc) {
    sc = make_scene(ctx);
    sc.stack_limit = stack_limit_of(st);
    sc.alpha_test = (st->flags & OHAO_PT_FLAG_ALPHA_TEST) && any_non_opaque(ctx) ? 1u : 0u;
    if (st->flags & OHAO_PT_FLAG_EMITTER_MIS) {
        if (ctx->emis_dirty) {
            const ohao_status s = build_emitter_table(ctx);
            if (s != OHAO_OK) return s;
        }
        sc.emitter_mis = 1u;
        sc.nemis = ctx->nemis;
        if (ctx->nemis) {
            sc.emis_tri = ctx->emis_tri.as<float4>();
            sc.emis_cdf = ctx->emis_cdf.as<float>();
            sc.emis_rank = ctx->emis_rank.as<uint32_t>();
            sc.emis_inst = ctx->emis_inst.as<uint2>();
        }
    }
    return OHAO_OK;
}

static std::vector<ohao::RenderView> to_render_views(const ohao_pt_view* views, uint32_t n, float* const* dev_accum) {
    std::vector<ohao::RenderView> out(n);
    for (uint32_t v = 0; v < n; ++v) {
        ohao::RenderView& rv = out[v];
        std::memcpy(rv.vp.inv_view, views[v].inv_view, 64);
        std::memcpy(rv.vp.inv_proj, views[v].inv_proj, 64);
        rv.vp.width = views[v].width;
        rv.vp.height = views[v].height;
        rv.accum = dev_accum[v];
        rv.history = views[v].history;
        rv.path_out = views[v].path_radiance;
        rv.aov = views[v].aov;
        rv.accum_ready = nullptr;
    }
    return out;
}

static bool use_persistent(const ohao_pt_settings* st, uint32_t n_views) {
    return st->mode == OHAO_PT_MODE_PERSISTENT || (st->mode == OHAO_PT_MODE_AUTO && n_views > 1);
}

static ohao_status ensure_persistent(ohao_pt_ctx* ctx) {
    if (!ctx->persistent) ctx->persistent = ohao::persistent_create();
    if (!ctx->persistent) return fail(ctx, OHAO_ERR_OOM, "persistent renderer: allocation failed");
    return OHAO_OK;
}

// ready: per view, an event recorded when its accumulator's history is in
// place (or null: it is); the render waits for it before reading it.
static ohao_status render_views(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                const ohao_pt_settings* st, float* const* dev_accum, cudaStream_t cs,
                                const cudaEvent_t* ready = nullptr) {
    const bool profile = (st->flags & OHAO_PT_FLAG_PROFILE) != 0;
    ohao::ProfileAcc acc;
    ohao::DScene sc;
    {
        const ohao_status s = render_scene(ctx, st, sc);
        if (s != OHAO_OK) return s;
    }
    ohao::PathParams pp{st->max_bounces, st->sampler, st->flags, st->clamp_luminance, st->aniso_strength,
                        st->aniso_rotation, st->sample_index_base, wavefront_refill(ctx, st)};
    std::vector<ohao::RenderView> rvs = to_render_views(views, n_views, dev_accum);
    if (ready)
        for (uint32_t v = 0; v < n_views; ++v) rvs[v].accum_ready = ready[v];
    if (use_persistent(st, n_views)) {
        // the pool folds paths into the accumulators from its first chunk on
        if (ready)
            for (uint32_t v = 0; v < n_views; ++v)
                if (ready[v]) CK(cudaStreamWaitEvent(cs, ready[v], 0), "wait for the history upload");
        ohao_status s = ensure_persistent(ctx);
        if (s != OHAO_OK) return s;
        if (n_views > ohao::persistent_max_views())
            return fail(ctx, OHAO_ERR_INVALID_ARG, "render: more views than the persistent queue holds (1024)");
        std::string err;
        s = ohao::persistent_render(ctx->persistent, sc, rvs.data(), n_views, pp, st->spp, ctx->flat.root_box, cs,
                                    ctx->err_flag.as<int>(), profile, &acc, err);
        if (s != OHAO_OK) return fail(ctx, s, err);
    } else {
        const uint32_t cap = ohao::wavefront_default_capacity();
        CK(ctx->scratch.ensure(std::max(ohao::wavefront_scratch_bytes(cap), ohao::wavefront_lanes_scratch_bytes(cap))),
           "render scratch");
        for (int l = 0; l < ohao::kWaveLanes; ++l) {
            if (l > 0 && !ctx->wave.main[l])
                CK(cudaStreamCreateWithFlags(&ctx->wave.main[l], cudaStreamNonBlocking), "wavefront streams");
            if (!ctx->wave.aux[l])
                CK(cudaStreamCreateWithFlags(&ctx->wave.aux[l], cudaStreamNonBlocking), "wavefront streams");
        }
        const ohao::WaveStreams& ws = ctx->wave;
        for (uint32_t v = 0; v < n_views; ++v) {
            std::string err;
            const ohao_status s = ohao::wavefront_render(sc, rvs[v], pp, st->spp, ctx->scratch.p, ctx->scratch.n, cap,
                                                         cs, profile, &acc, ctx->err_flag.as<int>(), err, &ws);
            if (s != OHAO_OK) return fail(ctx, s, err);
        }
    }
    if (profile) {
        ohao_pt_profile& p = ctx->profile;
        p.extend_ms = acc.extend_ms; p.shade_ms = acc.shade_ms; p.shadow_ms = acc.shadow_ms;
        p.other_ms = acc.other_ms; p.total_ms = acc.total_ms;
        p.extend_launches = acc.extend_launches; p.shade_launches = acc.shade_launches;
        p.shadow_launches = acc.shadow_launches; p.other_launches = acc.other_launches;
        p.rays_closest = acc.rays_closest; p.rays_shadow = acc.rays_shadow;
        p.nodes_closest = acc.nodes_closest; p.tris_closest = acc.tris_closest;
        p.nodes_shadow = acc.nodes_shadow; p.tris_shadow = acc.tris_shadow;
        p.lanes = acc.lanes;
        p.reserved = 0;
    }
    return OHAO_OK;
}

ohao_status ohao_pt_autotune(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                             const ohao_pt_settings* st, float* best_ms, ohao_stream stream) {
    ohao_status s = validate_render(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    if (n_views > ohao::persistent_max_views()) return fail(ctx, OHAO_ERR_INVALID_ARG, "autotune: too many views");
    std::vector<float*> acc(n_views);
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!views[v].accum) return fail(ctx, OHAO_ERR_INVALID_ARG, "autotune: view accum is null");
        acc[v] = views[v].accum;
    }
    if ((s = ensure_persistent(ctx)) != OHAO_OK) return s;
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    ohao::PathParams pp{st->max_bounces, st->sampler, st->flags, st->clamp_luminance, st->aniso_strength,
                        st->aniso_rotation, st->sample_index_base, wavefront_refill(ctx, st)};
    const std::vector<ohao::RenderView> rvs = to_render_views(views, n_views, acc.data());
    ohao::DScene sc;
    if ((s = render_scene(ctx, st, sc)) != OHAO_OK) return s;
    std::string err;
    s = ohao::persistent_autotune(ctx->persistent, sc, rvs.data(), n_views, pp, st->spp,
                                  ctx->flat.root_box, cs, ctx->err_flag.as<int>(), best_ms, err);
    if (s != OHAO_OK) return fail(ctx, s, err);
    return check_device_error(ctx, cs);
}

const char* ohao_pt_launch_config(const ohao_pt_ctx* ctx) {
    return ctx && ctx->persistent ? ohao::persistent_variant_name(ctx->persistent) : "default";
}

const char* ohao_pt_launch_config_at(uint32_t index) { return ohao::persistent_variant_at(index); }

ohao_status ohao_pt_set_launch_config(ohao_pt_ctx* ctx, const char* name) {
    if (!ctx || !name) return OHAO_ERR_INVALID_ARG;
    ohao_status s = ensure_persistent(ctx);
    if (s != OHAO_OK) return s;
    if (!ohao::persistent_select(ctx->persistent, name))
        return fail(ctx, OHAO_ERR_INVALID_ARG, std::string("set_launch_config: unknown launch shape ") + name);
    return OHAO_OK;
}

ohao_status ohao_pt_render(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                           const ohao_pt_settings* st, ohao_stream stream) {
    ohao_status s = validate_render(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    std::vector<float*> acc(n_views);
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!views[v].accum) return fail(ctx, OHAO_ERR_INVALID_ARG, "render: view accum is null (use ohao_pt_render_host)");
        acc[v] = views[v].accum;
    }
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    if ((s = render_views(ctx, views, n_views, st, acc.data(), cs)) != OHAO_OK) return s;
    for (uint32_t v = 0; v < n_views; ++v)
        if (views[v].display)
            CK(ohao::launch_display(acc[v], views[v].width * views[v].height, views[v].display, cs), "display");
    return check_device_error(ctx, cs);
}

ohao_status ohao_pt_aov(ohao_pt_ctx* ctx, const ohao_pt_view* view, const ohao_pt_settings* st, float* d_aov,
                        ohao_stream stream) {
    ohao_status s = validate_render(ctx, view, 1, st);
    if (s != OHAO_OK) return s;
    if (!d_aov) return fail(ctx, OHAO_ERR_INVALID_ARG, "aov: null output");
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    ohao::DScene sc = make_scene(ctx);
    sc.stack_limit = stack_limit_of(st);
    sc.alpha_test = (st->flags & OHAO_PT_FLAG_ALPHA_TEST) && any_non_opaque(ctx) ? 1u : 0u;
    const ohao::PathParams pp{st->max_bounces, st->sampler, st->flags, st->clamp_luminance, st->aniso_strength,
                              st->aniso_rotation, st->sample_index_base, wavefront_refill(ctx, st)};
    float* none = nullptr;
    const std::vector<ohao::RenderView> rv = to_render_views(view, 1, &none);
    CK(ohao::launch_aov_mean(sc, pp, rv[0].vp, st->spp, d_aov, ctx->err_flag.as<int>(), cs), "aov");
    return check_device_error(ctx, cs);
}

ohao_status ohao_pt_render_host(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                const ohao_pt_settings* st, float* const* host_accum, ohao_stream stream) {
    ohao_status s = validate_render(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    if (!host_accum) return fail(ctx, OHAO_ERR_INVALID_ARG, "render_host: null host_accum");
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    while (ctx->host_accum_bufs.size() < n_views) ctx->host_accum_bufs.push_back(new DevBuf());
    if (!ctx->upload_stream) CK(cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking), "upload stream");
    while (ctx->upload_done.size() < n_views) {
        cudaEvent_t a = nullptr, b = nullptr;
        CK(cudaEventCreateWithFlags(&a, cudaEventDisableTiming), "upload event");
        if (cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
            cudaEventDestroy(a);
            return fail(ctx, OHAO_ERR_CUDA, "upload event");
        }
        ctx->upload_after.push_back(a);
        ctx->upload_done.push_back(b);
    }
    std::vector<float*> acc(n_views);
    std::vector<cudaEvent_t> ready(n_views, nullptr);
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!host_accum[v]) return fail(ctx, OHAO_ERR_INVALID_ARG, "render_host: null host buffer");
        const size_t bytes = static_cast<size_t>(views[v].width) * views[v].height * 16;
        CK(ctx->host_accum_bufs[v]->ensure(bytes), "host accum");
        acc[v] = ctx->host_accum_bufs[v]->as<float>();
        if (views[v].history > 0) {
            // after everything already on the caller's stream (an earlier
            // call's download of the same buffer), on the upload stream
            CK(cudaEventRecord(ctx->upload_after[v], cs), "upload order");
            CK(cudaStreamWaitEvent(ctx->upload_stream, ctx->upload_after[v], 0), "upload order");
            CK(cudaMemcpyAsync(acc[v], host_accum[v], bytes, cudaMemcpyHostToDevice, ctx->upload_stream),
               "accum upload");
            CK(cudaEventRecord(ctx->upload_done[v], ctx->upload_stream), "upload done");
            ready[v] = ctx->upload_done[v];
        }
    }
    if ((s = render_views(ctx, views, n_views, st, acc.data(), cs, ready.data())) != OHAO_OK) {
        // nothing may still write the buffers once the call has returned
        for (uint32_t v = 0; v < n_views; ++v)
            if (ready[v]) cudaStreamWaitEvent(cs, ready[v], 0);
        return s;
    }
    for (uint32_t v = 0; v < n_views; ++v) {
        const size_t npix = static_cast<size_t>(views[v].width) * views[v].height;
        CK(cudaMemcpyAsync(host_accum[v], acc[v], npix * 16, cudaMemcpyDeviceToHost, cs), "accum download");
        if (views[v].display) {   // host RGBA8 readback of the display image
            while (ctx->host_display_bufs.size() <= v) ctx->host_display_bufs.push_back(new DevBuf());
            CK(ctx->host_display_bufs[v]->ensure(npix * 4), "display image");
            CK(ohao::launch_display(acc[v], static_cast<uint32_t>(npix), ctx->host_display_bufs[v]->as<uint8_t>(), cs),
               "display");
            CK(cudaMemcpyAsync(views[v].display, ctx->host_display_bufs[v]->p, npix * 4, cudaMemcpyDeviceToHost, cs),
               "display download");
        }
    }
    return check_device_error(ctx, cs);
}

static ohao_status validate_backward(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                     const ohao_pt_settings* st) {
    ohao_status s = validate_render(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    if ((st->flags & OHAO_PT_FLAG_FIREFLY_CLAMP) && st->clamp_luminance > 0.0f)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: the firefly clamp is not differentiable; clear the flag");
    if (st->max_bounces > ohao::adjoint_max_bounces())
        return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: max_bounces above 16");
    if (st->flags & OHAO_PT_FLAG_GGX_VNDF)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: the replay differentiates the offline estimator; clear GGX_VNDF");
    if (st->flags & OHAO_PT_FLAG_EMITTER_MIS)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: the replay differentiates the offline estimator; clear EMITTER_MIS");
    if ((st->flags & OHAO_PT_FLAG_ALPHA_TEST) || material_uses_textures(ctx))
        return fail(ctx, OHAO_ERR_UNSUPPORTED,
                    "backward: bindless textures and the alpha test are not differentiated (the tile albedo map is)");
    return OHAO_OK;
}

static ohao_status run_backward(ohao_pt_ctx* ctx, const std::vector<ohao::RenderView>& rvs, const float* const* grads,
                                const ohao_pt_settings* st, float* d_grad_map, float* d_grad_rough, cudaStream_t cs) {
    ohao::PathParams pp{st->max_bounces, st->sampler, st->flags, st->clamp_luminance, st->aniso_strength,
                        st->aniso_rotation, st->sample_index_base, wavefront_refill(ctx, st)};
    const uint32_t n = static_cast<uint32_t>(rvs.size());
    CK(ctx->adj_scratch.ensure(ohao::adjoint_scratch_bytes(n)), "backward scratch");
    std::string err;
    ohao::DScene sc = make_scene(ctx);
    sc.stack_limit = stack_limit_of(st);
    const ohao_status s = ohao::adjoint_backward(sc, rvs.data(), grads, n, pp, st->spp, ctx->nmats,
                                                 ctx->adj_scratch.p, ctx->adj_scratch.n, d_grad_map, d_grad_rough, cs,
                                                 ctx->err_flag.as<int>(), err);
    if (s != OHAO_OK) return fail(ctx, s, err);
    return check_device_error(ctx, cs);
}

ohao_status ohao_pt_backward(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                             const ohao_pt_settings* st, const float* const* d_grad_image, float* d_grad_albedo_map,
                             float* d_grad_roughness, ohao_stream stream) {
    ohao_status s = validate_backward(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    if (!d_grad_image) return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: null image gradient list");
    for (uint32_t v = 0; v < n_views; ++v)
        if (!d_grad_image[v]) return fail(ctx, OHAO_ERR_INVALID_ARG, "backward: null image gradient");
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    std::vector<float*> none(n_views, nullptr);
    const std::vector<ohao::RenderView> rvs = to_render_views(views, n_views, none.data());
    return run_backward(ctx, rvs, d_grad_image, st, d_grad_albedo_map, d_grad_roughness, cs);
}

ohao_status ohao_pt_adjoint(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                  const ohao_pt_settings* st, const float* const* d_targets,
                                  float* d_grad_albedo_map, float* d_grad_roughness, float* loss,
                                  ohao_stream stream) {
    ohao_status s = validate_backward(ctx, views, n_views, st);
    if (s != OHAO_OK) return s;
    if (!d_targets) return fail(ctx, OHAO_ERR_INVALID_ARG, "adjoint: null target list");
    std::vector<ohao_pt_view> fresh(views, views + n_views);
    std::vector<float*> acc(n_views);
    uint64_t total = 0;
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!views[v].accum || !d_targets[v])
            return fail(ctx, OHAO_ERR_INVALID_ARG, "adjoint: null accum or target");
        fresh[v].history = 0;
        acc[v] = views[v].accum;
        total += static_cast<uint64_t>(views[v].width) * views[v].height;
    }
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    if ((s = render_views(ctx, fresh.data(), n_views, st, acc.data(), cs)) != OHAO_OK) return s;
    CK(ctx->adj_grads.ensure(total * 16), "loss gradient images");
    CK(ctx->adj_scratch.ensure(ohao::adjoint_scratch_bytes(n_views)), "backward scratch");
    std::vector<float*> grads(n_views);
    uint64_t off = 0;
    for (uint32_t v = 0; v < n_views; ++v) {
        grads[v] = ctx->adj_grads.as<float>() + off * 4;
        off += static_cast<uint64_t>(views[v].width) * views[v].height;
    }
    const std::vector<ohao::RenderView> rvs = to_render_views(fresh.data(), n_views, acc.data());
    std::string err;
    float l = 0.0f;
    s = ohao::adjoint_mse(rvs.data(), d_targets, n_views, (st->flags & OHAO_PT_FLAG_ADJOINT_LDR_LOSS) != 0,
                          ctx->adj_scratch.p, ctx->adj_scratch.n, grads.data(), &l, cs, err);
    if (s != OHAO_OK) return fail(ctx, s, err);
    if (loss) *loss = l;
    std::vector<const float*> cgrads(grads.begin(), grads.end());
    ohao_pt_settings replay = *st;
    if (st->flags & OHAO_PT_FLAG_ADJOINT_DECORRELATE) replay.sample_index_base = st->sample_index_base + st->spp;
    return run_backward(ctx, rvs, cgrads.data(), &replay, d_grad_albedo_map, d_grad_roughness, cs);
}

ohao_status ohao_pt_adjoint_host(ohao_pt_ctx* ctx, const ohao_pt_view* views, uint32_t n_views,
                                 const ohao_pt_settings* st, const float* const* host_targets,
                                 float* host_grad_albedo_map, float* host_grad_roughness, float* loss,
                                 ohao_stream stream) {
    if (!ctx || !views || !host_targets || n_views == 0) return fail(ctx, OHAO_ERR_INVALID_ARG, "adjoint_host: null argument");
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    while (ctx->host_accum_bufs.size() < n_views) ctx->host_accum_bufs.push_back(new DevBuf());
    while (ctx->host_target_bufs.size() < n_views) ctx->host_target_bufs.push_back(new DevBuf());
    std::vector<ohao_pt_view> dv(views, views + n_views);
    std::vector<const float*> tgt(n_views);
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!host_targets[v]) return fail(ctx, OHAO_ERR_INVALID_ARG, "adjoint_host: null target");
        const size_t bytes = static_cast<size_t>(views[v].width) * views[v].height * 16;
        CK(ctx->host_accum_bufs[v]->ensure(bytes), "adjoint_host accum");
        CK(ctx->host_target_bufs[v]->ensure(bytes), "adjoint_host target");
        CK(cudaMemcpyAsync(ctx->host_target_bufs[v]->p, host_targets[v], bytes, cudaMemcpyHostToDevice, cs),
           "target upload");
        dv[v].accum = ctx->host_accum_bufs[v]->as<float>();
        dv[v].path_radiance = nullptr;
        dv[v].aov = nullptr;
        dv[v].display = nullptr;
        tgt[v] = ctx->host_target_bufs[v]->as<float>();
    }
    const size_t map_floats = static_cast<size_t>(ctx->map_w) * ctx->map_h * 3;
    float* gm = nullptr;
    float* gr = nullptr;
    if (host_grad_albedo_map && map_floats) {
        CK(ctx->host_grad_bufs[0].ensure(map_floats * 4), "gradient buffer");
        gm = ctx->host_grad_bufs[0].as<float>();
    }
    if (host_grad_roughness && ctx->nmats) {
        CK(ctx->host_grad_bufs[1].ensure(static_cast<size_t>(ctx->nmats) * 4), "gradient buffer");
        gr = ctx->host_grad_bufs[1].as<float>();
    }
    const ohao_status s = ohao_pt_adjoint(ctx, dv.data(), n_views, st, tgt.data(), gm, gr, loss, stream);
    if (s != OHAO_OK) return s;
    if (gm) CK(cudaMemcpyAsync(host_grad_albedo_map, gm, map_floats * 4, cudaMemcpyDeviceToHost, cs), "gradient download");
    if (gr)
        CK(cudaMemcpyAsync(host_grad_roughness, gr, static_cast<size_t>(ctx->nmats) * 4, cudaMemcpyDeviceToHost, cs),
           "gradient download");
    CK(cudaStreamSynchronize(cs), "adjoint_host");
    return OHAO_OK;
}

ohao_status ohao_pt_display(const float* d_rgba32f, uint32_t npix, uint8_t* d_rgba8, ohao_stream stream) {
    if (npix && (!d_rgba32f || !d_rgba8)) return OHAO_ERR_INVALID_ARG;
    const cudaError_t e = ohao::launch_display(d_rgba32f, npix, d_rgba8, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? OHAO_OK : OHAO_ERR_CUDA;
}

ohao_status ohao_pt_get_profile(const ohao_pt_ctx* ctx, ohao_pt_profile* out) {
    if (!ctx || !out) return OHAO_ERR_INVALID_ARG;
    *out = ctx->profile;
    return OHAO_OK;
}

ohao_status ohao_pt_trace(ohao_pt_ctx* ctx, const float* rays, uint32_t n, uint32_t* hits, int32_t any_hit,
                          uint32_t* stats, ohao_stream stream) {
    if (!ctx || (n && (!rays || !hits))) return OHAO_ERR_INVALID_ARG;
    if (!ctx->built) return fail(ctx, OHAO_ERR_NOT_BUILT, "trace before ohao_pt_build");
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(ctx->device), "set device");
    std::string err;
    ohao::DScene sc = make_scene(ctx);
    sc.alpha_test = (any_hit & 2) && any_non_opaque(ctx) ? 1u : 0u;
    if ((any_hit & 2) && !material_textures_bound(ctx))
        return fail(ctx, OHAO_ERR_INVALID_ARG, "trace: a material's texture index names no texture");
    const ohao_status s = ohao::trace_rays(sc, rays, n, hits, any_hit & 1, stats, cs, ctx->err_flag.as<int>(), err);
    if (s != OHAO_OK) return fail(ctx, s, err);
    return check_device_error(ctx, cs);
}

ohao_status ohao_pt_bvh_info(const ohao_pt_ctx* ctx, int32_t which, uint32_t* n_nodes, uint32_t* n_prims,
                             uint32_t* height) {
    if (!ctx || !n_nodes || !n_prims || !height) return OHAO_ERR_INVALID_ARG;
    if (!ctx->built) return OHAO_ERR_NOT_BUILT;
    const BvhDev* b;
    if (which < 0) b = &ctx->flat;
    else if (ctx->two_level && static_cast<size_t>(which) < ctx->blas_bvh.size()) b = &ctx->blas_bvh[which];
    else return OHAO_ERR_INVALID_ARG;
    *n_nodes = b->nnodes;
    *n_prims = b->nprims;
    *height = b->height;
    return OHAO_OK;
}

ohao_status ohao_pt_bvh_download(ohao_pt_ctx* ctx, int32_t which, void* nodes, void* prims) {
    uint32_t nn, np, h;
    ohao_status s = ohao_pt_bvh_info(ctx, which, &nn, &np, &h);
    if (s != OHAO_OK) return s;
    const BvhDev* b = which < 0 ? &ctx->flat : &ctx->blas_bvh[which];
    const size_t pbytes = (which < 0 && ctx->two_level) ? 4 : 48;
    if (nn && nodes) CK(cudaMemcpy(nodes, b->nodes.p, static_cast<size_t>(nn) * 80, cudaMemcpyDeviceToHost), "download");
    if (np && prims) CK(cudaMemcpy(prims, b->prims.p, static_cast<size_t>(np) * pbytes, cudaMemcpyDeviceToHost), "download");
    return OHAO_OK;
}

}  // extern "C"
