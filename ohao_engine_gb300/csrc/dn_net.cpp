// dn_net.cpp -- the U-Net denoiser: network graph, buffers, training and
// inference around the tcgen05 convolution kernels, and the ohao_dn_* C ABI.
//
// Graph (level l has 1/2^l of the resolution; C = 32, 48, 64, 96, 128):
//   x -> e0a -> e0 -pool-> p0 -> e1a -> e1 -pool-> p1 -> ... -> p3 -> b4a -> b4
//   d3a = conv(up(b4) | e3), d3 = conv(d3a); ... d0a = conv(up(d1) | e0), d0
//   out = conv(d0) (3 channels, no ReLU), FP32
// Every convolution but the last is followed by ReLU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ohao_dn.h"
#include "dn_types.hpp"

namespace {

using namespace ohao::dn;

struct Buf {
    void* p = nullptr;
    size_t n = 0;
    Buf() = default;
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    Buf(Buf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 256);
        if (e != cudaSuccess) { p = nullptr; return e; }
        n = bytes;
        return cudaMemset(p, 0, bytes ? bytes : 256);
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct Tensor {
    int level = 0;
    int c8 = 0;
    bool f32 = false;     // FP32 activations (the output layer)
    Buf act, grad;
};

struct Layer {
    LayerShape s{};
    int in0 = -1, in1 = -1, out = -1;
    bool up0 = false, relu = true;
    int level = 0;
    Buf w32, w16, wt16, b32, gw, gb, mw, vw, mb, vb;
};

struct Op {
    int kind;   // 0 conv, 1 pool
    int idx;    // layer index (conv) or input tensor (pool)
    int out;    // pool output tensor
};

constexpr int kChannels[5] = {32, 48, 64, 96, 128};
// input channels used: log1p demodulated radiance (3), albedo (3), normal (3),
// inverse depth, roughness, metallic
constexpr int kInputChannels = 12;
constexpr int kWgradBN = 256;  // N tile of the weight-gradient GEMM (features per CTA)

// Deterministic normal draws (PCG32 + Box-Muller), identical on every host.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 6364136223846793005ull + 1442695040888963407ull) {}
    uint32_t next() {
        const uint64_t old = s;
        s = old * 6364136223846793005ull + 1442695040888963407ull;
        const uint32_t x = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (x >> rot) | (x << ((32u - rot) & 31u));
    }
    double uniform() { return (next() + 0.5) / 4294967296.0; }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

struct ohao_dn_ctx {
    int device = 0;
    std::string last_error;
    uint64_t max_pixels = 0;
    std::vector<Tensor> T;
    std::vector<Layer> L;
    std::vector<Op> ops;
    int out_tensor = -1;
    bool grads_ready = false;
    int adam_t = 0;
    Buf err_flag, loss_acc;
    Buf up_scratch;       // the upsampled source of an upsample + concatenation layer's forward
    Geo g0{0, 0, 0, 0};   // grid of the last forward
};

namespace {

ohao_status fail(ohao_dn_ctx* c, ohao_status s, const std::string& m) {
    if (c) c->last_error = m;
    return s;
}
ohao_status cuda_fail(ohao_dn_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? OHAO_ERR_OOM : OHAO_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define DN_CK(expr, what)                                         \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what);   \
    } while (0)

int add_tensor(ohao_dn_ctx* c, int level, int ch, bool f32 = false) {
    Tensor t;
    t.level = level;
    t.c8 = round_up(ch, 8);
    t.f32 = f32;
    c->T.push_back(std::move(t));
    return static_cast<int>(c->T.size()) - 1;
}

int add_conv(ohao_dn_ctx* c, int in0, int in1, bool up0, int cout, bool relu, int cin_used = -1) {
    Layer l;
    l.in0 = in0;
    l.in1 = in1;
    l.up0 = up0;
    l.relu = relu;
    l.level = up0 ? c->T[in0].level - 1 : c->T[in0].level;
    const int cin8 = c->T[in0].c8 + (in1 >= 0 ? c->T[in1].c8 : 0);
    l.s.cin8 = cin8;
    l.s.cin = cin_used > 0 ? cin_used : cin8;
    l.s.cout = cout;
    l.s.cout8 = round_up(cout, 8);
    l.s.cout_n = round_up(cout, 16);
    l.s.cin_n = round_up(cin8, 16);
    l.s.k_pad = round_up(9 * cin8, 64);
    l.s.k2_pad = round_up(9 * l.s.cout8, 64);
    l.out = add_tensor(c, l.level, cout, !relu);
    c->L.push_back(std::move(l));
    c->ops.push_back({0, static_cast<int>(c->L.size()) - 1, -1});
    return c->L.back().out;
}

int add_pool(ohao_dn_ctx* c, int in) {
    const int out = add_tensor(c, c->T[in].level + 1, c->T[in].c8);
    c->ops.push_back({1, in, out});
    return out;
}

void build_graph(ohao_dn_ctx* c) {
    const int x = add_tensor(c, 0, 16);
    int cur = x;
    int skip[4];
    for (int l = 0; l < 5; ++l) {
        const int a = add_conv(c, cur, -1, false, kChannels[l], true, l == 0 ? kInputChannels : -1);
        const int e = add_conv(c, a, -1, false, kChannels[l], true);
        if (l < 4) {
            skip[l] = e;
            cur = add_pool(c, e);
        } else {
            cur = e;
        }
    }
    for (int l = 3; l >= 0; --l) {
        const int a = add_conv(c, cur, skip[l], true, kChannels[l], true);
        cur = add_conv(c, a, -1, false, kChannels[l], true);
    }
    c->out_tensor = add_conv(c, cur, -1, false, 3, false);
}

Geo level_geo(const Geo& g0, int level) {
    Geo g{g0.n, g0.h >> level, g0.w >> level, 0};
    g.npix = static_cast<int64_t>(g.n) * g.h * g.w;
    return g;
}

uint64_t count_params(const ohao_dn_ctx* c) {
    uint64_t n = 0;
    for (const Layer& l : c->L) n += static_cast<uint64_t>(l.s.cout) * 9 * l.s.cin + l.s.cout;
    return n;
}

ohao_status alloc_params(ohao_dn_ctx* ctx) {
    for (Layer& l : ctx->L) {
        const size_t wn = static_cast<size_t>(l.s.cout) * l.s.k_pad;
        DN_CK(l.w32.alloc(wn * 4), "weights");
        DN_CK(l.gw.alloc(wn * 4), "weight grads");
        DN_CK(l.mw.alloc(wn * 4), "adam m");
        DN_CK(l.vw.alloc(wn * 4), "adam v");
        DN_CK(l.w16.alloc(static_cast<size_t>(l.s.cout_n) * l.s.k_pad * 2), "bf16 weights");
        DN_CK(l.wt16.alloc(static_cast<size_t>(l.s.cin_n) * l.s.k2_pad * 2), "bf16 weights^T");
        DN_CK(l.b32.alloc(l.s.cout * 4), "bias");
        DN_CK(l.gb.alloc(l.s.cout * 4), "bias grads");
        DN_CK(l.mb.alloc(l.s.cout * 4), "adam m");
        DN_CK(l.vb.alloc(l.s.cout * 4), "adam v");
    }
    return OHAO_OK;
}

ohao_status alloc_acts(ohao_dn_ctx* ctx, bool grads) {
    for (Tensor& t : ctx->T) {
        const size_t pix = static_cast<size_t>(ctx->max_pixels >> (2 * t.level));
        if (!t.act.p) DN_CK(t.act.alloc(pix * t.c8 * (t.f32 ? 4 : 2)), "activations");
        if (grads && !t.grad.p) DN_CK(t.grad.alloc(pix * t.c8 * 4), "activation grads");
    }
    if (grads) ctx->grads_ready = true;
    if (!ctx->up_scratch.p) {   // the largest upsampled source, at its layer's resolution
        size_t bytes = 0;
        for (const Layer& l : ctx->L)
            if (l.up0)
                bytes = std::max(bytes, static_cast<size_t>(ctx->max_pixels >> (2 * l.level)) * ctx->T[l.in0].c8 * 2);
        if (bytes) DN_CK(ctx->up_scratch.alloc(bytes), "upsample scratch");
    }
    return OHAO_OK;
}

// host layout W[cout][tap][cin] + b[cout] <-> device w32 [cout][k_pad] (k = tap*cin8 + ci)
ohao_status upload_params(ohao_dn_ctx* ctx, const float* host) {
    size_t off = 0;
    for (Layer& l : ctx->L) {
        std::vector<float> w(static_cast<size_t>(l.s.cout) * l.s.k_pad, 0.0f);
        for (int co = 0; co < l.s.cout; ++co)
            for (int tap = 0; tap < 9; ++tap)
                for (int ci = 0; ci < l.s.cin; ++ci)
                    w[static_cast<size_t>(co) * l.s.k_pad + tap * l.s.cin8 + ci] = host[off++];
        DN_CK(cudaMemcpy(l.w32.p, w.data(), w.size() * 4, cudaMemcpyHostToDevice), "weights upload");
        DN_CK(cudaMemcpy(l.b32.p, host + off, l.s.cout * 4, cudaMemcpyHostToDevice), "bias upload");
        off += l.s.cout;
        launch_refresh(l.s, l.w32.as<float>(), l.w16.as<__nv_bfloat16>(), l.wt16.as<__nv_bfloat16>(), nullptr);
    }
    DN_CK(cudaDeviceSynchronize(), "weights refresh");
    return OHAO_OK;
}

ohao_status download(ohao_dn_ctx* ctx, bool grads, float* host) {
    size_t off = 0;
    for (Layer& l : ctx->L) {
        std::vector<float> w(static_cast<size_t>(l.s.cout) * l.s.k_pad);
        DN_CK(cudaMemcpy(w.data(), grads ? l.gw.p : l.w32.p, w.size() * 4, cudaMemcpyDeviceToHost), "download");
        for (int co = 0; co < l.s.cout; ++co)
            for (int tap = 0; tap < 9; ++tap)
                for (int ci = 0; ci < l.s.cin; ++ci)
                    host[off++] = w[static_cast<size_t>(co) * l.s.k_pad + tap * l.s.cin8 + ci];
        DN_CK(cudaMemcpy(host + off, grads ? l.gb.p : l.b32.p, l.s.cout * 4, cudaMemcpyDeviceToHost), "download");
        off += l.s.cout;
    }
    return OHAO_OK;
}

ConvArgs conv_args(ohao_dn_ctx* ctx, Layer& l, const Geo& g0) {
    ConvArgs a{};
    a.g = level_geo(g0, l.level);
    const Tensor& t0 = ctx->T[l.in0];
    a.x0 = t0.act.as<__nv_bfloat16>();
    a.c0 = t0.c8;
    a.c0s = t0.c8;
    a.up0 = l.up0 ? 1 : 0;
    if (l.in1 >= 0) {
        const Tensor& t1 = ctx->T[l.in1];
        a.x1 = t1.act.as<__nv_bfloat16>();
        a.c1 = t1.c8;
        a.c1s = t1.c8;
    }
    a.cin8 = l.s.cin8;
    a.cout = l.s.cout;
    a.cout8 = l.s.cout8;
    a.k_pad = l.s.k_pad;
    a.k2_pad = l.s.k2_pad;
    a.w = l.w16.as<__nv_bfloat16>();
    a.wt = l.wt16.as<__nv_bfloat16>();
    a.bias = l.b32.as<float>();
    a.relu = l.relu ? 1 : 0;
    Tensor& to = ctx->T[l.out];
    if (to.f32) a.yf = to.act.as<float>();
    else a.yout = to.act.as<__nv_bfloat16>();
    a.y = to.f32 ? nullptr : to.act.as<__nv_bfloat16>();
    a.dy = to.grad.as<float>();
    a.dx0 = t0.grad.as<float>();
    if (l.in1 >= 0) a.dx1 = ctx->T[l.in1].grad.as<float>();
    a.dw = l.gw.as<float>();
    return a;
}

ohao_status forward(ohao_dn_ctx* ctx, const Geo& g0, cudaStream_t st) {
    ctx->g0 = g0;
    for (const Op& op : ctx->ops) {
        if (op.kind == 0) {
            Layer& l = ctx->L[op.idx];
            ConvArgs a = conv_args(ctx, l, g0);
            a.bn = l.s.cout_n;
            a.n_tiles = 1;
            if (l.up0 && static_cast<size_t>(a.g.npix) * a.c0s * 2 <= ctx->up_scratch.n)
                a.up_scratch = ctx->up_scratch.as<__nv_bfloat16>();
            DN_CK(launch_conv(kFwd, a, 1, ctx->err_flag.as<int>(), st), "conv forward");
        } else {
            const Tensor& ti = ctx->T[op.idx];
            launch_pool_fwd(ti.act.as<__nv_bfloat16>(), ctx->T[op.out].act.as<__nv_bfloat16>(),
                            level_geo(g0, ti.level + 1), ti.c8, st);
        }
    }
    return OHAO_OK;
}

ohao_status backward(ohao_dn_ctx* ctx, const Geo& g0, cudaStream_t st) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    for (auto it = ctx->ops.rbegin(); it != ctx->ops.rend(); ++it) {
        const Op& op = *it;
        if (op.kind == 0) {
            Layer& l = ctx->L[op.idx];
            ConvArgs a = conv_args(ctx, l, g0);
            launch_bias_grad(a.dy, a.y, l.relu, a.g, l.s.cout, l.s.cout8, l.gb.as<float>(), st);
            // weight gradient: N = features (tap, ci), K = pixels
            const int feat = 9 * l.s.cin8;
            a.bn = std::min(kWgradBN, round_up(feat, 16));
            a.n_tiles = (feat + a.bn - 1) / a.bn;
            const int64_t chunks = (a.g.npix + 63) / 64;
            const int splits = static_cast<int>(
                std::max<int64_t>(1, std::min<int64_t>(chunks, (2 * sms + a.n_tiles - 1) / a.n_tiles)));
            DN_CK(launch_conv(kWgrad, a, splits, ctx->err_flag.as<int>(), st), "conv weight grad");
            if (l.in0 != 0) {   // no gradient for the network input
                a.bn = l.s.cin_n;
                a.n_tiles = 1;
                DN_CK(launch_conv(kDgrad, a, 1, ctx->err_flag.as<int>(), st), "conv data grad");
            }
        } else {
            const Tensor& ti = ctx->T[op.idx];
            launch_pool_bwd(ti.act.as<__nv_bfloat16>(), ctx->T[op.out].grad.as<float>(), ti.grad.as<float>(),
                            level_geo(g0, ti.level + 1), ti.c8, st);
        }
    }
    return OHAO_OK;
}

ohao_status check_flag(ohao_dn_ctx* ctx, cudaStream_t st) {
    DN_CK(cudaStreamSynchronize(st), "denoiser");
    int flag = 0;
    DN_CK(cudaMemcpy(&flag, ctx->err_flag.p, 4, cudaMemcpyDeviceToHost), "error flag");
    if (flag) {
        cudaMemset(ctx->err_flag.p, 0, 4);
        return fail(ctx, OHAO_ERR_TIMEOUT, "denoiser: a tensor-core pipeline wait gave up");
    }
    return OHAO_OK;
}

ohao_status pack_inputs(ohao_dn_ctx* ctx, const float* const* rad, const float* const* aov, uint32_t n, uint32_t w,
                        uint32_t h, Geo& g0, cudaStream_t st) {
    const int wp = round_up(static_cast<int>(w), 16), hp = round_up(static_cast<int>(h), 16);
    g0 = Geo{static_cast<int>(n), hp, wp, static_cast<int64_t>(n) * wp * hp};
    if (static_cast<uint64_t>(g0.npix) > ctx->max_pixels)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "denoiser: batch larger than max_pixels");
    for (uint32_t i = 0; i < n; ++i) {
        if (!rad[i] || !aov[i]) return fail(ctx, OHAO_ERR_INVALID_ARG, "denoiser: null input image");
        launch_pack(rad[i], aov[i], ctx->T[0].act.as<__nv_bfloat16>(), static_cast<int>(w), static_cast<int>(h), wp,
                    hp, static_cast<int64_t>(i) * wp * hp, st);
    }
    return OHAO_OK;
}

}  // namespace

extern "C" {

ohao_status ohao_dn_create(const ohao_dn_desc* desc, ohao_dn_ctx** out) {
    if (!desc || !out || desc->max_pixels == 0 || desc->max_pixels >= (1ull << 31)) return OHAO_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || desc->device < 0 || desc->device >= ndev)
        return OHAO_ERR_INVALID_ARG;
    if (cudaSetDevice(desc->device) != cudaSuccess) return OHAO_ERR_CUDA;
    auto* ctx = new ohao_dn_ctx();
    ctx->device = desc->device;
    ctx->max_pixels = (desc->max_pixels + 255) / 256 * 256;
    build_graph(ctx);
    // every GEMM must fit the kernels' tcgen05.mma shapes: M = 128 and N in
    // [16, 256] a multiple of 16 (forward: N = output channels; data gradient:
    // N = input channels; weight gradient: M = output channels)
    for (const Layer& l : ctx->L) {
        if (l.s.cout_n > 256 || l.s.cin_n > 256 || l.s.cout > 128) {
            delete ctx;
            return OHAO_ERR_UNSUPPORTED;
        }
    }
    ohao_status s = alloc_params(ctx);
    if (s == OHAO_OK) s = alloc_acts(ctx, false);
    if (s == OHAO_OK && (ctx->err_flag.alloc(4) != cudaSuccess || ctx->loss_acc.alloc(8) != cudaSuccess))
        s = OHAO_ERR_OOM;
    if (s == OHAO_OK) {
        // He-normal initialisation, zero biases
        std::vector<float> p(count_params(ctx));
        Rng rng(desc->seed);
        size_t off = 0;
        for (const Layer& l : ctx->L) {
            const double sd = std::sqrt(2.0 / (9.0 * l.s.cin));
            for (size_t i = 0; i < static_cast<size_t>(l.s.cout) * 9 * l.s.cin; ++i) p[off++] = float(rng.normal() * sd);
            for (int i = 0; i < l.s.cout; ++i) p[off++] = 0.0f;
        }
        s = upload_params(ctx, p.data());
    }
    if (s != OHAO_OK) {
        delete ctx;
        return s;
    }
    *out = ctx;
    return OHAO_OK;
}

void ohao_dn_destroy(ohao_dn_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    delete ctx;
}

const char* ohao_dn_last_error(const ohao_dn_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

ohao_status ohao_dn_wait_selftest(ohao_dn_ctx* ctx, uint32_t spin_limit, ohao_stream stream) {
    if (!ctx || spin_limit == 0 || spin_limit > (1u << 16)) return fail(ctx, OHAO_ERR_INVALID_ARG, "wait_selftest: limit");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    DN_CK(cudaSetDevice(ctx->device), "set device");
    DN_CK(launch_wait_probe(spin_limit, ctx->err_flag.as<int>(), st), "wait probe");
    return check_flag(ctx, st);
}

uint64_t ohao_dn_param_count(const ohao_dn_ctx* ctx) { return ctx ? count_params(ctx) : 0; }

ohao_status ohao_dn_get_params(ohao_dn_ctx* ctx, float* host, uint64_t n) {
    if (!ctx || !host || n != count_params(ctx)) return fail(ctx, OHAO_ERR_INVALID_ARG, "get_params: size");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    return download(ctx, false, host);
}

ohao_status ohao_dn_get_grads(ohao_dn_ctx* ctx, float* host, uint64_t n) {
    if (!ctx || !host || n != count_params(ctx)) return fail(ctx, OHAO_ERR_INVALID_ARG, "get_grads: size");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    return download(ctx, true, host);
}

ohao_status ohao_dn_set_params(ohao_dn_ctx* ctx, const float* host, uint64_t n) {
    if (!ctx || !host || n != count_params(ctx)) return fail(ctx, OHAO_ERR_INVALID_ARG, "set_params: size");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    ctx->adam_t = 0;
    for (Layer& l : ctx->L) {
        cudaMemset(l.mw.p, 0, l.mw.n);
        cudaMemset(l.vw.p, 0, l.vw.n);
        cudaMemset(l.mb.p, 0, l.mb.n);
        cudaMemset(l.vb.p, 0, l.vb.n);
    }
    return upload_params(ctx, host);
}

ohao_status ohao_dn_save(ohao_dn_ctx* ctx, const char* path) {
    if (!ctx || !path) return OHAO_ERR_INVALID_ARG;
    std::vector<float> p(count_params(ctx));
    ohao_status s = ohao_dn_get_params(ctx, p.data(), p.size());
    if (s != OHAO_OK) return s;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, OHAO_ERR_INVALID_ARG, std::string("save: cannot open ") + path);
    const char magic[8] = {'O', 'H', 'A', 'O', 'D', 'N', '0', '1'};
    const uint64_t n = p.size();
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(&n, 8, 1, f) == 1 &&
              std::fwrite(p.data(), 4, p.size(), f) == p.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? OHAO_OK : fail(ctx, OHAO_ERR_INVALID_ARG, "save: write failed");
}

ohao_status ohao_dn_load(ohao_dn_ctx* ctx, const char* path) {
    if (!ctx || !path) return OHAO_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(ctx, OHAO_ERR_INVALID_ARG, std::string("load: cannot open ") + path);
    char magic[8];
    uint64_t n = 0;
    std::vector<float> p(count_params(ctx));
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "OHAODN01", 8) == 0 &&
              std::fread(&n, 8, 1, f) == 1 && n == p.size() && std::fread(p.data(), 4, p.size(), f) == p.size();
    std::fclose(f);
    if (!ok) return fail(ctx, OHAO_ERR_INVALID_ARG, "load: not a parameter file of this network");
    return ohao_dn_set_params(ctx, p.data(), p.size());
}

ohao_status ohao_dn_infer(ohao_dn_ctx* ctx, const float* const* d_radiance, const float* const* d_aov,
                          uint32_t n_images, uint32_t width, uint32_t height, float* const* d_out,
                          ohao_stream stream) {
    if (!ctx || !d_radiance || !d_aov || !d_out || n_images == 0 || width == 0 || height == 0)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "infer: null argument");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Geo g0;
    ohao_status s = pack_inputs(ctx, d_radiance, d_aov, n_images, width, height, g0, st);
    if (s != OHAO_OK) return s;
    if ((s = forward(ctx, g0, st)) != OHAO_OK) return s;
    for (uint32_t i = 0; i < n_images; ++i) {
        if (!d_out[i]) return fail(ctx, OHAO_ERR_INVALID_ARG, "infer: null output image");
        launch_unpack(ctx->T[ctx->out_tensor].act.as<float>(), d_aov[i], d_out[i], static_cast<int>(width),
                      static_cast<int>(height), g0.w, static_cast<int64_t>(i) * g0.w * g0.h, st);
    }
    DN_CK(cudaGetLastError(), "infer launch");
    return check_flag(ctx, st);
}

ohao_status ohao_dn_train_step(ohao_dn_ctx* ctx, const float* const* d_radiance, const float* const* d_aov,
                               const float* const* d_target, uint32_t n_images, uint32_t width, uint32_t height,
                               float lr, float* loss, ohao_stream stream) {
    if (!ctx || !d_radiance || !d_aov || !d_target || n_images == 0)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "train_step: null argument");
    if (width % 16 || height % 16 || width == 0 || height == 0)
        return fail(ctx, OHAO_ERR_INVALID_ARG, "train_step: width and height must be multiples of 16");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    ohao_status s = alloc_acts(ctx, true);
    if (s != OHAO_OK) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Geo g0;
    if ((s = pack_inputs(ctx, d_radiance, d_aov, n_images, width, height, g0, st)) != OHAO_OK) return s;
    if ((s = forward(ctx, g0, st)) != OHAO_OK) return s;
    for (Tensor& t : ctx->T) DN_CK(cudaMemsetAsync(t.grad.p, 0, t.grad.n, st), "zero grads");
    for (Layer& l : ctx->L) {
        DN_CK(cudaMemsetAsync(l.gw.p, 0, l.gw.n, st), "zero grads");
        DN_CK(cudaMemsetAsync(l.gb.p, 0, l.gb.n, st), "zero grads");
    }
    DN_CK(cudaMemsetAsync(ctx->loss_acc.p, 0, 8, st), "zero loss");
    const float inv = 1.0f / static_cast<float>(static_cast<double>(n_images) * width * height * 3.0);
    Tensor& to = ctx->T[ctx->out_tensor];
    for (uint32_t i = 0; i < n_images; ++i) {
        if (!d_target[i]) return fail(ctx, OHAO_ERR_INVALID_ARG, "train_step: null target");
        launch_l1(to.act.as<float>(), d_target[i], d_aov[i], to.grad.as<float>(), static_cast<int>(width),
                  static_cast<int>(height), g0.w, static_cast<int64_t>(i) * g0.w * g0.h, inv,
                  ctx->loss_acc.as<double>(), st);
    }
    if ((s = backward(ctx, g0, st)) != OHAO_OK) return s;
    ctx->adam_t++;
    for (Layer& l : ctx->L)
        launch_adam(l.s, l.w32.as<float>(), l.gw.as<float>(), l.mw.as<float>(), l.vw.as<float>(),
                    l.w16.as<__nv_bfloat16>(), l.wt16.as<__nv_bfloat16>(), l.b32.as<float>(), l.gb.as<float>(),
                    l.mb.as<float>(), l.vb.as<float>(), lr, ctx->adam_t, st);
    DN_CK(cudaGetLastError(), "train launch");
    if ((s = check_flag(ctx, st)) != OHAO_OK) return s;
    double l = 0.0;
    DN_CK(cudaMemcpy(&l, ctx->loss_acc.p, 8, cudaMemcpyDeviceToHost), "loss");
    if (loss) *loss = static_cast<float>(l);
    return OHAO_OK;
}

ohao_status ohao_dn_tensor(ohao_dn_ctx* ctx, int32_t index, int32_t grad, float* host, uint64_t n,
                           uint32_t* channels, uint64_t* pixels) {
    if (!ctx || index < 0 || index >= static_cast<int32_t>(ctx->T.size()))
        return fail(ctx, OHAO_ERR_INVALID_ARG, "tensor: bad index");
    const Tensor& t = ctx->T[index];
    const Geo g = level_geo(ctx->g0, t.level);
    const uint64_t cnt = static_cast<uint64_t>(g.npix) * t.c8;
    if (channels) *channels = static_cast<uint32_t>(t.c8);
    if (pixels) *pixels = static_cast<uint64_t>(g.npix);
    if (!host) return OHAO_OK;
    if (n < cnt) return fail(ctx, OHAO_ERR_INVALID_ARG, "tensor: host buffer too small");
    DN_CK(cudaSetDevice(ctx->device), "set device");
    if (grad) {
        if (!t.grad.p) return fail(ctx, OHAO_ERR_INVALID_ARG, "tensor: no gradients before a train step");
        DN_CK(cudaMemcpy(host, t.grad.p, cnt * 4, cudaMemcpyDeviceToHost), "tensor");
    } else if (t.f32) {
        DN_CK(cudaMemcpy(host, t.act.p, cnt * 4, cudaMemcpyDeviceToHost), "tensor");
    } else {
        // channel-blocked [n][c8/8][h][w][8] on the device -> [pixel][c8]
        std::vector<uint16_t> b(cnt);
        DN_CK(cudaMemcpy(b.data(), t.act.p, cnt * 2, cudaMemcpyDeviceToHost), "tensor");
        const uint64_t hw = static_cast<uint64_t>(g.h) * g.w;
        const uint64_t cbs = static_cast<uint64_t>(t.c8) / 8;
        for (uint64_t i = 0; i < cnt; ++i) {
            const uint64_t lane = i & 7, rem = (i >> 3) % hw, nc = (i >> 3) / hw;
            const uint64_t n = nc / cbs, cb = nc % cbs;
            const uint32_t u = static_cast<uint32_t>(b[i]) << 16;
            std::memcpy(host + (n * hw + rem) * t.c8 + cb * 8 + lane, &u, 4);
        }
    }
    return OHAO_OK;
}

}  // extern "C"
