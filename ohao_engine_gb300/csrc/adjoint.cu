// adjoint.cu -- path-replay gradient of an image loss.
//
// Replaces the inverse lab's coordinate finite differences
// (ohao/inverse/staged_fit.hpp:316-332, ohao/inverse/diff_fit.hpp:177-200,
// which render the views twice per parameter) with one replay of the paths
// of the primal render. Each path is re-traced from its own RNG seed (pixel
// and sample index) and its radiance is differentiated with respect to
//   * the linear tile albedo map read through diffuse texture slot 0
//     (bilinear, ohao/render/diff/diff_map.hpp:40-67), and
//   * each material's roughness (matColors[3*id+1].x).
// The result estimates the derivative of the expected image. Each path keeps
// its primal decisions and directions; albedo factors, BRDF values and MIS
// weights are differentiated (pathwise part), and where the reference's
// estimator is not importance-weighted by the density it samples from, the
// score of that density is added: the roughness-scaled specular jitter, the
// lobe choice where its divisor is clamped or forced, and the
// Russian-roulette divisor where it exceeds the survival probability
// (p = maxc(T) > 1, which makes 1/p a value of the throughput). Per chain
//   R = sum_j T_j * G_j,   T_{j+1} = (T_j / p_j) * a_j,
// where G_j is the light added at vertex j (emission, light NEE, env NEE, or
// the environment seen by a ray that missed) and a_j the lobe factor. Each
// vertex's G_j, a_j and outgoing MIS pdf are evaluated with 4-wide forward
// duals over its local parameters (albedo r, g, b, roughness); a reverse
// sweep over a per-thread record of the chain's vertices carries
// lambda_j = d loss / d T_j and the suffix value that multiplies the scores.
// Nothing is stored between kernels: memory traffic is the replayed
// traversal plus the gradient scatter, which goes through a block-shared copy
// of the map.
#include "pt_path.cuh"

#include <algorithm>
#include <vector>

namespace ohao {

namespace {

// ---- 4-wide forward dual: slots 0-2 albedo r, g, b; slot 3 roughness ----
struct D4 {
    float v;
    float d[4];
};
__device__ __forceinline__ D4 dc(float v) { D4 r; r.v = v; r.d[0] = r.d[1] = r.d[2] = r.d[3] = 0.f; return r; }
__device__ __forceinline__ D4 dvar(float v, int i) { D4 r = dc(v); r.d[i] = 1.0f; return r; }
__device__ __forceinline__ D4 operator+(D4 a, D4 b) {
    D4 r; r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator*(D4 a, D4 b) {
    D4 r; r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ D4 operator/(D4 a, D4 b) {
    D4 r; r.v = a.v / b.v;
    const float inv = 1.0f / b.v;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
__device__ __forceinline__ D4 operator*(D4 a, float s) {
    D4 r; r.v = a.v * s;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] * s;
    return r;
}
__device__ __forceinline__ D4 operator+(D4 a, float s) { a.v = a.v + s; return a; }
__device__ __forceinline__ D4 operator-(float s, D4 a) {
    D4 r; r.v = s - a.v;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.d[i] = -a.d[i];
    return r;
}
__device__ __forceinline__ D4 dmax(D4 a, float b) { return a.v > b ? a : dc(b); }
__device__ __forceinline__ D4 dmax(D4 a, D4 b) { return a.v > b.v ? a : b; }

struct D3 {
    D4 x, y, z;
};
__device__ __forceinline__ D3 d3c(V3 v) { return D3{dc(v.x), dc(v.y), dc(v.z)}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, D4 s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 operator*(D3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 operator-(float s, D3 a) { return {s - a.x, s - a.y, s - a.z}; }
__device__ __forceinline__ D3 dmul(D3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ D4 dmaxc(D3 a) { return dmax(a.x, dmax(a.y, a.z)); }
__device__ __forceinline__ D3 dvmix(D3 a, D3 b, float t) { return a * (1.0f - t) + b * t; }

// Local parameters of a hit: the albedo after the map lookup and the
// roughness after max(param, 0.04) (pt_closesthit.rchit:104-150).
struct LocalMat {
    D3 alb;
    D4 rough;
    float metal;
};

// Where a vertex's gradient goes: texels of the map and a material slot.
struct Prov {
    float tu, tv;
    uint32_t matid;
    uint32_t flags;   // bit 0: albedo is base * map; bit 1: roughness above its floor
};

__device__ __forceinline__ void local_mat(const DScene& sc, const Surf& s, LocalMat& m, Prov& pv) {
    const float4 m0 = __ldg(sc.mats + s.matid * 3), m1 = __ldg(sc.mats + s.matid * 3 + 1);
    const bool mapped = __float_as_uint(m0.w) == 0u && sc.map_w > 0;
    // s.rough = max(param, 0.04) below 10: derivative 1 above the floor
    const bool live = m1.x > 0.04f && m1.x < 10.0f;
    m.alb = D3{dvar(s.albedo.x, 0), dvar(s.albedo.y, 1), dvar(s.albedo.z, 2)};
    m.rough = live ? dvar(s.rough, 3) : dc(s.rough);
    m.metal = s.metal;
    pv.tu = s.tu;
    pv.tv = s.tv;
    pv.matid = s.matid;
    pv.flags = (mapped ? 1u : 0u) | (live ? 2u : 0u);
}

// GGX D as a dual in roughness: isotropic (ggx_aniso.glsl:31-35 with pi_const,
// or the inline chain form), or the anisotropic lobe of ggx_aniso.glsl:37-55
// at the first hit.
__device__ D4 ggx_d(const PathParams& pp, const LocalMat& lm, V3 N, V3 H, float NdotH, float pi_const, bool bounce0) {
    if (bounce0 && pp.aniso >= 0.001f) {
        const V3 up = v3(0.0f, 1.0f, 0.0f);
        const V3 ref = fabsf(dot(up, N)) > 0.97f ? v3(1.0f, 0.0f, 0.0f) : up;
        const V3 T = normalize(ref - N * dot(ref, N));
        const V3 B = cross(N, T);
        float s, c;
        sincos_f(pp.aniso_rot, &s, &c);
        const V3 Tr = T * c + B * s;
        const V3 Br = B * c - T * s;
        const D4 r2 = lm.rough * lm.rough;
        const float aspect = sqrtf(1.0f - pp.aniso * 0.9f);
        const D4 rT = dmax(r2 / dc(aspect), 0.001f);
        const D4 rB = dmax(r2 * aspect, 0.001f);
        const float TdotH = dot(Tr, H), BdotH = dot(Br, H);
        const D4 dd = dc(TdotH * TdotH) / rT + dc(BdotH * BdotH) / rB + NdotH * NdotH;
        return dc(1.0f) / (rT * rB * (dd * dd) * 3.14159265f + 0.0001f);
    }
    const D4 a = lm.rough * lm.rough, a2 = a * a;
    const D4 denom = a2 * (NdotH * NdotH) + (1.0f - NdotH * NdotH);
    return a2 / ((denom * denom) * pi_const + 0.0001f);
}

struct BrdfD {
    D3 f;
    D4 D;
    float NdotH, VdotH;
};

// Cook-Torrance + Lambert of the NEE blocks (pt_raygen.rgen:392-415).
__device__ BrdfD brdf_d(const PathParams& pp, const LocalMat& lm, V3 N, V3 inDir, V3 L, float NdotL, bool bounce0,
                        float pi_chain, float pi_diff) {
    const V3 V = normalize(-inDir);
    const V3 H = normalize(L + V);
    BrdfD b;
    b.NdotH = gmaxf(dot(N, H), 0.001f);
    const float NdotV = gmaxf(dot(N, V), 0.001f);
    b.VdotH = gmaxf(dot(V, H), 0.001f);
    b.D = ggx_d(pp, lm, N, H, b.NdotH, bounce0 ? 3.14159265f : pi_chain, bounce0);
    const D3 F0 = dvmix(d3c(v3s(0.04f)), lm.alb, lm.metal);
    const D3 F = F0 + (1.0f - F0) * pow5f(1.0f - b.VdotH);
    const D4 k = (lm.rough + 1.0f) * (lm.rough + 1.0f) * 0.125f;
    const D4 G = (dc(NdotL) / ((1.0f - k) * NdotL + k)) * (dc(NdotV) / ((1.0f - k) * NdotV + k));
    const D3 spec = (F * (b.D * G)) * (1.0f / (4.0f * NdotV * NdotL + 0.001f));
    const D3 diff = ((1.0f - F) * (1.0f - lm.metal) * lm.alb) * (1.0f / pi_diff);
    b.f = diff + spec;
    return b;
}

// selection probability of the specular lobe (pt_raygen.rgen:775-779)
__device__ D4 spec_prob(const LocalMat& lm, V3 inDir, V3 N) {
    const float cosI = fabsf(dot(normalize(inDir), N));
    const D3 F0 = dvmix(d3c(v3s(0.04f)), lm.alb, lm.metal);
    const D3 fres = F0 + (1.0f - F0) * pow5f(1.0f - cosI);
    const D4 sp = dmaxc(fres) * (1.0f - lm.rough * 0.9f);
    return sp * (1.0f - lm.metal) + lm.metal;
}

// GGX half-vector pdf of a sampled specular direction (pt_raygen.rgen:531-540, 803-810)
__device__ D4 spec_pdf(const PathParams& pp, const LocalMat& lm, V3 N, V3 inDir, V3 outDir, bool bounce0) {
    const V3 Hs = normalize(-inDir + outDir);
    const float NdotHs = gmaxf(dot(N, Hs), 0.001f);
    const float VdotHs = gmaxf(dot(-inDir, Hs), 0.001f);
    const D4 Ds = ggx_d(pp, lm, N, Hs, NdotHs, kPI, bounce0);
    return (Ds * NdotHs) * (1.0f / (4.0f * VdotHs + 1e-4f));
}

// Traversal entry points of the adjoint. It traces from several places (the
// primary hit, two replayed chains, light and environment shadow rays);
// inlined at each, the kernel's code outgrew the instruction cache (warps
// mostly stalled on instruction fetch). Out of line there is one copy of each
// traversal, behind an interface of a few registers.
struct AdjHit {
    Hit h;
    int err;
};
__device__ __noinline__ AdjHit adj_closest(const DScene* sc, V3 o, V3 d) {
    TravCount tc{0, 0};
    int e = 0;
    const Hit h = scene_closest<false>(*sc, o, d, 0.001f, 10000.0f, tc, e);
    return AdjHit{h, e};
}
// bit 0: occluded, bit 1: traversal error
__device__ __noinline__ int adj_occluded(const DScene* sc, V3 o, V3 d, float tmax) {
    TravCount tc{0, 0};
    int e = 0;
    const bool occ = scene_occluded<false>(*sc, o, d, 0.001f, tmax, tc, e);
    return (occ ? 1 : 0) | (e ? 2 : 0);
}

// Light NEE and env NEE at a vertex (primal draws and visibility, dual
// values), without throughput.
__device__ D3 nee_d(const DScene& sc, const PathParams& pp, Rng& rng, uint32_t& dim, const Surf& s, V3 inDir,
                    const LocalMat& lm, bool bounce0, int& err) {
    D3 g = d3c(v3s(0.0f));
    const V3 org = s.pos + s.N * 0.01f;
    if (sc.nlights > 0) {
        const LightSample ls = sample_light(sc, rng, dim, s.pos, s.N);
        const int oc = ls.valid ? adj_occluded(&sc, org, ls.L, ls.shadowDist) : 1;
        if (oc & 2) err = 1;
        if (!(oc & 1)) {
            const BrdfD b = brdf_d(pp, lm, s.N, inDir, ls.L, ls.NdotL, bounce0, 3.14159f, 3.14159f);
            g = g + dmul(b.f, ls.Le) * (ls.NdotL * ls.weight * ls.n);
        }
    }
    if (sc.has_cdf) {
        const EnvSample es = sample_env_nee(sc, pp, rng, dim, s.N);
        const int oc = es.valid ? adj_occluded(&sc, org, es.dir, 10000.0f) : 1;
        if (oc & 2) err = 1;
        if (!(oc & 1)) {
            const BrdfD b = brdf_d(pp, lm, s.N, inDir, es.dir, es.NdotL, bounce0, kPI, kPI);
            const D4 sp = spec_prob(lm, inDir, s.N);
            const D4 pdfS = (b.D * b.NdotH) * (1.0f / (4.0f * b.VdotH + 1e-4f));
            const D4 bsdfPdf = (1.0f - sp) * (es.NdotL / kPI) + pdfS * sp;
            const D4 w = dc(es.pdf) / dmax(bsdfPdf + es.pdf, 1e-6f);
            g = g + dmul(b.f, es.rad) * (w * (es.NdotL / es.pdf));
        }
    }
    return g;
}

constexpr uint32_t kSharedRough = 64;

struct Sink {
    float* map;          // block-shared (or global) d loss / d map texel; null = not wanted
    float* rough_s;      // block-shared, materials < kSharedRough
    float* rough_g;      // global, all materials; null = not wanted
    const float4* mats;
    uint32_t map_w, map_h;
};

// d loss / d (albedo r, g, b, roughness) of one vertex -> map texels and
// the material's roughness.
__device__ void scatter(const Sink& sk, const Prov& pv, const float dl[4]) {
    if ((pv.flags & 1u) && sk.map && (dl[0] != 0.0f || dl[1] != 0.0f || dl[2] != 0.0f)) {
        const float4 m0 = __ldg(sk.mats + pv.matid * 3);
        const int w = static_cast<int>(sk.map_w), h = static_cast<int>(sk.map_h);
        const float u = gclampf(pv.tu, 0.0f, 1.0f), v = gclampf(pv.tv, 0.0f, 1.0f);
        const float x = u * static_cast<float>(w - 1), y = v * static_cast<float>(h - 1);
        const int x0 = static_cast<int>(x), y0 = static_cast<int>(y);
        const int x1 = min(x0 + 1, w - 1), y1 = min(y0 + 1, h - 1);
        const float tx = x - static_cast<float>(x0), ty = y - static_cast<float>(y0);
        const float wt[4] = {(1.0f - tx) * (1.0f - ty), tx * (1.0f - ty), (1.0f - tx) * ty, tx * ty};
        const int idx[4] = {y0 * w + x0, y0 * w + x1, y1 * w + x0, y1 * w + x1};
        // d albedo_c / d map_c(texel) = base_c * bilinear weight
        const float gb[3] = {dl[0] * m0.x, dl[1] * m0.y, dl[2] * m0.z};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (wt[q] == 0.0f) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (gb[c] != 0.0f) atomicAdd(sk.map + idx[q] * 3 + c, gb[c] * wt[q]);
        }
    }
    if ((pv.flags & 2u) && sk.rough_g && dl[3] != 0.0f) {
        if (pv.matid < kSharedRough) atomicAdd(sk.rough_s + pv.matid, dl[3]);
        else atomicAdd(sk.rough_g + pv.matid, dl[3]);
    }
}

constexpr int kMaxRec = 16;   // vertices per chain = max_bounces (validated on the host)

// One chain vertex; the lobe factor a_c depends on albedo_c alone, so its
// derivative is one number per channel.
struct VRec {
    float T[3];     // throughput arriving at the vertex
    float G[3];     // light added at the vertex (value)
    float a[3];     // lobe factor (value)
    float da;       // d a_c / d albedo_c (the same for all channels)
    float dl[4];    // d loss / d local parameters
    float S[4];     // d log (probability of this vertex's sampling decisions) / d local parameters
    float invp;     // 1 / Russian-roulette divisor applied here
    int has_a;
    int cmax;       // >= 0: the divisor is maxc(T) > 1, a value of the throughput (channel of the max)
    Prov pv;
};

// Score of the reference's specular jitter (pt_raygen.rgen:516-525): the
// direction w = normalize(R + r h), h cosine-distributed around R, has the
// solid-angle density q(w | r) = (s c - 1) s^2 / (pi r^2 sqrt(c^2 - 1 + r^2))
// with c = w.R and s = c + sqrt(c^2 - 1 + r^2). Its derivative in r at fixed
// w, written with t = h.R, is
//   d log q / d r = (1 - t^2) / (t (t + r)^2) + 2 / (t + r) - 2 / r.
// The sampling weight of the lobe does not contain q, so the expectation
// depends on r through it; the derivative of the expectation adds
// (radiance after the sample) * this score (score-function estimator on the
// jittered direction, also when the fallback direction replaced it).
__device__ __forceinline__ float jitter_score(V3 refl, V3 h, float rough) {
    const double t = fmax(static_cast<double>(dot(h, refl)), 1e-12);
    const double r = rough;
    const double tr = t + r;
    return static_cast<float>((1.0 - t * t) / (t * tr * tr) + 2.0 / tr - 2.0 / r);
}

// spec_dir with the jitter score; same draws and same result.
__device__ V3 spec_dir_score(Rng& rng, uint32_t& dim, V3 inDir, V3 N, float rough, float& score) {
    V3 refl = reflect(inDir, N);
    score = 0.0f;
    if (rough > 0.01f) {
        const float j0 = rng.s1(dim), j1 = rng.s1(dim + 1);
        dim += 2;
        const V3 h = cos_hemi(refl, j0, j1);
        score = jitter_score(refl, h, rough);
        const V3 jit = h * rough;
        refl = normalize(refl + jit);
        if (dot(refl, N) < 0.0f) {
            const float f0 = rng.s1(dim), f1 = rng.s1(dim + 1);
            dim += 2;
            refl = cos_hemi(N, f0, f1);
        }
    }
    return refl;
}

// lambda[c] * d g_c / d theta, accumulated
__device__ __forceinline__ void add_lam(float dl[4], const float lam[3], const D3& g) {
#pragma unroll
    for (int i = 0; i < 4; ++i) dl[i] += lam[0] * g.x.d[i] + lam[1] * g.y.d[i] + lam[2] * g.z.d[i];
}

__device__ __forceinline__ void add_dl(float dl[4], const float delta[3], const float T[3], const D3& g) {
#pragma unroll
    for (int i = 0; i < 4; ++i) dl[i] += delta[0] * T[0] * g.x.d[i] + delta[1] * T[1] * g.y.d[i] + delta[2] * T[2] * g.z.d[i];
}

struct ChainOut {
    float lam[3];   // d loss / d (throughput at the chain's first vertex)
    float value;    // the chain's contribution to the loss's linearisation, sum_k delta . (T_k G_k)
};

// Replays one chain (stage B when specChain, stage C otherwise) from its
// first outgoing ray and accumulates the gradients of its vertices. prev_dl
// is the gradient slot of the vertex the chain leaves from, which owns
// lastPdf. Reverse sweep with lambda_j = d loss / d T_j:
//   lambda_j = delta G_j + J_j^T (a_j * lambda_{j+1}),
// J_j = d (T_j / p_j) / d T_j: diagonal 1/p_j while the Russian-roulette
// divisor is the survival probability (p_j <= 1), plus the rank-one term of
// p_j = maxc(T_j) when p_j > 1 (the divisor is then a value, not a
// probability).
__device__ ChainOut replay_chain(const DScene& sc, const PathParams& pp, Rng& rng, uint32_t& dim, bool specChain, V3 ro,
                                 V3 rd, V3 thr, D4 lastPdf, bool lastDelta, const float delta[3], float* prev_dl,
                                 VRec* rec, const Sink& sk, int& err) {
    int nrec = 0;
    float* last_dl = prev_dl;
    for (uint32_t bounce = 1; bounce <= pp.max_bounces && nrec < kMaxRec; ++bounce) {
        const AdjHit ah = adj_closest(&sc, ro, rd);
        if (ah.err) err = 1;
        const Hit h = ah.h;
        VRec& R = rec[nrec];
        R.T[0] = thr.x; R.T[1] = thr.y; R.T[2] = thr.z;
        R.has_a = 0;
        R.cmax = -1;
        R.invp = 1.0f;
        R.dl[0] = R.dl[1] = R.dl[2] = R.dl[3] = 0.0f;
        R.S[0] = R.S[1] = R.S[2] = R.S[3] = 0.0f;
        R.pv.flags = 0;
        if (h.prim == 0xFFFFFFFFu) {
            Surf ms;
            miss_shade(sc, pp, rd, ms);
            D4 w = dc(1.0f);
            if (ms.env_pdf > 0.0f && sc.has_cdf && !lastDelta) w = lastPdf / dmax(lastPdf + ms.env_pdf, 1e-6f);
            const D3 gM = d3c(ms.color) * w;   // the MIS weight belongs to the previous vertex
            add_dl(last_dl, delta, R.T, gM);
            R.G[0] = gM.x.v; R.G[1] = gM.y.v; R.G[2] = gM.z.v;
            nrec++;
            break;
        }
        Surf s;
        hit_shade<false>(sc, ro, rd, h, s);
        LocalMat lm;
        local_mat(sc, s, lm, R.pv);
        D3 G = d3c(length(s.color) > 0.001f ? s.color : v3s(0.0f));
        G = G + nee_d(sc, pp, rng, dim, s, rd, lm, false, err);
        add_dl(R.dl, delta, R.T, G);
        R.G[0] = G.x.v; R.G[1] = G.y.v; R.G[2] = G.z.v;
        nrec++;
        last_dl = R.dl;
        if (bounce > 1) {   // Russian roulette (survival probability min(p, 1), divisor p)
            const float p = maxc(thr);
            const float rr = rng.s1(dim);
            dim += 1;
            if (p < 0.01f || rr > p) break;
            if (p > 1.0f) R.cmax = (thr.x >= thr.y && thr.x >= thr.z) ? 0 : (thr.y >= thr.z ? 1 : 2);
            thr = thr / p;
            R.invp = 1.0f / p;
        }
        const float bR = s.rough, bM = s.metal;
        const V3 bF0 = vmix(v3s(0.04f), s.albedo, bM);
        const float cosI = fabsf(dot(normalize(rd), s.N));
        const V3 fres = bF0 + (1.0f - bF0) * pow5f(1.0f - cosI);
        float sp = maxc(fres);
        sp = sp * (1.0f - bR * 0.9f);
        sp = gmixf(sp, 1.0f, bM);
        const float choice = rng.s1(dim);
        dim += 1;
        const D4 spd = spec_prob(lm, rd, s.N);
        float fa, fb;   // a_c = fa * albedo_c + fb
        // Lobe choice: probability P_b, divisor max(P, 0.01). Where they differ
        // (clamped divisor, or the specular lobe forced below roughness 0.05)
        // the expectation keeps d log P_b - d log div_b as a score.
        if (bR < 0.05f) {
            if (sp > 0.01f)
#pragma unroll
                for (int i = 0; i < 4; ++i) R.S[i] -= spd.d[i] / spd.v;
        } else if (choice < sp) {
            if (sp < 0.01f)
#pragma unroll
                for (int i = 0; i < 4; ++i) R.S[i] += spd.d[i] / spd.v;
        } else if (1.0f - sp < 0.01f) {
#pragma unroll
            for (int i = 0; i < 4; ++i) R.S[i] -= spd.d[i] / (1.0f - spd.v);
        }
        if (choice < sp || bR < 0.05f) {
            const V3 inDir = rd;
            float js;
            rd = spec_dir_score(rng, dim, rd, s.N, bR, js);
            if (R.pv.flags & 2u) R.S[3] += js;
            ro = s.pos + s.N * 0.01f;
            const float div = gmaxf(sp, 0.01f);
            if (specChain) {
                thr = thr * vmix(v3s(1.0f), s.albedo, bM);
                fa = bM / div;
                fb = (1.0f - bM) / div;
            } else {
                thr = thr * (s.albedo * (1.0f - bM));
                fa = (1.0f - bM) / div;
                fb = 0.0f;
            }
            thr = thr / div;
            if (bR < 0.05f) {
                lastPdf = dc(1.0f);
                lastDelta = true;
            } else {
                lastPdf = spd * spec_pdf(pp, lm, s.N, inDir, rd, false);
                lastDelta = false;
            }
        } else {
            const float d0 = rng.s1(dim), d1 = rng.s1(dim + 1);
            dim += 2;
            rd = cos_hemi(s.N, d0, d1);
            ro = s.pos + s.N * 0.01f;
            const float div = gmaxf(1.0f - sp, 0.01f);
            thr = thr * s.albedo;
            thr = thr / div;
            fa = 1.0f / div;
            fb = 0.0f;
            lastPdf = (1.0f - spd) * (gmaxf(dot(rd, s.N), 0.0f) / kPI);
            lastDelta = false;
        }
        R.has_a = 1;
        R.a[0] = fa * s.albedo.x + fb;
        R.a[1] = fa * s.albedo.y + fb;
        R.a[2] = fa * s.albedo.z + fb;
        R.da = fa;
    }
    // reverse sweep over lambda (d loss / d T) and the suffix value V
    ChainOut out;
    float lam[3] = {0.f, 0.f, 0.f};
    float V = 0.0f;
    for (int j = nrec - 1; j >= 0; --j) {
        VRec& R = rec[j];
        float nl[3] = {0.f, 0.f, 0.f};
        if (R.has_a) {
            float mu[3];   // d loss / d (T_j / p_j)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                mu[c] = R.a[c] * lam[c];
                R.dl[c] += R.T[c] * R.invp * lam[c] * R.da;   // through a_c(albedo_c)
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) R.dl[i] += V * R.S[i];   // sampling scores times what follows
#pragma unroll
            for (int c = 0; c < 3; ++c) nl[c] = mu[c] * R.invp;
            if (R.cmax >= 0) {
                const float tm = R.T[0] * mu[0] + R.T[1] * mu[1] + R.T[2] * mu[2];
                nl[R.cmax] -= tm * R.invp * R.invp;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            nl[c] += delta[c] * R.G[c];
            V += delta[c] * R.T[c] * R.G[c];
            lam[c] = nl[c];
        }
    }
    for (int j = 0; j < nrec; ++j) scatter(sk, rec[j].pv, rec[j].dl);
    out.lam[0] = lam[0]; out.lam[1] = lam[1]; out.lam[2] = lam[2];
    out.value = V;
    return out;
}

struct AdjParams {
    PathParams pp;
    uint32_t spp;
    uint32_t nviews;
    uint32_t total_pix;
    uint32_t map_w, map_h;
    uint32_t nmats;
    float inv_spp;
};

struct AdjView {
    ViewParams vp;
    const float4* grad;   // d loss / d pixel (RGB)
    uint32_t pix_begin;
    uint32_t pad;
};

// One thread per path (global pixel, sample), grid-stride.
template <bool kSharedMap>
__global__ void __launch_bounds__(128) k_adjoint(const __grid_constant__ DScene sc, AdjParams ap,
                                                 const AdjView* __restrict__ views,
                                                 float* __restrict__ grad_map, float* __restrict__ grad_rough,
                                                 int* err_flag) {
    extern __shared__ float smem[];
    const uint32_t map_n = ap.map_w * ap.map_h * 3;
    float* s_rough = smem;
    float* s_map = smem + kSharedRough;
    for (uint32_t i = threadIdx.x; i < kSharedRough; i += blockDim.x) s_rough[i] = 0.0f;
    if (kSharedMap)
        for (uint32_t i = threadIdx.x; i < map_n; i += blockDim.x) s_map[i] = 0.0f;
    __syncthreads();
    const Sink sk{kSharedMap ? s_map : grad_map, s_rough, grad_rough, sc.mats, ap.map_w, ap.map_h};
    const PathParams& pp = ap.pp;
    const uint64_t total = static_cast<uint64_t>(ap.total_pix) * ap.spp;
    int err = 0;
    VRec rec[kMaxRec];
    for (uint64_t lin = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; lin < total;
         lin += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t g = static_cast<uint32_t>(lin / ap.spp), k = static_cast<uint32_t>(lin % ap.spp);
        uint32_t lo = 0, hi = ap.nviews - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (views[mid].pix_begin <= g) lo = mid; else hi = mid - 1;
        }
        const AdjView& av = views[lo];
        const uint32_t pix = g - av.pix_begin;
        const float4 gp = av.grad[pix];
        const float delta[3] = {gp.x * ap.inv_spp, gp.y * ap.inv_spp, gp.z * ap.inv_spp};
        if (delta[0] == 0.0f && delta[1] == 0.0f && delta[2] == 0.0f) continue;
        const ViewParams& vp = av.vp;
        const uint32_t px = pix % vp.width, py = pix / vp.width, sidx = pp.sample_base + k;
        PathState ps;
        path_start(vp, pp, px, py, sidx, ps);
        Rng rng = make_rng(pp, px, py, sidx, ps.rng);
        uint32_t dim = ps.dim;
        const AdjHit ah = adj_closest(&sc, ps.ro, ps.rd);
        if (ah.err) err = 1;
        const Hit h = ah.h;
        if (h.prim == 0xFFFFFFFFu) continue;   // primary miss: no parameter dependence
        Surf s0;
        hit_shade<false>(sc, ps.ro, ps.rd, h, s0);
        LocalMat m0;
        Prov p0;
        local_mat(sc, s0, m0, p0);
        const V3 rayDir = ps.rd;
        const float one[3] = {1.0f, 1.0f, 1.0f};
        float dl0[4] = {0.f, 0.f, 0.f, 0.f};
        // stage A: light NEE and env NEE at throughput 1
        add_dl(dl0, delta, one, nee_d(sc, pp, rng, dim, s0, rayDir, m0, true, err));
        // stage B (specular chain) then stage C (diffuse chain) from vertex 0,
        // through one copy of the replay (a loop, not unrolled: inlined twice
        // the kernel's code outgrows the instruction cache)
        const D3 tB = dvmix(d3c(v3s(1.0f)), m0.alb, s0.metal);
#pragma unroll 1
        for (int chain = 0; chain < 2; ++chain) {
            const bool spec = chain == 0;
            V3 dir, thr0;
            D4 pdf0;
            bool delta0 = false;
            float js0 = 0.0f;
            if (spec) {
                dir = spec_dir_score(rng, dim, rayDir, s0.N, s0.rough, js0);
                delta0 = s0.rough < 0.05f;
                pdf0 = delta0 ? dc(1.0f) : spec_pdf(pp, m0, s0.N, rayDir, dir, true);
                thr0 = vmix(v3s(1.0f), s0.albedo, s0.metal);
            } else {
                const float d0 = rng.s1(dim), d1 = rng.s1(dim + 1);
                dim += 2;
                dir = cos_hemi(s0.N, d0, d1);
                pdf0 = dc(gmaxf(dot(dir, s0.N), 0.0f) / kPI);
                thr0 = s0.albedo;
            }
            const ChainOut co = replay_chain(sc, pp, rng, dim, spec, s0.pos + s0.N * 0.01f, dir, thr0, pdf0, delta0,
                                             delta, dl0, rec, sk, err);
            add_lam(dl0, co.lam, spec ? tB : m0.alb);
            if (spec && (p0.flags & 2u)) dl0[3] += co.value * js0;
        }
        scatter(sk, p0, dl0);
    }
    __syncthreads();
    if (kSharedMap)
        for (uint32_t i = threadIdx.x; i < map_n; i += blockDim.x)
            if (s_map[i] != 0.0f) atomicAdd(grad_map + i, s_map[i]);
    if (grad_rough)
        for (uint32_t i = threadIdx.x; i < min(ap.nmats, kSharedRough); i += blockDim.x)
            if (s_rough[i] != 0.0f) atomicAdd(grad_rough + i, s_rough[i]);
    if (err) atomicOr(err_flag, 1);
}

// Per-view MSE over RGB and its gradient: loss += scale * sum (I - T)^2,
// grad = 2 scale (I - T), scale = 1 / (n_views * npix * 3).
// Display transform of the reference, D(x) = pow(ACES(x / 2), 1/2.2)
// (pt_raygen.rgen:99-102, 1263-1264), in float before the 8-bit rounding,
// and its derivative (zero where ACES clamps).
__device__ __forceinline__ void display_and_slope(float x, float& d, float& slope) {
    const float u = 0.5f * x;
    const float num = u * (2.51f * u + 0.03f), den = u * (2.43f * u + 0.59f) + 0.14f;
    const float a = num / den;
    if (!(a > 0.0f)) { d = 0.0f; slope = 0.0f; return; }
    if (a >= 1.0f) { d = 1.0f; slope = 0.0f; return; }
    d = powf(a, 1.0f / 2.2f);
    const float da_du = ((5.02f * u + 0.03f) * den - num * (4.86f * u + 0.59f)) / (den * den);
    slope = (1.0f / 2.2f) * (d / a) * da_du * 0.5f;
}

// Per-pixel loss gradient and loss sum of one view. Linear: RGB squared error
// of the radiance against the target radiance. Display (ldr): RGB squared
// error of D(radiance) against the target's display values in [0, 1] (an
// RGBA8 target / 255), the mseRGB of the reference's inverse lab.
__global__ void k_mse_grad(const float4* __restrict__ img, const float4* __restrict__ target, uint32_t npix,
                           float scale, int ldr, float4* __restrict__ grad, double* __restrict__ loss_sum) {
    double part = 0.0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const float4 a = img[p], t = target[p];
        float ex, ey, ez;
        float4 g;
        if (ldr) {
            float dx, dy, dz, sx, sy, sz;
            display_and_slope(a.x, dx, sx);
            display_and_slope(a.y, dy, sy);
            display_and_slope(a.z, dz, sz);
            ex = dx - t.x; ey = dy - t.y; ez = dz - t.z;
            g = make_float4(2.0f * scale * ex * sx, 2.0f * scale * ey * sy, 2.0f * scale * ez * sz, 0.0f);
        } else {
            ex = a.x - t.x; ey = a.y - t.y; ez = a.z - t.z;
            g = make_float4(2.0f * scale * ex, 2.0f * scale * ey, 2.0f * scale * ez, 0.0f);
        }
        part += static_cast<double>(ex) * ex + static_cast<double>(ey) * ey + static_cast<double>(ez) * ez;
        grad[p] = g;
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xFFFFFFFFu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, part * static_cast<double>(scale));
}

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

uint32_t adjoint_max_bounces() { return static_cast<uint32_t>(kMaxRec); }

size_t adjoint_scratch_bytes(uint32_t nviews) { return round256(nviews * sizeof(AdjView)) + 256; }

ohao_status adjoint_mse(const RenderView* views, const float* const* targets, uint32_t nviews, bool ldr, void* scratch,
                        size_t scratch_bytes, float* const* grads_out, float* loss_out, cudaStream_t st,
                        std::string& err) {
    if (scratch_bytes < adjoint_scratch_bytes(nviews)) {
        err = "loss: scratch too small";
        return OHAO_ERR_INVALID_ARG;
    }
    double* dloss = reinterpret_cast<double*>(static_cast<char*>(scratch) + round256(nviews * sizeof(AdjView)));
    if (cudaMemsetAsync(dloss, 0, sizeof(double), st) != cudaSuccess) {
        err = "loss: memset failed";
        return OHAO_ERR_CUDA;
    }
    for (uint32_t v = 0; v < nviews; ++v) {
        const uint32_t npix = views[v].vp.width * views[v].vp.height;
        const float scale = static_cast<float>(1.0 / (static_cast<double>(nviews) * npix * 3.0));
        k_mse_grad<<<std::max(1u, std::min(1024u, (npix + 255) / 256)), 256, 0, st>>>(
            reinterpret_cast<const float4*>(views[v].accum), reinterpret_cast<const float4*>(targets[v]), npix, scale,
            ldr ? 1 : 0, reinterpret_cast<float4*>(grads_out[v]), dloss);
    }
    double lsum = 0.0;
    cudaMemcpyAsync(&lsum, dloss, sizeof(double), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("loss: ") + cudaGetErrorString(e);
        return OHAO_ERR_CUDA;
    }
    if (loss_out) *loss_out = static_cast<float>(lsum);
    return OHAO_OK;
}

ohao_status adjoint_backward(const DScene& sc, const RenderView* views, const float* const* grads, uint32_t nviews,
                             const PathParams& pp, uint32_t spp, uint32_t nmats, void* scratch, size_t scratch_bytes,
                             float* grad_map, float* grad_rough, cudaStream_t st, int* d_err, std::string& err) {
    uint64_t total = 0;
    for (uint32_t v = 0; v < nviews; ++v) total += static_cast<uint64_t>(views[v].vp.width) * views[v].vp.height;
    if (total >= (1ull << 32) || total * spp >= (1ull << 40)) {
        err = "backward: too many paths";
        return OHAO_ERR_INVALID_ARG;
    }
    if (pp.max_bounces > static_cast<uint32_t>(kMaxRec)) {
        err = "backward: max_bounces above 16";
        return OHAO_ERR_INVALID_ARG;
    }
    if (scratch_bytes < adjoint_scratch_bytes(nviews)) {
        err = "backward: scratch too small";
        return OHAO_ERR_INVALID_ARG;
    }
    AdjView* dviews = static_cast<AdjView*>(scratch);
    std::vector<AdjView> hv(nviews);
    uint32_t off = 0;
    for (uint32_t v = 0; v < nviews; ++v) {
        hv[v].vp = views[v].vp;
        hv[v].grad = reinterpret_cast<const float4*>(grads[v]);
        hv[v].pix_begin = off;
        hv[v].pad = 0;
        off += views[v].vp.width * views[v].vp.height;
    }
    const uint32_t mw = grad_map ? sc.map_w : 0u, mh = grad_map ? sc.map_h : 0u;
    const size_t map_n = static_cast<size_t>(mw) * mh * 3;
    if (map_n) cudaMemsetAsync(grad_map, 0, map_n * sizeof(float), st);
    if (grad_rough && nmats) cudaMemsetAsync(grad_rough, 0, nmats * sizeof(float), st);
    cudaMemcpyAsync(dviews, hv.data(), nviews * sizeof(AdjView), cudaMemcpyHostToDevice, st);
    const AdjParams ap{pp, spp, nviews, static_cast<uint32_t>(total), mw, mh, nmats, 1.0f / static_cast<float>(spp)};
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem_shared = kSharedRough * sizeof(float) + map_n * sizeof(float);
    const bool shared_map = map_n > 0 && smem_shared <= 96 * 1024;
    const uint64_t paths = total * spp;
    // One traversal for both scene kinds (decided per ray at run time): the
    // scene-kind-specialised kernels measured slower, their larger inlined
    // code costing more in instruction fetch than the branch saves. Grid:
    // 32 blocks per SM over a grid-stride path loop, enough small blocks for
    // the uneven path lengths to balance across SMs.
    float* gm = map_n ? grad_map : nullptr;
    auto fn = shared_map ? k_adjoint<true> : k_adjoint<false>;
    const size_t smem = shared_map ? smem_shared : kSharedRough * sizeof(float);
    if (shared_map) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    const unsigned grid = static_cast<unsigned>(
        std::max<uint64_t>(1, std::min<uint64_t>((paths + 127) / 128, static_cast<uint64_t>(sms) * 32)));
    fn<<<grid, 128, smem, st>>>(sc, ap, dviews, gm, grad_rough, d_err);
    const cudaError_t e = cudaStreamSynchronize(st);   // also keeps hv alive until the copy has read it
    if (e != cudaSuccess) {
        err = std::string("backward: ") + cudaGetErrorString(e);
        return OHAO_ERR_CUDA;
    }
    return OHAO_OK;
}

}  // namespace ohao
