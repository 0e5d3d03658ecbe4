// oracle_bvh.hpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// Host restatement of the acceleration structure that replaces the Vulkan
// driver's BLAS/TLAS build (rt_acceleration_structure.cpp:205-300, 419-530)
// and the traversal behind traceRayEXT (pt_raygen.rgen:197,389,550,857).
// The reference delegates both to the closed driver, so this file defines the
// algorithm the CUDA builder must reproduce bit-for-bit:
//   1. 30-bit Morton code of each primitive-box centroid in the centroid
//      bounds (10 bits per axis, x in the most significant slot);
//   2. stable sort of (code, build index);
//   3. Karras (HPG 2012) binary radix tree, ties broken by index;
//   4. bottom-up box union and half-area;
//   5. greedy collapse to 8-wide: starting from a node's two children, the
//      internal child with the largest half-area (smallest id on ties) is
//      replaced by its two children until 8 slots are used or none is left;
//      members covering <= 3 primitives become leaf slots;
//   6. layout: a node's internal children are contiguous, followed by their
//      subtrees in slot order; leaf primitives of a node are contiguous;
//   7. child boxes quantized to 8 bits per side on a per-axis power-of-two
//      grid anchored at the node's lower corner, rounded outward; unused
//      slots hold the inverted box (lo 255, hi 0) and meta 0.
// Closest hit: smallest t in (tmin, tmax) by the watertight ray/triangle test
// of Woop, Benthin and Wald (JCGT 2013); equal t resolves to the smallest
// (instance, primitive) pair, so the answer does not depend on traversal
// order. Parity of this layer is unpinned by the reference (driver-defined);
// it is pinned against brute force over all triangles.
#pragma once
#include "oracle_math.hpp"
#include <vector>
#include <algorithm>
#include <numeric>
#include <cstdint>
#include <cmath>

namespace orc {

struct Box {
    float lo[3], hi[3];
};
inline Box box_empty() { return Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}}; }
inline Box box_union(const Box& a, const Box& b) {
    Box r;
    for (int k = 0; k < 3; ++k) { r.lo[k] = std::min(a.lo[k], b.lo[k]); r.hi[k] = std::max(a.hi[k], b.hi[k]); }
    return r;
}
inline float half_area(const Box& b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// 80-byte wide node; byte layout identical to ohao_bvh8_node in include/ohao_pt.h.
struct WideNode {
    float origin[3];
    int8_t exps[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "wide node is 80 bytes");

inline uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

struct BinaryTree {
    uint32_t n = 0;                  // primitives
    std::vector<uint32_t> order;     // sorted position -> build index
    std::vector<uint32_t> codes;     // sorted codes
    std::vector<uint32_t> left, right, first, last;  // per internal node
    std::vector<Box> box;            // internal [0,n-1) then leaves [n-1, 2n-1)
    std::vector<float> sa;
};

inline int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }

inline void morton_codes(const std::vector<Box>& prims, std::vector<uint32_t>& codes) {
    const size_t n = prims.size();
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<float> cen(n * 3);
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            float c = (prims[i].lo[k] + prims[i].hi[k]) * 0.5f;
            cen[i * 3 + k] = c;
            cmin[k] = std::min(cmin[k], c);
            cmax[k] = std::max(cmax[k], c);
        }
    float scale[3];
    for (int k = 0; k < 3; ++k) {
        float ext = cmax[k] - cmin[k];
        scale[k] = ext > 0.0f ? 1024.0f / ext : 0.0f;
    }
    codes.resize(n);
    for (size_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            float f = (cen[i * 3 + k] - cmin[k]) * scale[k];
            f = std::min(std::max(f, 0.0f), 1023.0f);
            q[k] = static_cast<uint32_t>(f);
        }
        codes[i] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    }
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs".
inline void karras_tree(BinaryTree& t) {
    const int64_t n = t.n;
    if (n < 2) return;
    auto delta = [&](int64_t i, int64_t j) -> int {
        if (j < 0 || j >= n) return -1;
        uint32_t a = t.codes[i], b = t.codes[j];
        if (a != b) return clz32(a ^ b);
        return 32 + clz32(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
    };
    t.left.assign(n - 1, 0); t.right.assign(n - 1, 0); t.first.assign(n - 1, 0); t.last.assign(n - 1, 0);
    for (int64_t i = 0; i < n - 1; ++i) {
        int d = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
        int dmin = delta(i, i - d);
        int64_t lmax = 2;
        while (delta(i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t s = lmax / 2; s >= 1; s /= 2)
            if (delta(i, i + (l + s) * d) > dmin) l += s;
        int64_t j = i + l * d;
        int dnode = delta(i, j);
        int64_t s = 0;
        int64_t div = 2;
        while (true) {
            int64_t step = (l + div - 1) / div;
            if (delta(i, i + (s + step) * d) > dnode) s += step;
            if (step <= 1) break;
            div *= 2;
        }
        int64_t gamma = i + s * d + std::min(d, 0);
        int64_t lo = std::min(i, j), hi = std::max(i, j);
        t.left[i] = (lo == gamma) ? static_cast<uint32_t>(n - 1 + gamma) : static_cast<uint32_t>(gamma);
        t.right[i] = (hi == gamma + 1) ? static_cast<uint32_t>(n - 1 + gamma + 1) : static_cast<uint32_t>(gamma + 1);
        t.first[i] = static_cast<uint32_t>(lo);
        t.last[i] = static_cast<uint32_t>(hi);
    }
}

struct WideBVH {
    std::vector<WideNode> nodes;
    std::vector<uint32_t> prim_order;   // leaf slot order -> build index
    uint32_t height = 0;
};

struct Collapse {
    uint32_t cnt = 0;
    uint32_t member[8];
};

class WideBuilder {
public:
    explicit WideBuilder(const std::vector<Box>& prims) : prims_(prims) {}

    WideBVH build() {
        WideBVH out;
        const uint32_t n = static_cast<uint32_t>(prims_.size());
        t_.n = n;
        if (n == 0) return out;
        std::vector<uint32_t> codes;
        morton_codes(prims_, codes);
        t_.order.resize(n);
        std::iota(t_.order.begin(), t_.order.end(), 0u);
        std::stable_sort(t_.order.begin(), t_.order.end(), [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; });
        t_.codes.resize(n);
        for (uint32_t i = 0; i < n; ++i) t_.codes[i] = codes[t_.order[i]];
        karras_tree(t_);
        // boxes: leaves then internal nodes bottom-up (children have larger
        // ids than... not guaranteed, so iterate by recursion-free post-order).
        t_.box.assign(2 * n - 1, box_empty());
        t_.sa.assign(2 * n - 1, 0.0f);
        for (uint32_t i = 0; i < n; ++i) {
            t_.box[n - 1 + i] = prims_[t_.order[i]];
            t_.sa[n - 1 + i] = half_area(t_.box[n - 1 + i]);
        }
        if (n >= 2) {
            std::vector<uint32_t> post;
            post_order(post);
            for (uint32_t x : post) {
                t_.box[x] = box_union(t_.box[t_.left[x]], t_.box[t_.right[x]]);
                t_.sa[x] = half_area(t_.box[x]);
            }
        }
        // wide counts / heights in post order
        wide_count_.assign(n >= 2 ? n - 1 : 0, 0);
        wide_height_.assign(n >= 2 ? n - 1 : 0, 0);
        if (n >= 2) {
            std::vector<uint32_t> post;
            post_order(post);
            for (uint32_t x : post) {
                Collapse c = collapse(x);
                uint32_t wc = 1, h = 0;
                for (uint32_t k = 0; k < c.cnt; ++k) {
                    uint32_t m = c.member[k];
                    if (is_internal_wide(m)) { wc += wide_count_[m]; h = std::max(h, wide_height_[m]); }
                }
                wide_count_[x] = wc;
                wide_height_[x] = h + 1;
            }
        }
        uint32_t total = (n >= 2) ? wide_count_[0] : 1;
        out.nodes.assign(total, WideNode{});
        out.prim_order.assign(n, 0);
        out.height = (n >= 2) ? wide_height_[0] : 1;
        // top-down layout (explicit stack; results independent of visit order)
        struct Item { uint32_t bin, widx, below, tbase; };
        std::vector<Item> stack;
        stack.push_back({n >= 2 ? 0u : (n - 1), 0u, 1u, 0u});
        while (!stack.empty()) {
            Item it = stack.back();
            stack.pop_back();
            emit(it.bin, it.widx, it.below, it.tbase, out, [&](uint32_t b, uint32_t w, uint32_t bl, uint32_t tb) {
                stack.push_back({b, w, bl, tb});
            });
        }
        return out;
    }

    const BinaryTree& tree() const { return t_; }

    uint32_t prims_of(uint32_t id) const {
        const uint32_t n = t_.n;
        if (id >= n - 1) return 1;
        return t_.last[id] - t_.first[id] + 1;
    }
    uint32_t first_of(uint32_t id) const {
        const uint32_t n = t_.n;
        if (id >= n - 1) return id - (n - 1);
        return t_.first[id];
    }
    bool is_internal_bin(uint32_t id) const { return id < t_.n - 1; }
    bool is_internal_wide(uint32_t id) const { return is_internal_bin(id) && prims_of(id) > 3; }

    Collapse collapse(uint32_t x) const {
        Collapse c;
        if (!is_internal_bin(x)) { c.cnt = 1; c.member[0] = x; return c; }
        c.cnt = 2;
        c.member[0] = t_.left[x];
        c.member[1] = t_.right[x];
        while (c.cnt < 8) {
            int best = -1;
            for (uint32_t k = 0; k < c.cnt; ++k) {
                uint32_t m = c.member[k];
                if (!is_internal_bin(m)) continue;
                if (best < 0) { best = static_cast<int>(k); continue; }
                uint32_t b = c.member[best];
                float sm = t_.sa[m], sb = t_.sa[b];
                if (sm > sb || (sm == sb && m < b)) best = static_cast<int>(k);
            }
            if (best < 0) break;
            uint32_t m = c.member[best];
            c.member[best] = t_.left[m];
            c.member[c.cnt++] = t_.right[m];
        }
        return c;
    }

private:
    void post_order(std::vector<uint32_t>& post) const {
        post.clear();
        const uint32_t n = t_.n;
        std::vector<std::pair<uint32_t, int>> st;
        st.push_back({0u, 0});
        while (!st.empty()) {
            auto& [x, state] = st.back();
            if (state == 0) {
                state = 1;
                uint32_t l = t_.left[x], r = t_.right[x];
                uint32_t xx = x;
                (void)xx;
                if (r < n - 1) st.push_back({r, 0});
                if (l < n - 1) st.push_back({l, 0});
            } else {
                post.push_back(x);
                st.pop_back();
            }
        }
    }

    template <class Push>
    void emit(uint32_t bin, uint32_t widx, uint32_t below, uint32_t tbase, WideBVH& out, Push push) {
        Collapse c = collapse(bin);
        const Box& nb = t_.box[bin];
        WideNode& w = out.nodes[widx];
        std::memset(&w, 0, sizeof(w));
        int e[3];
        for (int a = 0; a < 3; ++a) {
            w.origin[a] = nb.lo[a];
            e[a] = axis_exponent(nb.lo[a], nb.hi[a]);
        }
        // quantize children; bump an axis exponent if a child needs > 255
        for (int a = 0; a < 3; ++a) {
            for (;;) {
                bool ok = true;
                for (uint32_t k = 0; k < c.cnt && ok; ++k) {
                    const Box& cb = t_.box[c.member[k]];
                    double qh = std::ceil(std::ldexp(static_cast<double>(cb.hi[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                    if (qh > 255.0) ok = false;
                }
                if (ok) break;
                e[a] += 1;
            }
            w.exps[a] = static_cast<int8_t>(e[a]);
            for (uint32_t k = 0; k < c.cnt; ++k) {
                const Box& cb = t_.box[c.member[k]];
                double ql = std::floor(std::ldexp(static_cast<double>(cb.lo[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                double qh = std::ceil(std::ldexp(static_cast<double>(cb.hi[a]) - static_cast<double>(nb.lo[a]), -e[a]));
                w.qlo[a][k] = static_cast<uint8_t>(std::max(0.0, ql));
                w.qhi[a][k] = static_cast<uint8_t>(std::min(255.0, qh));
            }
            for (uint32_t k = c.cnt; k < 8; ++k) {   // unused slot: the inverted box 255..0
                w.qlo[a][k] = 255;
                w.qhi[a][k] = 0;
            }
        }
        // slots
        uint32_t nint = 0, nleaf = 0;
        for (uint32_t k = 0; k < c.cnt; ++k) {
            uint32_t m = c.member[k];
            if (is_internal_wide(m)) nint++;
            else nleaf += prims_of(m);
        }
        w.child_base = below;
        w.tri_base = tbase;
        uint32_t rank = 0, loff = 0;
        uint32_t sub_below = below + nint;
        uint32_t sub_tri = tbase + nleaf;
        for (uint32_t k = 0; k < c.cnt; ++k) {
            uint32_t m = c.member[k];
            if (is_internal_wide(m)) {
                w.imask |= static_cast<uint8_t>(1u << k);
                w.meta[k] = static_cast<uint8_t>(0x80u | rank);
                push(m, below + rank, sub_below, sub_tri);
                sub_below += wide_count_[m] - 1;
                sub_tri += prims_of(m);
                rank++;
            } else {
                uint32_t cnt = prims_of(m), f = first_of(m);
                w.meta[k] = static_cast<uint8_t>((cnt << 5) | loff);
                for (uint32_t q = 0; q < cnt; ++q) out.prim_order[tbase + loff + q] = t_.order[f + q];
                loff += cnt;
            }
        }
    }

    static int axis_exponent(float lo, float hi) {
        double d = static_cast<double>(hi) - static_cast<double>(lo);
        if (!(d > 0.0)) return -100;
        int ex;
        double m = std::frexp(d / 255.0, &ex);
        int e = (m == 0.5) ? ex - 1 : ex;
        return std::max(e, -100);
    }

    const std::vector<Box>& prims_;
    BinaryTree t_;
    std::vector<uint32_t> wide_count_, wide_height_;
};

// ---------------------------------------------------------------------------
// Ray / triangle and traversal
// ---------------------------------------------------------------------------
struct TriRec {      // 48 bytes, identical to ohao_bvh_tri
    float v0[3]; uint32_t prim;
    float v1[3]; uint32_t inst;
    float v2[3]; uint32_t ref;
};
static_assert(sizeof(TriRec) == 48, "tri record is 48 bytes");

struct RayPre {
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float invd[3];
};

inline RayPre ray_pre(const float o[3], const float d[3]) {
    RayPre r;
    for (int k = 0; k < 3; ++k) {
        r.o[k] = o[k];
        r.d[k] = d[k];
        float dd = std::fabs(d[k]) > 0x1p-80f ? d[k] : std::copysign(0x1p-80f, d[k]);
        r.invd[k] = 1.0f / dd;
    }
    int kz = 0;
    if (std::fabs(d[1]) > std::fabs(d[kz])) kz = 1;
    if (std::fabs(d[2]) > std::fabs(d[kz])) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

// Woop-Benthin-Wald watertight test; returns true with (t,u,v) when
// tmin < t < tmax. u,v are the barycentric weights of v1 and v2.
inline bool tri_intersect(const RayPre& r, const float* v0, const float* v1, const float* v2,
                          float tmin, float tmax, float& t_out, float& u_out, float& v_out) {
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) { A[k] = v0[k] - r.o[k]; B[k] = v1[k] - r.o[k]; C[k] = v2[k] - r.o[k]; }
    float Ax = A[r.kx] - r.Sx * A[r.kz];
    float Ay = A[r.ky] - r.Sy * A[r.kz];
    float Bx = B[r.kx] - r.Sx * B[r.kz];
    float By = B[r.ky] - r.Sy * B[r.kz];
    float Cx = C[r.kx] - r.Sx * C[r.kz];
    float Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = static_cast<double>(Cx) * static_cast<double>(By);
        double CyBx = static_cast<double>(Cy) * static_cast<double>(Bx);
        U = static_cast<float>(CxBy - CyBx);
        double AxCy = static_cast<double>(Ax) * static_cast<double>(Cy);
        double AyCx = static_cast<double>(Ay) * static_cast<double>(Cx);
        V = static_cast<float>(AxCy - AyCx);
        double BxAy = static_cast<double>(Bx) * static_cast<double>(Ay);
        double ByAx = static_cast<double>(By) * static_cast<double>(Ax);
        W = static_cast<float>(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * A[r.kz];
    float Bz = r.Sz * B[r.kz];
    float Cz = r.Sz * C[r.kz];
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

struct HitRec {
    float t = 0.0f, u = 0.0f, v = 0.0f;
    uint32_t inst = 0xFFFFFFFFu, prim = 0xFFFFFFFFu;
    bool hit() const { return prim != 0xFFFFFFFFu; }
};

inline bool key_less(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb) {
    return ia < ib || (ia == ib && pa < pb);
}

struct TravStats {
    uint64_t nodes = 0, tris = 0, insts = 0;
};

// Per-node slab test in the node's quantized frame; conservative margins
// make the culling safe against rounding (see the file header).
struct NodeHits {
    uint32_t mask = 0;
    float tnear[8];
};

constexpr float kTravRelSlack = 0x1p-14f;   // relative slack on tbest
constexpr float kTravAbsScale = 0x1p-21f;   // per-node absolute margin factor
constexpr float kTravBiasMargin = 0x1p-8f;  // extra margin for the biased slab offsets

inline NodeHits node_test(const WideNode& n, const RayPre& r, float tmin, float tbest) {
    NodeHits h;
    // t = q a + b -+ m evaluated as fma(2^23 + 256 q, a / 256, b -+ m - 2^15 a):
    // the offset rounded once, the extra 2^-8 |a| of margin covering it
    float a[3], bn[3], bf[3];
    for (int k = 0; k < 3; ++k) {
        float s = std::ldexp(1.0f, n.exps[k]);
        float ak = s * r.invd[k];
        float b = (n.origin[k] - r.o[k]) * r.invd[k];
        float m = 255.0f * std::fabs(ak) + std::fabs(b);
        m = m * kTravAbsScale;
        m = m + std::fabs(ak) * kTravBiasMargin;
        a[k] = ak * 0x1p-8f;
        bn[k] = fma_(-0x1p15f, ak, b - m);
        bf[k] = fma_(-0x1p15f, ak, b + m);
    }
    float tlimit = tbest + tbest * kTravRelSlack;
    for (int i = 0; i < 8; ++i) {
        float tn = 0.0f, tf = 0.0f;
        for (int k = 0; k < 3; ++k) {
            float lo = 8388608.0f + 256.0f * static_cast<float>(n.qlo[k][i]);
            float hi = 8388608.0f + 256.0f * static_cast<float>(n.qhi[k][i]);
            float qn = r.invd[k] < 0.0f ? hi : lo, qf = r.invd[k] < 0.0f ? lo : hi;
            float vn = fma_(qn, a[k], bn[k]), vf = fma_(qf, a[k], bf[k]);
            tn = (k == 0) ? vn : std::fmax(tn, vn);
            tf = (k == 0) ? vf : std::fmin(tf, vf);
        }
        h.tnear[i] = tn;
        // tn <= tf, tn <= tlimit and tf >= tmin in one comparison (tmin <= tlimit)
        if (n.meta[i] != 0 && std::fmax(tn, tmin) <= std::fmin(tf, tlimit)) h.mask |= 1u << i;
    }
    return h;
}

// Optional test of a candidate hit (an any-hit shader): false ignores it.
struct HitFilter {
    const void* ctx = nullptr;
    bool (*accept)(const void* ctx, uint32_t inst, uint32_t prim, float u, float v) = nullptr;
    bool operator()(uint32_t inst, uint32_t prim, float u, float v) const { return accept(ctx, inst, prim, u, v); }
};

struct BvhView {
    const WideNode* nodes = nullptr;
    const TriRec* tris = nullptr;
    uint32_t nnodes = 0;
    bool empty() const { return nnodes == 0; }
};

// Closest hit in one BVH over the ray interval (tmin, tmax). `best` may
// already hold a hit from another BVH (two-level traversal). `inst_override`
// != ~0 replaces the record's instance field (BLAS inside an instance).
inline float cull_limit(const HitRec& best, float tmax) {
    float t = best.hit() ? best.t : tmax;
    return t + t * kTravRelSlack;
}

inline void bvh_closest(const BvhView& bvh, const RayPre& r, float tmin, float tmax, HitRec& best,
                        uint32_t inst_override, TravStats* st, const HitFilter* filter = nullptr) {
    if (bvh.empty()) return;
    std::vector<std::pair<uint32_t, float>> stack;
    stack.reserve(64);
    stack.push_back({0u, -INFINITY});
    while (!stack.empty()) {
        auto [ni, tn0] = stack.back();
        stack.pop_back();
        if (tn0 > cull_limit(best, tmax)) continue;
        const WideNode& n = bvh.nodes[ni];
        if (st) st->nodes++;
        NodeHits h = node_test(n, r, tmin, best.hit() ? best.t : tmax);
        for (int i = 0; i < 8; ++i) {
            if (!(h.mask & (1u << i)) || (n.imask & (1u << i))) continue;
            uint32_t cnt = n.meta[i] >> 5, off = n.meta[i] & 31u;
            for (uint32_t q = 0; q < cnt; ++q) {
                const TriRec& tr = bvh.tris[n.tri_base + off + q];
                if (st) st->tris++;
                float t, u, v;
                if (!tri_intersect(r, tr.v0, tr.v1, tr.v2, tmin, tmax, t, u, v)) continue;
                uint32_t inst = (inst_override != 0xFFFFFFFFu) ? inst_override : tr.inst;
                if (filter && !(*filter)(inst, tr.prim, u, v)) continue;
                if (!best.hit() || t < best.t || (t == best.t && key_less(inst, tr.prim, best.inst, best.prim))) {
                    best.t = t; best.u = u; best.v = v; best.inst = inst; best.prim = tr.prim;
                }
            }
        }
        uint32_t ids[8]; float tns[8]; int cnt = 0;
        for (int i = 0; i < 8; ++i) {
            if (!(h.mask & (1u << i)) || !(n.imask & (1u << i))) continue;
            ids[cnt] = n.child_base + (n.meta[i] & 7u);
            tns[cnt] = h.tnear[i];
            cnt++;
        }
        for (int i = 1; i < cnt; ++i)
            for (int j = i; j > 0 && tns[j] > tns[j - 1]; --j) { std::swap(tns[j], tns[j - 1]); std::swap(ids[j], ids[j - 1]); }
        for (int i = 0; i < cnt; ++i) stack.push_back({ids[i], tns[i]});
    }
}

inline bool bvh_any(const BvhView& bvh, const RayPre& r, float tmin, float tmax, TravStats* st,
                    const HitFilter* filter = nullptr, uint32_t inst_override = 0xFFFFFFFFu) {
    if (bvh.empty()) return false;
    std::vector<uint32_t> stack;
    stack.reserve(64);
    stack.push_back(0u);
    while (!stack.empty()) {
        uint32_t ni = stack.back();
        stack.pop_back();
        const WideNode& n = bvh.nodes[ni];
        if (st) st->nodes++;
        NodeHits h = node_test(n, r, tmin, tmax);
        for (int i = 0; i < 8; ++i) {
            if (!(h.mask & (1u << i))) continue;
            if (n.imask & (1u << i)) { stack.push_back(n.child_base + (n.meta[i] & 7u)); continue; }
            uint32_t cnt = n.meta[i] >> 5, off = n.meta[i] & 31u;
            for (uint32_t q = 0; q < cnt; ++q) {
                const TriRec& tr = bvh.tris[n.tri_base + off + q];
                if (st) st->tris++;
                float t, u, v;
                if (!tri_intersect(r, tr.v0, tr.v1, tr.v2, tmin, tmax, t, u, v)) continue;
                if (!filter || (*filter)(inst_override != 0xFFFFFFFFu ? inst_override : tr.inst, tr.prim, u, v))
                    return true;
            }
        }
    }
    return false;
}

}  // namespace orc
