// pt_traverse.cuh -- 8-wide BVH traversal (closest hit and any hit).
//
// Node record: 80 bytes = 5 x uint4, the layout of ohao_bvh8_node:
//   q0 = origin.xyz, (exponents x,y,z, internal mask)
//   q1 = child_base, tri_base, meta[0..3], meta[4..7]
//   q2 = qlo.x[0..7], qlo.y[0..7]   q3 = qlo.z[0..7], qhi.x[0..7]
//   q4 = qhi.y[0..7], qhi.z[0..7]
// Child boxes are tested in the node's quantised frame: one FMA per slab side
// (t = q * (2^e / d) + (origin - o) / d) with per-axis conservative margins
// folded into the offsets. Near/far planes are chosen once per node by
// swapping the lo/hi byte words of axes with a negative direction. A byte q
// enters the FMA as the float 2^23 + 256 q (one byte permute, exact), the
// 2^15 a it carries being taken out of the offset once per node.
//
// Visit order (kept identical to the host oracle, so node/triangle visit
// counts match): leaves of a node are tested first, in slot order; then the
// nearest internal child is visited next and the others are pushed far to
// near (ties: lower slot pushed first). Popped entries whose entry distance
// exceeds the best hit (with a 2^-14 relative slack) are skipped. Any-hit
// queries return at the first hit; in a flat BVH they test a node's leaves,
// then continue with the nearest internal child (others pushed far to near,
// so nearby occluders are found sooner; the host oracle walks in slot order
// -- the answer is the same boolean either way); the two-level any-hit
// keeps slot order.
// The stack holds 64 (node, t_near) entries in local memory (fewer when the
// scene's stack_limit says so); overflow sets the error flag instead of
// faulting or writing past the stack.
#pragma once

namespace ohao {

constexpr float kTravRelSlack = 0x1p-14f;
constexpr float kTravAbsScale = 0x1p-21f;
constexpr float kTravBiasMargin = 0x1p-8f;   // covers the rounding of the biased slab offsets
constexpr int kStackSize = 64;

// Stack entries a ray may use: the scene's limit, which the host sets in
// [1, kStackSize] (a smaller one makes deep traversals report the overflow
// error; used to test that check). Read from the kernel parameters at each
// use, so it costs no register.
OHAO_D int stack_limit(const DScene& sc) { return static_cast<int>(sc.stack_limit); }

struct Hit {
    float t, u, v;
    uint32_t inst, prim;
};

OHAO_D bool key_less(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb) {
    return ia < ib || (ia == ib && pa < pb);
}

struct TravCount {
    uint32_t nodes, tris;
};

struct NodeRec {
    uint4 q0, q1, q2, q3, q4;
};

// Traversal stack of (node, t_near) entries. The first kSh entries of a ray
// live in shared memory -- one column per thread, entry i at
// sh[i * kShStride], so a warp's accesses are conflict-free whatever mix of
// depths its lanes are at -- and the rest in local memory. kSh = 0 keeps the
// whole stack in local memory.
constexpr int kShStride = 128;   // threads per block of the traversal kernels
template <int kSh>
struct TravStack {
    uint2* sh;
    uint32_t ln[kStackSize - kSh];
    float lt[kStackSize - kSh];
    OHAO_D void put(int i, uint32_t n, float t) {
        if (kSh > 0 && i < kSh) {
            sh[i * kShStride] = make_uint2(n, __float_as_uint(t));
        } else {
            ln[i - kSh] = n;
            lt[i - kSh] = t;
        }
    }
    OHAO_D void get(int i, uint32_t& n, float& t) const {
        if (kSh > 0 && i < kSh) {
            const uint2 e = sh[i * kShStride];
            n = e.x;
            t = __uint_as_float(e.y);
        } else {
            n = ln[i - kSh];
            t = lt[i - kSh];
        }
    }
    OHAO_D void put_node(int i, uint32_t n) {
        if (kSh > 0 && i < kSh) sh[i * kShStride].x = n;
        else ln[i - kSh] = n;
    }
    OHAO_D uint32_t get_node(int i) const { return (kSh > 0 && i < kSh) ? sh[i * kShStride].x : ln[i - kSh]; }
};

// The same interface over two caller-owned local arrays.
struct ArrStack {
    uint32_t* node;
    float* t;
    OHAO_D void put(int i, uint32_t n, float tn) { node[i] = n; t[i] = tn; }
    OHAO_D void get(int i, uint32_t& n, float& tn) const { n = node[i]; tn = t[i]; }
    OHAO_D void put_node(int i, uint32_t n) { node[i] = n; }
    OHAO_D uint32_t get_node(int i) const { return node[i]; }
};

OHAO_D NodeRec load_node(const uint4* __restrict__ nodes, uint32_t ni) {
    const uint4* p = nodes + static_cast<size_t>(ni) * 5;
    NodeRec n;
    n.q0 = __ldg(p);
    n.q1 = __ldg(p + 1);
    n.q2 = __ldg(p + 2);
    n.q3 = __ldg(p + 3);
    n.q4 = __ldg(p + 4);
    return n;
}

// byte i (0-7) of the 8-byte word hi4:lo4: one byte permute (selector i in
// its low nibble picks the byte) and a mask
OHAO_D uint32_t byte_of(uint32_t lo4, uint32_t hi4, int i) {
    return __byte_perm(lo4, hi4, static_cast<uint32_t>(i)) & 0xFFu;
}

// three-input min / max of sm_100+ (one instruction each; NaN operands are
// ignored, as by fmaxf / fminf)
OHAO_D float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
OHAO_D float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Two independent fp32 FMAs in one paired instruction of sm_100+
// (fma.rn.f32x2): each half is rounded exactly as fmaf rounds it.
OHAO_D void fma2(float x0, float x1, float y0, float y1, float z0, float z1, float& d0, float& d1) {
    asm("{.reg .b64 x, y, z, d;\n\t"
        "mov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\tmov.b64 z, {%6, %7};\n\t"
        "fma.rn.f32x2 d, x, y, z;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d0), "=f"(d1)
        : "f"(x0), "f"(x1), "f"(y0), "f"(y1), "f"(z0), "f"(z1));
}

// byte b of `word` (q) as the float 2^23 + 256 q, exactly: one byte permute
// into the bits 0x4B00qq00 (no conversion instruction, no add)
OHAO_D float u8f_biased(uint32_t word, int b) {
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7604u | (static_cast<uint32_t>(b) << 4)));
}

// Hit mask of the 8 child boxes; tn[i] = conservative entry distance.
OHAO_D uint32_t node_test(const NodeRec& n, const RayPre& r, float tmin, float tbest, float tn[8]) {
    const float org[3] = {__uint_as_float(n.q0.x), __uint_as_float(n.q0.y), __uint_as_float(n.q0.z)};
    // Slab side of child plane q (a byte): t = q * a + b +- m. With x = 2^23 +
    // 256 q (the byte permuted into the mantissa) and A = a / 256, x * A =
    // 2^15 a + q a, so t = fma(x, A, b +- m - 2^15 a): one FMA per side. The
    // offset b +- m - 2^15 a is rounded once (error <= 2^-24 |b +- m| + 2^-9
    // |a|), which the extra 2^-8 |a| of margin covers.
    float a[3], bn[3], bf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int e = static_cast<int>(static_cast<int8_t>((n.q0.w >> (8 * k)) & 0xFFu));
        const float s = __int_as_float((e + 127) << 23);
        const float ak = s * r.invd[k];
        const float b = (org[k] - r.o[k]) * r.invd[k];
        float m = 255.0f * fabsf(ak) + fabsf(b);
        m = m * kTravAbsScale;
        m = m + fabsf(ak) * kTravBiasMargin;
        a[k] = ak * 0x1p-8f;
        bn[k] = fmaf(-0x1p15f, ak, b - m);
        bf[k] = fmaf(-0x1p15f, ak, b + m);
    }
    // near / far byte words per axis (slots 0-3, 4-7)
    const bool nx = r.invd[0] < 0.0f, ny = r.invd[1] < 0.0f, nz = r.invd[2] < 0.0f;
    const uint32_t nx0 = nx ? n.q3.z : n.q2.x, nx1 = nx ? n.q3.w : n.q2.y;
    const uint32_t fx0 = nx ? n.q2.x : n.q3.z, fx1 = nx ? n.q2.y : n.q3.w;
    const uint32_t ny0 = ny ? n.q4.x : n.q2.z, ny1 = ny ? n.q4.y : n.q2.w;
    const uint32_t fy0 = ny ? n.q2.z : n.q4.x, fy1 = ny ? n.q2.w : n.q4.y;
    const uint32_t nz0 = nz ? n.q4.z : n.q3.x, nz1 = nz ? n.q4.w : n.q3.y;
    const uint32_t fz0 = nz ? n.q3.x : n.q4.z, fz1 = nz ? n.q3.y : n.q4.w;
    const float tlimit = tbest + tbest * kTravRelSlack;
    uint32_t hit = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int b = i & 3;
        const float qnx = u8f_biased(i < 4 ? nx0 : nx1, b), qfx = u8f_biased(i < 4 ? fx0 : fx1, b);
        const float qny = u8f_biased(i < 4 ? ny0 : ny1, b), qfy = u8f_biased(i < 4 ? fy0 : fy1, b);
        const float qnz = u8f_biased(i < 4 ? nz0 : nz1, b), qfz = u8f_biased(i < 4 ? fz0 : fz1, b);
        // near and far side of each axis in one paired FMA
        float vnx, vfx, vny, vfy, vnz, vfz;
        fma2(qnx, qfx, a[0], a[0], bn[0], bf[0], vnx, vfx);
        fma2(qny, qfy, a[1], a[1], bn[1], bf[1], vny, vfy);
        fma2(qnz, qfz, a[2], a[2], bn[2], bf[2], vnz, vfz);
        const float t0 = max3f(vnx, vny, vnz);
        const float t1 = min3f(vfx, vfy, vfz);
        tn[i] = t0;
        // t0 <= t1, t0 <= tlimit and t1 >= tmin at once (tmin <= tlimit always).
        // Unused slots hold the inverted box 255..0, which fails this test (and
        // were it to pass, the slot is a leaf of no triangles: no effect).
        if (fmaxf(t0, tmin) <= fminf(t1, tlimit)) hit |= 1u << i;
    }
    return hit;
}

OHAO_D float pick8(const float v[8], int i) {
    float r = v[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) r = (i == k) ? v[k] : r;
    return r;
}

// Orders the internal children `rem`: pushes all but the nearest (far first,
// ties: lower slot first) and returns the nearest in (cur, cur_tn).
// Returns false on stack overflow.
template <class Stack>
OHAO_D bool order_children(uint32_t rem, const float tn[8], const NodeRec& n, Stack& stk, int& sp, uint32_t& cur,
                           float& cur_tn, int lim) {
    while (__popc(rem) > 1) {
        float bt = 0.0f;
        int bi = -1;
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (((rem >> i) & 1u) && (bi < 0 || tn[i] > bt)) { bt = tn[i]; bi = i; }
        if (sp >= lim) return false;
        stk.put(sp, n.q1.x + (byte_of(n.q1.z, n.q1.w, bi) & 7u), bt);
        sp++;
        rem &= ~(1u << bi);
    }
    const int li = __ffs(rem) - 1;
    cur = n.q1.x + (byte_of(n.q1.z, n.q1.w, li) & 7u);
    cur_tn = pick8(tn, li);
    return true;
}

// One step of the closest-hit walk of one BVH (flat, or a BLAS inside
// instance inst_override): the node (cur, cur_tn) -- culled against the best
// hit, else tested, its triangle leaves intersected and its internal
// children ordered (the nearest becomes the next node) -- or else a pop.
// Returns true when the walk is over (the stack is back at stack_base, or it
// overflowed: err).
template <bool kStats, bool kAlpha, class Stack>
OHAO_D bool closest_step(const DScene& sc, const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                         const RayPre& r, float tmin, float tmax, Hit& best, uint32_t inst_override, Stack& stk,
                         int stack_base, int lim, TravCount& cnt, int& err, int& sp, uint32_t& cur, float& cur_tn) {
    const float tb = best.prim != 0xFFFFFFFFu ? best.t : tmax;
    if (cur_tn <= tb + tb * kTravRelSlack) {
        const NodeRec n = load_node(nodes, cur);
        if (kStats) cnt.nodes++;
        float tn[8];
        const uint32_t hit = node_test(n, r, tmin, tb, tn);
        const uint32_t imask = n.q0.w >> 24;
        uint32_t lm = hit & ~imask;
        while (lm) {
            const int i = __ffs(lm) - 1;
            lm &= lm - 1;
            const uint32_t meta = byte_of(n.q1.z, n.q1.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const float4* tp = tris + static_cast<size_t>(n.q1.y + off + q) * 3;
                const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                if (kStats) cnt.tris++;
                float t, u, v;
                if (!tri_intersect(r, v0, v1, v2, tmin, tmax, t, u, v)) continue;
                const uint32_t prim = __float_as_uint(v0.w);
                const uint32_t inst = (inst_override != 0xFFFFFFFFu) ? inst_override : __float_as_uint(v1.w);
                if (kAlpha && sc.alpha_test && !alpha_accept(sc, inst, prim, u, v)) continue;
                if (best.prim == 0xFFFFFFFFu || t < best.t ||
                    (t == best.t && key_less(inst, prim, best.inst, best.prim))) {
                    best.t = t; best.u = u; best.v = v; best.inst = inst; best.prim = prim;
                }
            }
        }
        const uint32_t rem = hit & imask;
        if (rem) {
            if (!order_children(rem, tn, n, stk, sp, cur, cur_tn, lim)) { err = 1; return true; }
            return false;
        }
    }
    if (sp == stack_base) return true;
    sp--;
    stk.get(sp, cur, cur_tn);
    return false;
}

// Closest hit in one BVH (flat, or a BLAS inside instance inst_override).
template <bool kStats, bool kAlpha, class Stack>
OHAO_D void bvh_closest(const DScene& sc, const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                        const RayPre& r, float tmin, float tmax, Hit& best, uint32_t inst_override, Stack& stk,
                        int stack_base, int lim, TravCount& cnt, int& err) {
    if (stack_base >= lim) { err = 1; return; }
    int sp = stack_base;
    uint32_t cur = 0u;
    float cur_tn = -INFINITY;
    while (!closest_step<kStats, kAlpha>(sc, nodes, tris, r, tmin, tmax, best, inst_override, stk, stack_base, lim,
                                         cnt, err, sp, cur, cur_tn)) {
    }
}

// Any hit in one BVH.
template <bool kStats, bool kAlpha, class Stack>
OHAO_D bool bvh_any(const DScene& sc, const uint4* __restrict__ nodes, const float4* __restrict__ tris, const RayPre& r,
                    float tmin, float tmax, Stack& stk, int stack_base, int lim, TravCount& cnt, int& err) {
    if (stack_base >= lim) { err = 1; return false; }
    int sp = stack_base;
    uint32_t cur = 0u;
    while (true) {
        const NodeRec n = load_node(nodes, cur);
        if (kStats) cnt.nodes++;
        float tn[8];
        const uint32_t m = node_test(n, r, tmin, tmax, tn);
        const uint32_t imask = n.q0.w >> 24;
        uint32_t lm = m & ~imask;
        while (lm) {
            const int i = __ffs(lm) - 1;
            lm &= lm - 1;
            const uint32_t meta = byte_of(n.q1.z, n.q1.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            for (uint32_t q = 0; q < c; ++q) {
                const float4* tp = tris + static_cast<size_t>(n.q1.y + off + q) * 3;
                const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                if (kStats) cnt.tris++;
                float t, u, v;
                if (tri_intersect(r, v0, v1, v2, tmin, tmax, t, u, v) &&
                    (!kAlpha || !sc.alpha_test || alpha_accept(sc, __float_as_uint(v1.w), __float_as_uint(v0.w), u, v)))
                    return true;
            }
        }
        uint32_t rem = m & imask;
        if (rem) {   // nearest internal child next, the others pushed far to near
            while (__popc(rem) > 1) {
                float bt = 0.0f;
                int bi = -1;
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (((rem >> i) & 1u) && (bi < 0 || tn[i] > bt)) { bt = tn[i]; bi = i; }
                if (sp >= lim) { err = 1; return false; }
                stk.put_node(sp++, n.q1.x + (byte_of(n.q1.z, n.q1.w, bi) & 7u));
                rem &= ~(1u << bi);
            }
            cur = n.q1.x + (byte_of(n.q1.z, n.q1.w, __ffs(rem) - 1) & 7u);
            continue;
        }
        if (sp == stack_base) return false;
        cur = stk.get_node(--sp);
    }
}

OHAO_D void xform_point(const float m[12], V3 p, V3& o) {
    o.x = ((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3];
    o.y = ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7];
    o.z = ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11];
}
OHAO_D void xform_dir(const float m[12], V3 d, V3& o) {
    o.x = (m[0] * d.x + m[1] * d.y) + m[2] * d.z;
    o.y = (m[4] * d.x + m[5] * d.y) + m[6] * d.z;
    o.z = (m[8] * d.x + m[9] * d.y) + m[10] * d.z;
}

// Scene-level closest hit (flat or two-level). tmax <= tmin means no hit.
// kLevels: 0 = decided by the scene at run time, 1 = flat BVH only,
// 2 = two-level only (kernels specialised per scene kind keep the flat
// traversal at its own register count).
// kAlpha: rays without gl_RayFlagsOpaqueEXT are possible (the alpha test
// of non-opaque instances is compiled in; it runs when sc.alpha_test).
// kSh: stack entries of a flat traversal kept in shared memory (sh: this
// thread's column; the two-level traversal keeps its stack in local memory).
template <bool kStats, int kLevels = 0, bool kAlpha = false, int kSh = 0>
OHAO_D Hit scene_closest(const DScene& sc, V3 o, V3 d, float tmin, float tmax, TravCount& cnt, int& err,
                         uint2* sh = nullptr) {
    Hit best;
    best.t = 0.0f; best.u = 0.0f; best.v = 0.0f;
    best.inst = 0xFFFFFFFFu; best.prim = 0xFFFFFFFFu;
    if (!(tmax > tmin) || sc.nnodes == 0) return best;
    const RayPre r = ray_pre(o, d);
    if (kLevels == 1 || (kLevels == 0 && !sc.two_level)) {
        TravStack<kSh> stk;
        stk.sh = sh;
        bvh_closest<kStats, kAlpha>(sc, sc.nodes, sc.tris, r, tmin, tmax, best, 0xFFFFFFFFu, stk, 0, stack_limit(sc),
                                    cnt, err);
        return best;
    }
    uint32_t st_node[kStackSize];
    float st_t[kStackSize];
    ArrStack ast{st_node, st_t};
    // Two-level: one loop whose every iteration visits one node (TLAS or
    // BLAS) or enters one instance, so the lanes of a warp stay on the same
    // code whatever level each ray is in. Order of visits per ray: at a TLAS
    // node, its hit instance leaves in slot order (each BLAS fully), then the
    // nearest internal child, then the stack -- the order of a nested
    // TLAS-then-BLAS traversal, hence the same hits and visit counts.
    int sp = 0;
    bool in_blas = false;
    RayPre ra = r;                          // the ray of the current level (object space inside a BLAS)
    const uint4* bnodes = sc.nodes;
    const float4* btris = nullptr;
    uint32_t inst = 0u;
    int base = 0;                           // stack base of the current BLAS
    uint32_t cur = 0u;
    float cur_tn = -INFINITY;
    bool have_node = true;
    bool resume = false;                    // TLAS child to continue with after the pending instances
    uint32_t res_cur = 0u;
    float res_tn = 0.0f;
    uint4 pq = make_uint4(0, 0, 0, 0);      // pending instance leaves: the TLAS node's (child, leaf, meta, meta)
    uint32_t plm = 0u, pidx = 0u;
    while (true) {
        if (have_node) {
            const float tb = best.prim != 0xFFFFFFFFu ? best.t : tmax;
            bool desc = false;
            bool leaves = false;
            if (cur_tn <= tb + tb * kTravRelSlack) {
                const NodeRec n = load_node(in_blas ? bnodes : sc.nodes, cur);
                if (kStats) cnt.nodes++;
                float tn[8];
                const uint32_t hit = node_test(n, ra, tmin, tb, tn);
                const uint32_t imask = n.q0.w >> 24;
                uint32_t lm = hit & ~imask;
                if (in_blas) {
                    while (lm) {
                        const int i = __ffs(lm) - 1;
                        lm &= lm - 1;
                        const uint32_t meta = byte_of(n.q1.z, n.q1.w, i);
                        const uint32_t c = meta >> 5, off = meta & 31u;
                        for (uint32_t q = 0; q < c; ++q) {
                            const float4* tp = btris + static_cast<size_t>(n.q1.y + off + q) * 3;
                            const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                            if (kStats) cnt.tris++;
                            float t, u, v;
                            if (!tri_intersect(ra, v0, v1, v2, tmin, tmax, t, u, v)) continue;
                            const uint32_t prim = __float_as_uint(v0.w);
                            if (kAlpha && sc.alpha_test && !alpha_accept(sc, inst, prim, u, v)) continue;
                            if (best.prim == 0xFFFFFFFFu || t < best.t ||
                                (t == best.t && key_less(inst, prim, best.inst, best.prim))) {
                                best.t = t; best.u = u; best.v = v; best.inst = inst; best.prim = prim;
                            }
                        }
                    }
                } else if (lm) {
                    pq = n.q1;
                    plm = lm;
                    pidx = 0u;
                    leaves = true;
                }
                const uint32_t rem = hit & imask;
                if (rem) {
                    if (!order_children(rem, tn, n, ast, sp, cur, cur_tn, stack_limit(sc))) {
                        err = 1;
                        return best;
                    }
                    desc = true;
                }
            }
            if (leaves) {
                resume = desc;
                res_cur = cur;
                res_tn = cur_tn;
                have_node = false;
            } else if (!desc) {
                have_node = false;
            }
            if (have_node) continue;
        }
        if (in_blas) {
            if (sp > base) {
                sp--;
                cur = st_node[sp];
                cur_tn = st_t[sp];
                have_node = true;
                continue;
            }
            in_blas = false;
            ra = r;
        }
        if (plm) {   // enter the next pending instance
            const int i = __ffs(plm) - 1;
            const uint32_t meta = byte_of(pq.z, pq.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            if (pidx >= c) {
                plm &= plm - 1;
                pidx = 0u;
                continue;
            }
            const uint32_t ii = __ldg(sc.tlas_inst + pq.y + off + pidx);
            if (++pidx == c) {
                plm &= plm - 1;
                pidx = 0u;
            }
            const DInst& in = sc.inst[ii];
            const DBlas bl = sc.blas[in.blas];
            V3 oo, od;
            xform_point(in.w2o, o, oo);
            xform_dir(in.w2o, d, od);
            ra = ray_pre(oo, od);
            bnodes = sc.blas_nodes + static_cast<size_t>(bl.node_off) * 5;
            btris = sc.blas_tris + static_cast<size_t>(bl.tri_off) * 3;
            inst = ii;
            base = sp;
            if (base >= stack_limit(sc)) { err = 1; return best; }
            cur = 0u;
            cur_tn = -INFINITY;
            in_blas = true;
            have_node = true;
            continue;
        }
        if (resume) {
            resume = false;
            cur = res_cur;
            cur_tn = res_tn;
            have_node = true;
            continue;
        }
        if (sp == 0) return best;
        sp--;
        cur = st_node[sp];
        cur_tn = st_t[sp];
        have_node = true;
    }
}

template <bool kStats, int kLevels = 0, bool kAlpha = false, int kSh = 0>
OHAO_D bool scene_occluded(const DScene& sc, V3 o, V3 d, float tmin, float tmax, TravCount& cnt, int& err,
                           uint2* sh = nullptr) {
    if (!(tmax > tmin) || sc.nnodes == 0) return false;
    const RayPre r = ray_pre(o, d);
    if (kLevels == 1 || (kLevels == 0 && !sc.two_level)) {
        TravStack<kSh> stk;
        stk.sh = sh;
        return bvh_any<kStats, kAlpha>(sc, sc.nodes, sc.tris, r, tmin, tmax, stk, 0, stack_limit(sc), cnt, err);
    }
    uint32_t st_node[kStackSize];
    // Two-level, as one loop (see scene_closest): at a TLAS node the internal
    // children but the last (slot order) are pushed, its instance leaves are
    // entered in slot order, then the last internal child is visited.
    int sp = 0;
    bool in_blas = false;
    RayPre ra = r;
    const uint4* bnodes = sc.nodes;
    const float4* btris = nullptr;
    uint32_t inst = 0u;                     // instance of the current BLAS
    int base = 0;
    uint32_t cur = 0u;
    bool have_node = true;
    bool resume = false;
    uint32_t res_cur = 0u;
    uint4 pq = make_uint4(0, 0, 0, 0);
    uint32_t plm = 0u, pidx = 0u;
    while (true) {
        if (have_node) {
            const NodeRec n = load_node(in_blas ? bnodes : sc.nodes, cur);
            if (kStats) cnt.nodes++;
            float tn[8];
            uint32_t m = node_test(n, ra, tmin, tmax, tn);
            const uint32_t imask = n.q0.w >> 24;
            bool have = false;
            uint32_t next = 0u;
            if (!in_blas) {
                plm = m & ~imask;
                pq = n.q1;
                pidx = 0u;
                m &= imask;
            }
            while (m) {
                const int i = __ffs(m) - 1;
                m &= m - 1;
                const uint32_t meta = byte_of(n.q1.z, n.q1.w, i);
                if ((imask >> i) & 1u) {
                    if (have) {
                        if (sp >= stack_limit(sc)) { err = 1; return false; }
                        st_node[sp++] = next;
                    }
                    next = n.q1.x + (meta & 7u);
                    have = true;
                    continue;
                }
                const uint32_t c = meta >> 5, off = meta & 31u;
                for (uint32_t q = 0; q < c; ++q) {
                    const float4* tp = btris + static_cast<size_t>(n.q1.y + off + q) * 3;
                    const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                    if (kStats) cnt.tris++;
                    float t, u, v;
                    if (tri_intersect(ra, v0, v1, v2, tmin, tmax, t, u, v) &&
                        (!kAlpha || !sc.alpha_test || alpha_accept(sc, inst, __float_as_uint(v0.w), u, v)))
                        return true;
                }
            }
            if (!in_blas && plm) {
                resume = have;
                res_cur = next;
                have_node = false;
            } else if (have) {
                cur = next;
                continue;
            } else {
                have_node = false;
            }
        }
        if (in_blas) {
            if (sp > base) {
                cur = st_node[--sp];
                have_node = true;
                continue;
            }
            in_blas = false;
            ra = r;
        }
        if (plm) {   // enter the next pending instance
            const int i = __ffs(plm) - 1;
            const uint32_t meta = byte_of(pq.z, pq.w, i);
            const uint32_t c = meta >> 5, off = meta & 31u;
            if (pidx >= c) {
                plm &= plm - 1;
                pidx = 0u;
                continue;
            }
            const uint32_t ii = __ldg(sc.tlas_inst + pq.y + off + pidx);
            if (++pidx == c) {
                plm &= plm - 1;
                pidx = 0u;
            }
            const DInst& in = sc.inst[ii];
            const DBlas bl = sc.blas[in.blas];
            V3 oo, od;
            xform_point(in.w2o, o, oo);
            xform_dir(in.w2o, d, od);
            ra = ray_pre(oo, od);
            inst = ii;
            bnodes = sc.blas_nodes + static_cast<size_t>(bl.node_off) * 5;
            btris = sc.blas_tris + static_cast<size_t>(bl.tri_off) * 3;
            base = sp;
            if (base >= stack_limit(sc)) { err = 1; return false; }
            cur = 0u;
            in_blas = true;
            have_node = true;
            continue;
        }
        if (resume) {
            resume = false;
            cur = res_cur;
            have_node = true;
            continue;
        }
        if (sp == 0) return false;
        cur = st_node[--sp];
        have_node = true;
    }
}

}  // namespace ohao
