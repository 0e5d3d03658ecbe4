// pt_fetch.cuh -- BVH traversal (flat or two-level) as resumable state
// machines, for persistent warps that refill finished lanes from a ray queue.
//
// One *_step call does one unit of work of the traversal of scene_closest /
// scene_occluded -- a node test, ONE triangle test, an instance entry or a
// stack pop -- in the same per-ray order of node visits (a BLAS node's
// triangle leaves are tested, one per step, before the next node). Steps are
// short and of similar cost, so the lanes of a warp that are at different
// points of their traversals waste little issue time on each other, and a
// lane can stop after any step: a new ray starts in it while the others are
// mid-traversal, so a warp no longer waits for its longest ray.
//
// The result does not depend on how the steps of different rays interleave:
// each ray's state is its own, node culling is conservative (entry distance
// against the best hit with a relative slack) and equal distances go to the
// smaller (instance, primitive) key, so the closest hit is the minimum of
// (t, instance, primitive) over the intersected triangles -- the hit that
// scene_closest returns for the same ray.
#pragma once

namespace ohao {

constexpr uint32_t kNoHit = 0xFFFFFFFFu;

// closest-hit state of one ray. kLevels 1: flat BVH (walked as one BLAS
// whose triangle records carry their instance), 2: two-level.
struct Walk {
    RayPre ra;                   // ray of the current level (object space inside a BLAS)
    Hit best;
    const uint4* bnodes;
    const float4* btris;
    uint4 pq;                    // pending instance leaves of the last TLAS node: (child, leaf, meta, meta)
    uint32_t inst, cur, res_cur, plm, pidx;
    uint32_t tbase, tmz, tmw, tlm, tq;   // pending triangle leaves of the last BLAS node
    float cur_tn, res_tn;
    int sp, base;
    bool in_blas, have_node, resume;
};

template <int kLevels>
OHAO_D void walk_begin(const DScene& sc, Walk& w, const RayPre& r) {
    w.ra = r;
    w.best.t = 0.0f; w.best.u = 0.0f; w.best.v = 0.0f;
    w.best.inst = kNoHit; w.best.prim = kNoHit;
    w.bnodes = nullptr;
    w.btris = nullptr;
    w.pq = make_uint4(0, 0, 0, 0);
    w.inst = 0u; w.cur = 0u; w.res_cur = 0u; w.plm = 0u; w.pidx = 0u;
    w.tbase = 0u; w.tmz = 0u; w.tmw = 0u; w.tlm = 0u; w.tq = 0u;
    w.cur_tn = -INFINITY; w.res_tn = 0.0f;
    w.sp = 0; w.base = 0;
    w.in_blas = false; w.have_node = true; w.resume = false;
    if (kLevels == 1) {
        w.in_blas = true;
        w.bnodes = sc.nodes;
        w.btris = sc.tris;
    }
}

// Enters the next pending instance leaf of w.pq/w.plm (or skips an empty
// slot). r: the world-space ray.
OHAO_D void enter_instance(const DScene& sc, const RayPre& r, const uint4& pq, uint32_t& plm, uint32_t& pidx,
                           RayPre& ra, const uint4*& bnodes, const float4*& btris, uint32_t& inst, bool& entered) {
    const int i = __ffs(plm) - 1;
    const uint32_t meta = byte_of(pq.z, pq.w, i);
    const uint32_t c = meta >> 5, off = meta & 31u;
    entered = false;
    if (pidx >= c) {
        plm &= plm - 1;
        pidx = 0u;
        return;
    }
    const uint32_t ii = __ldg(sc.tlas_inst + pq.y + off + pidx);
    if (++pidx == c) {
        plm &= plm - 1;
        pidx = 0u;
    }
    const DInst& in = sc.inst[ii];
    const DBlas bl = sc.blas[in.blas];
    V3 oo, od;
    xform_point(in.w2o, V3{r.o[0], r.o[1], r.o[2]}, oo);
    xform_dir(in.w2o, V3{r.d[0], r.d[1], r.d[2]}, od);
    ra = ray_pre(oo, od);
    bnodes = sc.blas_nodes + static_cast<size_t>(bl.node_off) * 5;
    btris = sc.blas_tris + static_cast<size_t>(bl.tri_off) * 3;
    inst = ii;
    entered = true;
}

// One step of the closest-hit walk; true when the ray is finished (w.best
// holds its hit). r: the world-space ray. Stack overflow sets err and ends
// the walk.
template <int kLevels, bool kStats = false, bool kAlpha = false>
OHAO_D bool walk_step(const DScene& sc, Walk& w, const RayPre& r, float tmin, float tmax, uint32_t* st_node,
                      float* st_t, int& err, TravCount* cnt = nullptr) {
    if (w.tlm) {   // one pending triangle
        const int i = __ffs(w.tlm) - 1;
        const uint32_t meta = byte_of(w.tmz, w.tmw, i);
        const uint32_t c = meta >> 5, off = meta & 31u;
        if (w.tq < c) {
            const float4* tp = w.btris + static_cast<size_t>(w.tbase + off + w.tq) * 3;
            const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            if (kStats) cnt->tris++;
            float t, u, v;
            const bool h = tri_intersect(w.ra, v0, v1, v2, tmin, tmax, t, u, v);
            const uint32_t prim = __float_as_uint(v0.w);
            const uint32_t inst = kLevels == 1 ? __float_as_uint(v1.w) : w.inst;
            if (h && (!kAlpha || !sc.alpha_test || alpha_accept(sc, inst, prim, u, v))) {
                if (w.best.prim == kNoHit || t < w.best.t ||
                    (t == w.best.t && key_less(inst, prim, w.best.inst, w.best.prim))) {
                    w.best.t = t; w.best.u = u; w.best.v = v; w.best.inst = inst; w.best.prim = prim;
                }
            }
        }
        if (++w.tq >= c) {
            w.tlm &= w.tlm - 1;
            w.tq = 0u;
        }
        return false;
    }
    if (w.have_node) {
        const float tb = w.best.prim != kNoHit ? w.best.t : tmax;
        bool desc = false;
        bool leaves = false;
        if (w.cur_tn <= tb + tb * kTravRelSlack) {
            const NodeRec n = load_node(w.in_blas ? w.bnodes : sc.nodes, w.cur);
            if (kStats) cnt->nodes++;
            float tn[8];
            const uint32_t hit = node_test(n, w.ra, tmin, tb, tn);
            const uint32_t imask = n.q0.w >> 24;
            const uint32_t lm = hit & ~imask;
            if (kLevels == 1 || w.in_blas) {   // its triangle leaves, one triangle per step, before the next node
                w.tbase = n.q1.y;
                w.tmz = n.q1.z;
                w.tmw = n.q1.w;
                w.tlm = lm;
                w.tq = 0u;
            } else if (lm) {
                w.pq = n.q1;
                w.plm = lm;
                w.pidx = 0u;
                leaves = true;
            }
            const uint32_t rem = hit & imask;
            if (rem) {
                ArrStack ast{st_node, st_t};
                if (!order_children(rem, tn, n, ast, w.sp, w.cur, w.cur_tn, stack_limit(sc))) {
                    err = 1;
                    return true;
                }
                desc = true;
            }
        }
        if (leaves) {
            w.resume = desc;
            w.res_cur = w.cur;
            w.res_tn = w.cur_tn;
            w.have_node = false;
        } else if (!desc) {
            w.have_node = false;
        }
        if (w.have_node || w.tlm) return false;   // pending triangles run in this BLAS before any pop
    }
    if (w.in_blas) {
        if (w.sp > w.base) {
            w.sp--;
            w.cur = st_node[w.sp];
            w.cur_tn = st_t[w.sp];
            w.have_node = true;
            return false;
        }
        if (kLevels == 1) return true;
        w.in_blas = false;
        w.ra = r;
    }
    if (w.plm) {
        bool entered;
        enter_instance(sc, r, w.pq, w.plm, w.pidx, w.ra, w.bnodes, w.btris, w.inst, entered);
        if (entered) {
            w.base = w.sp;
            if (w.base >= stack_limit(sc)) { err = 1; return true; }
            w.cur = 0u;
            w.cur_tn = -INFINITY;
            w.in_blas = true;
            w.have_node = true;
        }
        return false;
    }
    if (w.resume) {
        w.resume = false;
        w.cur = w.res_cur;
        w.cur_tn = w.res_tn;
        w.have_node = true;
        return false;
    }
    if (w.sp == 0) return true;
    w.sp--;
    w.cur = st_node[w.sp];
    w.cur_tn = st_t[w.sp];
    w.have_node = true;
    return false;
}

// any-hit state of one ray (kLevels as for Walk)
struct Probe {
    RayPre ra;
    const uint4* bnodes;
    const float4* btris;
    uint4 pq;
    uint32_t inst, cur, res_cur, plm, pidx;
    uint32_t tbase, tmz, tmw, tlm, tq;
    int sp, base;
    bool in_blas, have_node, resume, hit;
};

template <int kLevels>
OHAO_D void probe_begin(const DScene& sc, Probe& w, const RayPre& r) {
    w.ra = r;
    w.bnodes = nullptr;
    w.btris = nullptr;
    w.pq = make_uint4(0, 0, 0, 0);
    w.inst = 0u; w.cur = 0u; w.res_cur = 0u; w.plm = 0u; w.pidx = 0u;
    w.tbase = 0u; w.tmz = 0u; w.tmw = 0u; w.tlm = 0u; w.tq = 0u;
    w.sp = 0; w.base = 0;
    w.in_blas = false; w.have_node = true; w.resume = false; w.hit = false;
    if (kLevels == 1) {
        w.in_blas = true;
        w.bnodes = sc.nodes;
        w.btris = sc.tris;
    }
}

// One step of the any-hit walk; true when finished (w.hit: occluded).
template <int kLevels, bool kStats = false, bool kAlpha = false>
OHAO_D bool probe_step(const DScene& sc, Probe& w, const RayPre& r, float tmin, float tmax, uint32_t* st_node,
                       int& err, TravCount* cnt = nullptr) {
    if (w.tlm) {   // one pending triangle
        const int i = __ffs(w.tlm) - 1;
        const uint32_t meta = byte_of(w.tmz, w.tmw, i);
        const uint32_t c = meta >> 5, off = meta & 31u;
        if (w.tq < c) {
            const float4* tp = w.btris + static_cast<size_t>(w.tbase + off + w.tq) * 3;
            const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            if (kStats) cnt->tris++;
            float t, u, v;
            if (tri_intersect(w.ra, v0, v1, v2, tmin, tmax, t, u, v) &&
                (!kAlpha || !sc.alpha_test ||
                 alpha_accept(sc, kLevels == 1 ? __float_as_uint(v1.w) : w.inst, __float_as_uint(v0.w), u, v))) {
                w.hit = true;
                return true;
            }
        }
        if (++w.tq >= c) {
            w.tlm &= w.tlm - 1;
            w.tq = 0u;
        }
        return false;
    }
    if (w.have_node) {
        const NodeRec n = load_node(w.in_blas ? w.bnodes : sc.nodes, w.cur);
        if (kStats) cnt->nodes++;
        float tn[8];
        uint32_t m = node_test(n, w.ra, tmin, tmax, tn);
        const uint32_t imask = n.q0.w >> 24;
        bool have = false;
        uint32_t next = 0u;
        if (kLevels == 2 && !w.in_blas) {
            w.plm = m & ~imask;
            w.pq = n.q1;
            w.pidx = 0u;
        } else {   // triangle leaves, one triangle per step, before the next node
            w.tbase = n.q1.y;
            w.tmz = n.q1.z;
            w.tmw = n.q1.w;
            w.tlm = m & ~imask;
            w.tq = 0u;
        }
        m &= imask;
        while (m) {
            const int i = __ffs(m) - 1;
            m &= m - 1;
            if (have) {
                if (w.sp >= stack_limit(sc)) { err = 1; return true; }
                st_node[w.sp++] = next;
            }
            next = n.q1.x + (byte_of(n.q1.z, n.q1.w, i) & 7u);
            have = true;
        }
        if (kLevels == 2 && !w.in_blas && w.plm) {
            w.resume = have;
            w.res_cur = next;
            w.have_node = false;
        } else if (have) {
            w.cur = next;
            return false;
        } else {
            w.have_node = false;
        }
        if (w.tlm) return false;   // pending triangles run in this BLAS before any pop
    }
    if (w.in_blas) {
        if (w.sp > w.base) {
            w.cur = st_node[--w.sp];
            w.have_node = true;
            return false;
        }
        if (kLevels == 1) return true;
        w.in_blas = false;
        w.ra = r;
    }
    if (w.plm) {
        bool entered;
        enter_instance(sc, r, w.pq, w.plm, w.pidx, w.ra, w.bnodes, w.btris, w.inst, entered);
        if (entered) {
            w.base = w.sp;
            if (w.base >= stack_limit(sc)) { err = 1; return true; }
            w.cur = 0u;
            w.in_blas = true;
            w.have_node = true;
        }
        return false;
    }
    if (w.resume) {
        w.resume = false;
        w.cur = w.res_cur;
        w.have_node = true;
        return false;
    }
    if (w.sp == 0) return true;
    w.cur = st_node[--w.sp];
    w.have_node = true;
    return false;
}

}  // namespace ohao
