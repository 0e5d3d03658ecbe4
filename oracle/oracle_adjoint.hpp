// oracle_adjoint.hpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// The detached-sampling path estimator that the device path-replay gradient
// differentiates, evaluated in FP64. Every sampling decision of a path --
// camera jitter, light choice and sample point, environment sample,
// lobe choice, jittered specular and cosine directions, the Russian-roulette
// probability and the lobe-selection divisor -- is taken exactly as the FP32
// forward estimator takes it with the scene's own parameters theta_s (the
// float tracer below, bit-identical to pt_raygen.rgen restated in
// oracle_pt.hpp). Every value that the parameters enter -- albedo factors of
// the throughput, BRDF values, the MIS pdfs -- is evaluated in double with a
// second parameter set theta_e (material table and tile albedo map). At
// theta_e == theta_s the result is the forward estimator's radiance; its
// derivative in theta_e is what the adjoint returns, so central finite
// differences of this function in theta_e check the device gradient without
// the discontinuities that re-sampling would add.
//
// Instantiated with D = Dd (below), a forward-mode dual number in double
// with one slot per selected parameter, the same code gives the analytic
// FP64 gradient of the estimator -- the host gradient the device adjoint is
// compared with besides the finite differences.
#pragma once
#include <type_traits>

#include "oracle_pt.hpp"

namespace orc {

constexpr int kGradSlots = 40;

// value + gradient over kGradSlots parameters
struct Dd {
    double v = 0.0;
    double d[kGradSlots] = {};
    Dd() = default;
    Dd(double x) : v(x) {}   // NOLINT: constants convert implicitly
    static Dd var(double x, int slot) {
        Dd r(x);
        if (slot >= 0) r.d[slot] = 1.0;
        return r;
    }
};
inline Dd operator+(const Dd& a, const Dd& b) { Dd r(a.v + b.v); for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
inline Dd operator-(const Dd& a, const Dd& b) { Dd r(a.v - b.v); for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
inline Dd operator-(const Dd& a) { Dd r(-a.v); for (int i = 0; i < kGradSlots; ++i) r.d[i] = -a.d[i]; return r; }
inline Dd operator*(const Dd& a, const Dd& b) {
    Dd r(a.v * b.v);
    for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
inline Dd operator/(const Dd& a, const Dd& b) {
    Dd r(a.v / b.v);
    for (int i = 0; i < kGradSlots; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
    return r;
}
inline Dd operator*(const Dd& a, double s) { Dd r(a.v * s); for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] * s; return r; }
inline Dd operator*(double s, const Dd& a) { return a * s; }
inline Dd operator/(const Dd& a, double s) { Dd r(a.v / s); for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] / s; return r; }
inline Dd operator+(const Dd& a, double s) { Dd r = a; r.v += s; return r; }
inline Dd operator+(double s, const Dd& a) { return a + s; }
inline Dd operator-(const Dd& a, double s) { Dd r = a; r.v -= s; return r; }
inline Dd operator-(double s, const Dd& a) { Dd r = -a; r.v += s; return r; }
inline bool operator<(const Dd& a, const Dd& b) { return a.v < b.v; }
inline bool operator>(const Dd& a, const Dd& b) { return a.v > b.v; }
inline bool operator<=(const Dd& a, const Dd& b) { return a.v <= b.v; }
inline bool operator>=(const Dd& a, const Dd& b) { return a.v >= b.v; }
inline Dd m_sqrt(const Dd& a) {
    Dd r(std::sqrt(a.v));
    for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] * (0.5 / r.v);
    return r;
}
inline double value_of(double x) { return x; }
inline double value_of(const Dd& x) { return x.v; }

template <class D>
struct DetachedPathT {
    const Scene& sc;
    const Settings& st;
    const float* mats_e;   // 12 floats per material
    const float* map_e;    // map_h x map_w x 3, or null when the scene has none
    const int32_t* rough_slot = nullptr;   // per material: dual slot of its roughness, or -1
    const int32_t* map_slot = nullptr;     // per map entry (texel*3 + c): dual slot, or -1
    // With duals: add the score terms of the sampling decisions whose density
    // the estimator's weight does not contain (specular jitter, clamped or
    // forced lobe choice), so that the derivative is that of the expectation.
    bool with_score = false;
    PathTracer<float> tf;

    DetachedPathT(const Scene& s, const Settings& t, const float* me, const float* ma)
        : sc(s), st(t), mats_e(me), map_e(ma), tf(s, t) {}

    static V3<D> dv(V3<float> a) { return V3<D>(a); }
    static constexpr double PI = double(3.14159265358979f);
    static D absv(D x) { return x < D(0) ? -x : x; }
    static D param(float x, const int32_t* slots, size_t i) {
        if constexpr (std::is_same_v<D, double>) {
            (void)slots; (void)i;
            return D(x);
        } else {
            return D::var(double(x), slots ? slots[i] : -1);
        }
    }

    struct Eval {
        V3<D> alb;
        D rough, metal;
        int rough_slot_id = -1;   // dual slot of this material's roughness when it is above its floor
    };

    // score bookkeeping (duals only): S carries d log(sampling density) for
    // the decisions taken so far on the chain, with value 0
    V3<D> sc_(const V3<D>& c, const D& S) const {
        if constexpr (std::is_same_v<D, double>) {
            (void)S;
            return c;
        } else {
            return with_score ? c + c * S : c;
        }
    }
    static void add_slot(D& S, int slot, double val) {
        if constexpr (!std::is_same_v<D, double>) {
            if (slot >= 0) S.d[slot] += val;
        } else {
            (void)S; (void)slot; (void)val;
        }
    }
    // d log p with value 0, sign +1 or -1 (p or 1 - p)
    static void add_dlog(D& S, const D& p, double sign, double pval) {
        if constexpr (!std::is_same_v<D, double>) {
            for (int i = 0; i < kGradSlots; ++i) S.d[i] += sign * p.d[i] / pval;
        } else {
            (void)S; (void)p; (void)sign; (void)pval;
        }
    }
    // d log q(w | r) / d r of the jittered specular direction, t = h.R
    static double jitter_score(V3<float> refl, V3<float> h, float rough) {
        const double t = std::max(double(dot(h, refl)), 1e-12), r = rough, tr = t + r;
        return (1.0 - t * t) / (t * tr * tr) + 2.0 / tr - 2.0 / r;
    }
    // PathTracer::spec_dir (pt_raygen.rgen:516-525) with the jitter score
    V3<float> spec_dir_s(Sampler& smp, uint32_t& dim, V3<float> inDir, V3<float> N, float rough, double& js) const {
        V3<float> refl = reflect(inDir, N);
        js = 0.0;
        if (rough > 0.01f) {
            const float j0 = smp.s1(dim), j1 = smp.s1(dim + 1);
            dim += 2;
            const V3<float> h = tf.cos_hemi(refl, j0, j1);
            js = jitter_score(refl, h, rough);
            const V3<float> jit = h * rough;
            refl = normalize(refl + jit);
            if (dot(refl, N) < 0.0f) {
                const float f0 = smp.s1(dim), f1 = smp.s1(dim + 1);
                dim += 2;
                refl = tf.cos_hemi(N, f0, f1);
            }
        }
        return refl;
    }

    // theta_e surface parameters at a hit (pt_closesthit.rchit:104-150 and
    // diff_map.hpp:40-67 in double; metalness is not a parameter).
    Eval eval_surface(const Surf<float>& s) const {
        Eval e;
        const float* m = mats_e + static_cast<size_t>(s.matid) * 12;
        e.alb = V3<D>(D(m[0]), D(m[1]), D(m[2]));
        if (f2u(sc.mats[static_cast<size_t>(s.matid) * 12 + 3]) == 0u && sc.map_w > 0 && map_e) {
            const int w = static_cast<int>(sc.map_w), h = static_cast<int>(sc.map_h);
            const float u = gclamp(s.uv[0], 0.0f, 1.0f), v = gclamp(s.uv[1], 0.0f, 1.0f);
            const float x = u * float(w - 1), y = v * float(h - 1);
            const int x0 = static_cast<int>(x), y0 = static_cast<int>(y);
            const int x1 = std::min(x0 + 1, w - 1), y1 = std::min(y0 + 1, h - 1);
            const D tx = D(x - float(x0)), ty = D(y - float(y0));
            D out[3];
            for (int c = 0; c < 3; ++c) {
                auto at = [&](int ix, int iy) {
                    const size_t k = (static_cast<size_t>(iy) * w + ix) * 3 + c;
                    return param(map_e[k], map_slot, k);
                };
                const D a = at(x0, y0) * (1 - tx) + at(x1, y0) * tx;
                const D b = at(x0, y1) * (1 - tx) + at(x1, y1) * tx;
                out[c] = a * (1 - ty) + b * ty;
            }
            e.alb = e.alb * V3<D>(out[0], out[1], out[2]);
        }
        D r = gmax(param(m[4], rough_slot, s.matid), D(0.04f));
        if (rough_slot && m[4] > 0.04f && m[4] < 10.0f) e.rough_slot_id = rough_slot[s.matid];
        if (r >= D(10)) r = r - D(10);
        e.rough = gmax(r, D(0.01f));
        e.metal = D(s.metal);
        return e;
    }

    D ggx_inline(D NdotH, D rough, double pi) const {
        const D a = rough * rough, a2 = a * a;
        const D denom = NdotH * NdotH * (a2 - 1) + 1;
        return a2 / (pi * denom * denom + D(0.0001f));
    }
    // GGX D of the first hit, isotropic or anisotropic (ggx_aniso.glsl:31-55)
    D ggx_first(V3<D> N, V3<D> H, D NdotH, D rough) const {
        const double an = st.aniso;
        if (an < double(0.001f)) return ggx_inline(NdotH, rough, double(3.14159265f));
        const V3<D> up(D(0), D(1), D(0));
        const V3<D> ref = absv(dot(up, N)) > D(0.97f) ? V3<D>(D(1), D(0), D(0)) : up;
        const V3<D> T = normalize(ref - N * dot(ref, N));
        const V3<D> B = cross(N, T);
        const D c = D(std::cos(double(st.aniso_rot))), s = D(std::sin(double(st.aniso_rot)));
        const V3<D> Tr = T * c + B * s;
        const V3<D> Br = B * c - T * s;
        const D r2 = rough * rough;
        const D aspect = D(std::sqrt(1.0 - an * double(0.9f)));
        const D rT = gmax(r2 / aspect, D(0.001f));
        const D rB = gmax(r2 * aspect, D(0.001f));
        const D TdotH = dot(Tr, H), BdotH = dot(Br, H);
        const D dd = (TdotH * TdotH / rT) + (BdotH * BdotH / rB) + NdotH * NdotH;
        return D(1) / (double(3.14159265f) * rT * rB * dd * dd + D(0.0001f));
    }

    struct Brdf {
        V3<D> f;
        D D_, NdotH, VdotH;
    };
    Brdf brdf(V3<D> N, V3<D> inDir, V3<D> L, D NdotL, const Eval& e, bool bounce0, double pi_chain,
              double pi_diff) const {
        const V3<D> V = normalize(-inDir);
        const V3<D> H = normalize(L + V);
        Brdf b;
        b.NdotH = gmax(dot(N, H), D(0.001f));
        const D NdotV = gmax(dot(N, V), D(0.001f));
        b.VdotH = gmax(dot(V, H), D(0.001f));
        b.D_ = bounce0 ? ggx_first(N, H, b.NdotH, e.rough) : ggx_inline(b.NdotH, e.rough, pi_chain);
        const V3<D> F0 = vmix(V3<D>(D(0.04f)), e.alb, e.metal);
        const V3<D> F = F0 + (D(1) - F0) * pow5(D(1) - b.VdotH);
        const D k = (e.rough + 1) * (e.rough + 1) / 8;
        const D G = (NdotL / (NdotL * (1 - k) + k)) * (NdotV / (NdotV * (1 - k) + k));
        const V3<D> spec = b.D_ * F * G / (4 * NdotV * NdotL + D(0.001f));
        const V3<D> diff = (D(1) - F) * (1 - e.metal) * e.alb / D(pi_diff);
        b.f = diff + spec;
        return b;
    }

    // specular-lobe selection probability (pt_raygen.rgen:775-779)
    D sel_prob(V3<D> inDir, V3<D> N, const Eval& e) const {
        const D cosI = absv(dot(normalize(inDir), N));
        const V3<D> F0 = vmix(V3<D>(D(0.04f)), e.alb, e.metal);
        const V3<D> fres = F0 + (D(1) - F0) * pow5(D(1) - cosI);
        const D sp = maxc(fres) * (1 - e.rough * D(0.9f));
        return gmix(sp, D(1), e.metal);
    }

    D spec_pdf(V3<D> N, V3<D> inDir, V3<D> outDir, const Eval& e, bool bounce0) const {
        const V3<D> Hs = normalize(-inDir + outDir);
        const D NdotHs = gmax(dot(N, Hs), D(0.001f));
        const D VdotHs = gmax(dot(-inDir, Hs), D(0.001f));
        const D Ds = bounce0 ? ggx_first(N, Hs, NdotHs, e.rough) : ggx_inline(NdotHs, e.rough, PI);
        return Ds * NdotHs / (4 * VdotHs + D(1e-4f));
    }

    // Light NEE and env NEE at a vertex: draws and visibility in float,
    // values with theta_e. Returns the light added without throughput.
    V3<D> nee(Sampler& smp, uint32_t& dim, const Surf<float>& s, V3<float> inDir, const Eval& e, bool bounce0) const {
        V3<D> g(D(0));
        const V3<float> P = s.hitPos, N = s.N;
        const V3<D> Nd = dv(N), inD = dv(inDir);
        if (!sc.lights.empty()) {
            const auto ls = tf.sample_light(smp, dim, P, N);
            Surf<float> sh;
            if (ls.valid && tf.shadow(P + N * 0.01f, ls.L, ls.shadowDist, sh, nullptr)) {
                const D NdotL = D(ls.NdotL);
                const Brdf b = brdf(Nd, inD, dv(ls.L), NdotL, e, bounce0, double(3.14159f), double(3.14159f));
                g = g + dv(ls.Le) * b.f * NdotL * D(ls.weight) * D(ls.n);
            }
        }
        if (sc.has_cdf) {
            const float u1 = smp.s1(dim), u2 = smp.s1(dim + 1);
            dim += 2;
            V3<float> dir;
            float pdf;
            tf.sample_env(u1, u2, dir, pdf);
            const float NdotLf = gmax(dot(N, dir), 0.0f);
            Surf<float> sh;
            if (NdotLf > 0.0f && pdf > 0.0f && tf.shadow(P + N * 0.01f, dir, 10000.0f, sh, nullptr)) {
                const D NdotL = D(NdotLf);
                const Brdf b = brdf(Nd, inD, dv(dir), NdotL, e, bounce0, PI, PI);
                const D sp = sel_prob(inD, Nd, e);
                const D pdfS = b.D_ * b.NdotH / (4 * b.VdotH + D(1e-4f));
                const D bsdfPdf = gmix(NdotL / PI, pdfS, sp);
                const D w = D(pdf) / gmax(D(pdf) + bsdfPdf, D(1e-6f));
                g = g + dv(sh.color) * b.f * NdotL * w / D(pdf);
            }
        }
        return g;
    }

    void chain(Sampler& smp, uint32_t& dim, bool specChain, V3<float> ro, V3<float> rd, V3<float> thrS, V3<D> thrE,
               D lastPdf, bool lastDelta, D S, V3<D>& rad) const {
        for (uint32_t bounce = 1; bounce <= st.max_bounces; ++bounce) {
            Surf<float> s;
            tf.trace(ro, rd, s, nullptr);
            if (!s.hit) {
                D w = 1;
                if (s.envPdf > 0.0f && sc.has_cdf && !lastDelta) w = lastPdf / gmax(lastPdf + D(s.envPdf), D(1e-6f));
                rad = rad + sc_(thrE * dv(s.color) * w, S);
                break;
            }
            const Eval e = eval_surface(s);
            const V3<float> P = s.hitPos, N = s.N;
            const V3<D> Nd = dv(N);
            if (length(s.color) > 0.001f) rad = rad + sc_(thrE * dv(s.color), S);
            rad = rad + sc_(thrE * nee(smp, dim, s, rd, e, false), S);
            if (bounce > 1) {   // survival probability min(p, 1), divisor p
                const float p = maxc(thrS);
                const float rr = smp.s1(dim);
                dim += 1;
                if (p < 0.01f || rr > p) break;
                if (p > 1.0f) {   // the divisor is a value of the throughput: maxc(T)
                    const int cm = (thrS.x >= thrS.y && thrS.x >= thrS.z) ? 0 : (thrS.y >= thrS.z ? 1 : 2);
                    thrE = thrE / thrE[cm];
                } else {
                    thrE = thrE / D(p);
                }
                thrS = thrS / p;
            }
            const float bR = s.rough, bM = s.metal;
            const V3<float> bF0 = vmix(V3<float>(0.04f), s.albedo, bM);
            const float cosI = std::fabs(dot(normalize(rd), N));
            const V3<float> fres = bF0 + (1.0f - bF0) * pow5(1.0f - cosI);
            float sp = maxc(fres);
            sp = sp * (1.0f - bR * 0.9f);
            sp = gmix(sp, 1.0f, bM);
            const float choice = smp.s1(dim);
            dim += 1;
            const D spE = sel_prob(dv(rd), Nd, e);
            // lobe choice: probability P_b, divisor max(P, 0.01); score d log P_b - d log div_b
            if (bR < 0.05f) {
                if (sp > 0.01f) add_dlog(S, spE, -1.0, value_of(spE));
            } else if (choice < sp) {
                if (sp < 0.01f) add_dlog(S, spE, 1.0, value_of(spE));
            } else if (1.0f - sp < 0.01f) {
                add_dlog(S, spE, -1.0, 1.0 - value_of(spE));
            }
            if (choice < sp || bR < 0.05f) {
                const V3<float> inDir = rd;
                double js;
                rd = spec_dir_s(smp, dim, rd, N, bR, js);
                add_slot(S, e.rough_slot_id, js);
                ro = P + N * 0.01f;
                if (specChain) {
                    thrS = thrS * vmix(V3<float>(1.0f), s.albedo, bM);
                    thrE = thrE * vmix(V3<D>(D(1)), e.alb, e.metal);
                } else {
                    thrS = thrS * (s.albedo * (1.0f - bM));
                    thrE = thrE * (e.alb * (1 - e.metal));
                }
                thrS = thrS / gmax(sp, 0.01f);
                thrE = thrE / D(gmax(sp, 0.01f));
                if (bR < 0.05f) {
                    lastPdf = 1;
                    lastDelta = true;
                } else {
                    lastPdf = spE * spec_pdf(Nd, dv(inDir), dv(rd), e, false);
                    lastDelta = false;
                }
            } else {
                const float d0 = smp.s1(dim), d1 = smp.s1(dim + 1);
                dim += 2;
                rd = tf.cos_hemi(N, d0, d1);
                ro = P + N * 0.01f;
                thrS = thrS * s.albedo;
                thrS = thrS / gmax(1.0f - sp, 0.01f);
                thrE = thrE * e.alb / D(gmax(1.0f - sp, 0.01f));
                lastPdf = (1 - spE) * gmax(dot(dv(rd), Nd), D(0)) / PI;
                lastDelta = false;
            }
        }
    }

    // One path (pt_raygen.rgen main(), stages A/B/C) without the firefly clamp.
    V3<D> path(const View& vw, uint32_t px, uint32_t py, uint32_t sidx) const {
        Sampler smp;
        smp.init(st.sampler, px, py, sidx);
        uint32_t dim = 0;
        const V3<float> rd = tf.camera_dir(vw, px, py, smp, dim);
        const V3<float> ro(vw.inv_view[12], vw.inv_view[13], vw.inv_view[14]);
        Surf<float> s;
        tf.trace(ro, rd, s, nullptr);
        if (!s.hit) return dv(s.color);
        const Eval e = eval_surface(s);
        const V3<float> P = s.hitPos, N = s.N;
        const V3<D> Nd = dv(N);
        V3<D> rad(D(0));
        if (length(s.color) > 0.001f) rad = rad + dv(s.color);
        rad = rad + nee(smp, dim, s, rd, e, true);
        // stage B
        double js0;
        const V3<float> sd = spec_dir_s(smp, dim, rd, N, s.rough, js0);
        D SB = D(0);
        add_slot(SB, e.rough_slot_id, js0);
        const V3<float> thrSB = vmix(V3<float>(1.0f), s.albedo, s.metal);
        const V3<D> thrEB = vmix(V3<D>(D(1)), e.alb, e.metal);
        const bool deltaB = s.rough < 0.05f;
        const D pdfB = deltaB ? D(1) : spec_pdf(Nd, dv(rd), dv(sd), e, true);
        chain(smp, dim, true, P + N * 0.01f, sd, thrSB, thrEB, pdfB, deltaB, SB, rad);
        // stage C
        const float d0 = smp.s1(dim), d1 = smp.s1(dim + 1);
        dim += 2;
        const V3<float> dd = tf.cos_hemi(N, d0, d1);
        const D pdfC = gmax(dot(dv(dd), Nd), D(0)) / PI;
        chain(smp, dim, false, P + N * 0.01f, dd, s.albedo, e.alb, pdfC, false, D(0), rad);
        return rad;
    }
};

using DetachedPath = DetachedPathT<double>;

}  // namespace orc
