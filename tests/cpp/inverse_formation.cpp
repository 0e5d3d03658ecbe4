// A C++ caller of the C ABI through include/ohao_pt_inverse.hpp, the way the
// reference's inverse lab would use it behind IInverseImageFormation
// (ohao/inverse/backend/image_formation.hpp:40-60): forward renders of RGBA8
// display images, then a fit of a tile albedo map to a target image driven by
// the analytic gradient of the display-space loss (mseRGB,
// ohao/inverse/image_loss.hpp:59-80) instead of coordinate finite
// differences. Prints "ok" and returns 0 when every check holds.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "ohao_pt.h"
#include "ohao_pt_inverse.hpp"

namespace {

int g_fail = 0;
void check(bool ok, const char* what) {
    if (!ok) {
        std::printf("FAILED: %s\n", what);
        g_fail = 1;
    }
}
bool ok(ohao_status s, ohao_pt_ctx* ctx, const char* what) {
    if (s != OHAO_OK) {
        std::printf("FAILED: %s -> %d (%s)\n", what, s, ctx ? ohao_pt_last_error(ctx) : "");
        g_fail = 1;
        return false;
    }
    return true;
}

// Column-major camera-to-world and inverse projection of a look-at camera
// (right-handed, -Z forward, Vulkan's y flip), 40 degree vertical field of view.
ohao_gb300::Camera look_at(const double eye[3], const double at[3], uint32_t w, uint32_t h) {
    double f[3] = {at[0] - eye[0], at[1] - eye[1], at[2] - eye[2]};
    double n = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& x : f) x /= n;
    const double up[3] = {0.0, 0.0, -1.0};
    double r[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double& x : r) x /= n;
    const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    ohao_gb300::Camera c{};
    for (int k = 0; k < 3; ++k) {
        c.inv_view[0 * 4 + k] = static_cast<float>(r[k]);
        c.inv_view[1 * 4 + k] = static_cast<float>(u[k]);
        c.inv_view[2 * 4 + k] = static_cast<float>(-f[k]);
        c.inv_view[3 * 4 + k] = static_cast<float>(eye[k]);
    }
    c.inv_view[15] = 1.0f;
    const double t = std::tan(20.0 * 3.14159265358979323846 / 180.0), aspect = double(w) / h;
    const double nearp = 0.01, farp = 1000.0;
    const double p00 = 1.0 / (aspect * t), p11 = -1.0 / t, p22 = farp / (nearp - farp), p23 = farp * nearp / (nearp - farp);
    // inverse of [[p00,0,0,0],[0,p11,0,0],[0,0,p22,p23],[0,0,-1,0]] (row-major), stored column-major
    double inv[4][4] = {{1.0 / p00, 0, 0, 0}, {0, 1.0 / p11, 0, 0}, {0, 0, 0, -1.0}, {0, 0, 1.0 / p23, p22 / p23}};
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) c.inv_proj[col * 4 + row] = static_cast<float>(inv[row][col]);
    return c;
}

double mse_rgb(const std::vector<uint8_t>& a, const std::vector<uint8_t>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); i += 4)
        for (int c = 0; c < 3; ++c) {
            const double d = (double(a[i + c]) - b[i + c]) / 255.0;
            s += d * d;
        }
    return s / double(a.size() / 4 * 3);
}

}  // namespace

int main() {
    ohao_pt_desc desc{0, 0, 0};
    ohao_pt_ctx* ctx = nullptr;
    if (!ok(ohao_pt_create(&desc, &ctx), nullptr, "create")) return 1;
    // a 2x2 floor quad at y = 0 with UVs over [0,1]^2, lit by a constant sky
    const float pos[12] = {-1, 0, -1, 1, 0, -1, 1, 0, 1, -1, 0, 1};
    const float nrm[16] = {0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0};
    const float uv[8] = {0, 0, 1, 0, 1, 1, 0, 1};
    const uint32_t idx[6] = {0, 2, 1, 0, 3, 2};
    const uint32_t mid[2] = {0, 0};
    ok(ohao_pt_set_geometry(ctx, pos, 12, 4, nrm, uv, idx, 2, mid), ctx, "set_geometry");
    uint32_t blas = 0;
    ok(ohao_pt_create_blas(ctx, 0, 6, &blas), ctx, "create_blas");
    ohao_pt_instance inst{};
    inst.blas = blas;
    inst.transform[0] = inst.transform[5] = inst.transform[10] = 1.0f;
    inst.mask = 0xFF;
    ok(ohao_pt_set_instances(ctx, &inst, 1), ctx, "set_instances");
    float mat[12] = {1, 1, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0};   // albedo 1, roughness 1, dielectric
    const uint32_t tex0 = 0u, none = 0xFFFFFFFFu;         // diffuse texture 0 = the tile albedo map
    std::memcpy(&mat[3], &tex0, 4);
    std::memcpy(&mat[6], &none, 4);
    std::memcpy(&mat[7], &none, 4);
    std::memcpy(&mat[8], &none, 4);
    ok(ohao_pt_set_materials(ctx, mat, 1), ctx, "set_materials");
    const uint32_t ew = 16, eh = 8;
    std::vector<float> env(ew * eh * 4, 1.0f), marg(eh), cond(ew * eh);
    float integral = 0.0f;
    ok(ohao_env_cdf_build(env.data(), ew, eh, marg.data(), cond.data(), &integral), ctx, "env_cdf_build");
    ok(ohao_pt_set_env(ctx, env.data(), ew, eh, marg.data(), cond.data(), integral, 1.0f), ctx, "set_env");
    const uint32_t mw = 4, mh = 4;
    std::vector<float> map_true(mw * mh * 3), map(mw * mh * 3, 0.3f);
    for (size_t i = 0; i < map_true.size(); ++i) map_true[i] = 0.15f + 0.7f * float((i * 7) % 11) / 10.0f;
    ok(ohao_pt_set_albedo_map(ctx, map_true.data(), mw, mh), ctx, "set_albedo_map");
    ok(ohao_pt_build(ctx, nullptr), ctx, "build");
    if (g_fail) return 1;

    const double eye[3] = {0.0, 2.6, 0.0}, at[3] = {0.0, 0.0, 0.0};
    const uint32_t w = 32, h = 32;
    ohao_gb300::PtImageFormation pt(ctx, {look_at(eye, at, w, h)}, 2);
    check(pt.supportsAnalyticGrads() && pt.viewCount() == 1, "interface");
    // target: the true map at 256 spp
    std::vector<uint8_t> target;
    ok(pt.forward(0, w, h, 256, 1, target), ctx, "forward target");
    check(target.size() == size_t(w) * h * 4, "target size");
    bool alpha = true, lit = false;
    for (size_t i = 0; i < target.size(); i += 4) {
        alpha = alpha && target[i + 3] == 255;
        lit = lit || target[i] > 40;
    }
    check(alpha && lit, "display image: alpha 255 and lit pixels");
    // the same request twice gives the same image; another seed another one
    std::vector<uint8_t> again, other;
    ok(pt.forward(0, w, h, 256, 1, again), ctx, "forward again");
    ok(pt.forward(0, w, h, 256, 2, other), ctx, "forward other seed");
    check(again == target && other != target, "seed selects the sample stream");

    // fit the map from 0.3 everywhere with the analytic gradient (Adam)
    ok(ohao_pt_set_albedo_map(ctx, map.data(), mw, mh), ctx, "set_albedo_map init");
    std::vector<uint8_t> img;
    ok(pt.forward(0, w, h, 256, 1, img), ctx, "forward init");
    const double mse0 = mse_rgb(img, target);
    std::vector<float> dmap(map.size()), drough(1);
    std::vector<double> m(map.size(), 0.0), v(map.size(), 0.0);
    float loss0 = 0.0f, loss = 0.0f;
    for (int it = 0; it < 60 && !g_fail; ++it) {
        if (!ok(pt.gradient({0}, w, h, {target.data()}, 16, 100 + it, dmap, drough, loss), ctx, "gradient")) break;
        if (it == 0) {
            loss0 = loss;
            double s = 0.0;
            for (float g : dmap) s += g;
            check(std::isfinite(s) && s < 0.0, "initial map gradient points to brighter albedo");
        }
        const double lr = 0.03, b1 = 0.9, b2 = 0.999;
        for (size_t i = 0; i < map.size(); ++i) {
            m[i] = b1 * m[i] + (1 - b1) * dmap[i];
            v[i] = b2 * v[i] + (1 - b2) * double(dmap[i]) * dmap[i];
            const double mh_ = m[i] / (1 - std::pow(b1, it + 1)), vh = v[i] / (1 - std::pow(b2, it + 1));
            map[i] = float(std::clamp(map[i] - lr * mh_ / (std::sqrt(vh) + 1e-8), 0.0, 1.0));
        }
        ok(ohao_pt_set_albedo_map(ctx, map.data(), mw, mh), ctx, "set_albedo_map step");
    }
    ok(pt.forward(0, w, h, 256, 1, img), ctx, "forward fitted");
    const double mse1 = mse_rgb(img, target);
    double err0 = 0.0, err1 = 0.0;
    for (size_t i = 0; i < map.size(); ++i) {
        err0 += std::fabs(0.3 - map_true[i]);
        err1 += std::fabs(map[i] - map_true[i]);
    }
    std::printf("display mse %.3e -> %.3e, adjoint loss %.3e -> %.3e, mean |map error| %.3f -> %.3f\n", mse0, mse1,
                loss0, loss, err0 / map.size(), err1 / map.size());
    check(loss0 > 0.0f && mse1 < 0.25 * mse0, "the fit lowers the display-space error");
    check(err1 < 0.5 * err0, "the fit moves the map towards the truth");
    // errors are status codes
    std::vector<uint8_t> none_img;
    check(pt.forward(5, w, h, 4, 1, none_img) == OHAO_ERR_INVALID_ARG, "unknown view is INVALID_ARG");
    ohao_pt_destroy(ctx);
    if (g_fail) return 1;
    std::printf("ok\n");
    return 0;
}
