"""The path-replay gradient on the inverse-fit configuration itself (studio:
200,002 triangles, 64x64x3 tile albedo map + 4 roughness regions, 8 train
views of 512x512, 16 spp per batch, depth 3) against central finite
differences (h = 1e-3) of the renderer's EXPECTED image.

The gradient under test is the full one -- pathwise derivatives plus the
sampling-score terms (roughness-scaled specular jitter, clamped lobe choice,
Russian roulette above one) -- of G(theta) = sum_p w_p . E[I_p(theta)] for a
fixed weight image w (dL/dI of the multi-view L2 loss at the starting
parameters). The finite differences render the real estimator (whose
sampling decisions move with theta, so the difference of expectations sees
the score part too) with common random numbers at theta +- h. Both sides
are Monte-Carlo estimates: each is taken over K independent sample batches,
and they are compared parameter by parameter (within 4 combined standard
errors plus 2%), and where both are sharp (combined standard error under 2%)
through their median relative difference (under 1.5%).
"""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes

pytestmark = pytest.mark.gpu

H_STEP = 1e-3
K_BATCH = 8        # independent sample batches per estimate
SPP_FD = 8         # samples per pixel of each finite-difference render
SPP_ADJ = 16       # samples per pixel of each adjoint batch
N_TILES = 32       # seeded tile-map texel channels checked, plus the 4 roughness values


def test_full_gradient_matches_fd_of_expectation_config4(gpu_lib):
    import torch
    og = gpu_lib
    sd = scenes.studio()
    assert sd.ntris == 200002 and sd.views[0].width == 512
    train = sd.views[:8]
    pt = og.PathTracer()
    pt.load_scene(sd)
    dev = torch.device("cuda")
    npix = [v.width * v.height for v in train]
    # targets at the ground truth, then the starting point of the fit
    tgt = [torch.zeros((n, 4), dtype=torch.float32, device=dev) for n in npix]
    pt.render([og.make_view(v, accum=a) for v, a in zip(train, tgt)],
              og.make_settings(spp=64, max_bounces=3, sample_index_base=1 << 20))
    rng = np.random.default_rng(21)
    amap = np.clip(sd.albedo_map + rng.uniform(-0.4, 0.4, sd.albedo_map.shape), 0.0, 1.0).astype(np.float32)
    mats = sd.materials.copy()
    mats[:4, 4] = np.clip(mats[:4, 4] + rng.uniform(-0.2, 0.2, 4), 0.05, 1.0).astype(np.float32)
    pt.set_albedo_map(amap)
    pt.update_materials(mats)
    img = [torch.zeros((n, 4), dtype=torch.float32, device=dev) for n in npix]
    pt.render([og.make_view(v, accum=a) for v, a in zip(train, img)],
              og.make_settings(spp=16, max_bounces=3, sample_index_base=1 << 21))
    # fixed weights: dL/dI of the mean over views of the RGB MSE
    w = []
    for a, t, n in zip(img, tgt, npix):
        g = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        g[:, :3] = 2.0 * (a[:, :3] - t[:, :3]) / (len(train) * n * 3)
        w.append(g)
    # the adjoint over K independent batches (fresh sample indices each)
    gm = torch.zeros(amap.size, dtype=torch.float32, device=dev)
    gr = torch.zeros(mats.shape[0], dtype=torch.float32, device=dev)
    adj = []
    for k in range(K_BATCH):
        pt.backward([og.make_view(v) for v in train],
                    og.make_settings(spp=SPP_ADJ, max_bounces=3, sample_index_base=(1 << 22) + k * SPP_ADJ),
                    w, gm, gr)
        torch.cuda.synchronize()
        adj.append(np.concatenate([gm.cpu().numpy().astype(np.float64), gr.cpu().numpy()[:4].astype(np.float64)]))
    adj = np.array(adj)
    # parameters: seeded tile-map entries the views see, and the 4 roughness values
    g_mean = adj.mean(0)
    seen = np.nonzero(np.abs(g_mean[:amap.size]) > 1e-3 * np.abs(g_mean[:amap.size]).max())[0]
    params = [("map", int(k)) for k in np.random.default_rng(5).choice(seen, N_TILES, replace=False)]
    params += [("rough", k) for k in range(4)]
    acc = [torch.zeros((n, 4), dtype=torch.float32, device=dev) for n in npix]

    def G(base):
        pt.render([og.make_view(v, accum=a) for v, a in zip(train, acc)],
                  og.make_settings(spp=SPP_FD, max_bounces=3, sample_index_base=base))
        return sum(float((a[:, :3].double() * ww[:, :3].double()).sum()) for a, ww in zip(acc, w))

    fd = np.zeros((K_BATCH, len(params)))
    for j, (which, k) in enumerate(params):
        for sgn_k, sgn in enumerate((+1.0, -1.0)):
            if which == "map":
                m2 = amap.copy()
                m2.reshape(-1)[k] += np.float32(sgn * H_STEP)
                pt.set_albedo_map(m2)
            else:
                mt = mats.copy()
                mt[k, 4] += np.float32(sgn * H_STEP)
                pt.update_materials(mt)
            for b in range(K_BATCH):   # common random numbers: the same base at +h and -h
                fd[b, j] += sgn * G((1 << 23) + b * SPP_FD)
        pt.set_albedo_map(amap)
        pt.update_materials(mats)
        if which == "map":
            step = float(np.float32(amap.reshape(-1)[k] + np.float32(H_STEP))) - float(
                np.float32(amap.reshape(-1)[k] - np.float32(H_STEP)))
        else:
            step = float(np.float32(mats[k, 4] + np.float32(H_STEP))) - float(np.float32(mats[k, 4] - np.float32(H_STEP)))
        fd[:, j] /= step
    idx = np.array([k if which == "map" else amap.size + k for which, k in params])
    a_mean, a_se = adj[:, idx].mean(0), adj[:, idx].std(0, ddof=1) / np.sqrt(K_BATCH)
    f_mean, f_se = fd.mean(0), fd.std(0, ddof=1) / np.sqrt(K_BATCH)
    se = np.sqrt(a_se ** 2 + f_se ** 2)
    z = (a_mean - f_mean) / np.maximum(se, 1e-300)
    rel = np.abs(a_mean - f_mean) / np.abs(f_mean)
    report = "\n".join(f"{p[0]:5s} {p[1]:6d} adjoint {a:+.4e} +- {sa:.1e}   fd {f:+.4e} +- {sf:.1e}   z {zz:+.2f}"
                       for p, a, sa, f, sf, zz in zip(params, a_mean, a_se, f_mean, f_se, z))
    print(report)
    sharp = se < 0.02 * np.abs(f_mean)
    print(f"chi2 {float((z ** 2).sum()):.1f} over {len(params)} parameters; {int(sharp.sum())} parameters with a "
          f"combined standard error below 2%: median relative difference {np.median(rel[sharp]):.4f}")
    # every parameter within 4 combined standard errors plus 2% (the finite
    # differences' own truncation and the heavy tails of their noise, which
    # 8 batches resolve only roughly)
    assert np.all(np.abs(a_mean - f_mean) <= 4 * se + 0.02 * np.abs(f_mean)), report
    # where both estimates are sharp, they agree to about a percent
    assert sharp.sum() >= 10 and np.median(rel[sharp]) < 0.015, report
    # roughness gradients the differences resolve agree in sign (the score
    # terms decide it: without them the fit moved roughness the wrong way)
    r = slice(N_TILES, None)
    resolved = np.abs(f_mean[r]) > 3 * f_se[r]
    assert resolved.sum() >= 1, report
    assert np.all(np.sign(a_mean[r][resolved]) == np.sign(f_mean[r][resolved])), report
    pt.close()
