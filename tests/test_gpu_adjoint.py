"""Path-replay gradients (ohao_pt_backward / ohao_pt_adjoint) against the
oracle's analytic FP64 gradient of the same estimator on the same paths
(forward-mode duals: pathwise part + sampling scores), whose pathwise part is
in turn checked against central finite differences of the oracle's FP64
detached-sampling estimator.

The loss is lossMulti on linear radiance (mean over views of the RGB MSE);
d loss / d theta = sum_p dL/dI_p . dI_p/dtheta, and the finite difference
uses the same dL/dI_p (from the device image) with I_p the oracle's mean of
the same paths (same seeds). Tolerance: 1e-3 relative on parameters whose
gradient is at least 1% of the largest tested one."""
import numpy as np
import pytest

import pt_harness as H
from ohao_engine_gb300 import scenes

REL_TOL = 1e-3
H_STEP = 1e-3

CASES = [
    ("studio_pcg", lambda: scenes.studio(freq=20, side=40), dict(max_bounces=3, sampler=0), 2),
    ("studio_sobol_aniso", lambda: scenes.studio(freq=20, side=32),
     dict(max_bounces=3, sampler=1, aniso_strength=0.6, aniso_rotation=0.4), 2),
    ("small_env_many_mats", lambda: H.small_env_scene(), dict(max_bounces=4, sampler=0), 2),
    ("cornell_lights", lambda: scenes.cornell(32, 32), dict(max_bounces=4, sampler=1), 2),
]


def _oracle_settings(st):
    return dict(max_bounces=st["max_bounces"], sampler=st["sampler"], aniso=st.get("aniso_strength", 0.0),
                aniso_rot=st.get("aniso_rotation", 0.0))


def _setup(og, sd, st, spp, seed=7):
    """Renders a target with perturbed parameters, then runs the adjoint at
    the scene's own parameters. Returns device results and dL/dI."""
    import torch
    pt = H.gpu_tracer(og, sd)
    view = sd.views[0]
    npix = view.width * view.height
    rng = np.random.default_rng(seed)
    settings = og.make_settings(spp=spp, **st)
    mats_t = sd.materials.copy()
    mats_t[:, 4] = np.clip(mats_t[:, 4] + rng.uniform(-0.2, 0.2, mats_t.shape[0]).astype(np.float32), 0.1, 1.0)
    pt.update_materials(mats_t)
    if sd.albedo_map is not None:
        pt.set_albedo_map(np.clip(sd.albedo_map + rng.uniform(-0.3, 0.3, sd.albedo_map.shape), 0.05, 1.0)
                          .astype(np.float32))
    target = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    pt.render([og.make_view(view, accum=target)], settings)
    pt.update_materials(sd.materials)
    if sd.albedo_map is not None:
        pt.set_albedo_map(sd.albedo_map)
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    nm = sd.materials.shape[0]
    gmap = torch.zeros(sd.albedo_map.size if sd.albedo_map is not None else 1, dtype=torch.float32, device="cuda")
    grough = torch.zeros(nm, dtype=torch.float32, device="cuda")
    loss = pt.adjoint([og.make_view(view, accum=acc)], settings, [target], gmap, grough)
    torch.cuda.synchronize()
    I = acc.cpu().numpy()[:, :3].astype(np.float64)
    T = target.cpu().numpy()[:, :3].astype(np.float64)
    dLdI = 2.0 * (I - T) / (npix * 3)
    return dict(pt=pt, settings=settings, loss=loss, I=I, T=T, dLdI=dLdI, gmap=gmap.cpu().numpy().astype(np.float64),
                grough=grough.cpu().numpy().astype(np.float64), acc=acc, target=target)


def _fd(o, sd, ost, spp, dLdI, which, k):
    mats = sd.materials.copy()
    amap = None if sd.albedo_map is None else sd.albedo_map.copy()
    if which == "rough":
        mp, mm = mats.copy(), mats.copy()
        mp[k, 4] += np.float32(H_STEP)
        mm[k, 4] -= np.float32(H_STEP)
        step = float(mp[k, 4]) - float(mm[k, 4])
        args_p, args_m = dict(materials=mp, albedo_map=amap), dict(materials=mm, albedo_map=amap)
    else:
        ap, am = amap.copy(), amap.copy()
        ap.reshape(-1)[k] += np.float32(H_STEP)
        am.reshape(-1)[k] -= np.float32(H_STEP)
        step = float(ap.reshape(-1)[k]) - float(am.reshape(-1)[k])
        args_p, args_m = dict(materials=mats, albedo_map=ap), dict(materials=mats, albedo_map=am)
    Ip = o.detached_paths(sd.views[0], ost, 0, spp, **args_p).mean(axis=0)
    Im = o.detached_paths(sd.views[0], ost, 0, spp, **args_m).mean(axis=0)
    return float((dLdI * (Ip - Im)).sum() / step)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,st,spp", CASES, ids=[c[0] for c in CASES])
def test_adjoint_matches_detached_fd(gpu_lib, oracle, name, make, st, spp):
    og = gpu_lib
    sd = make()
    r = _setup(og, sd, st, spp)
    ost = _oracle_settings(st)
    o = oracle.OracleScene(sd)
    # the device image is the oracle's forward estimator (bit-exact per path)
    fwd = o.render_paths(sd.views[0], ost, 0, spp, None, fp64=False).astype(np.float64).mean(axis=0)
    assert np.allclose(r["I"], fwd, rtol=1e-5, atol=1e-6)
    loss_ref = float(((r["I"] - r["T"]) ** 2).mean())
    assert abs(r["loss"] - loss_ref) <= 1e-5 * loss_ref
    rng = np.random.default_rng(11)
    checks = []
    live = np.nonzero((sd.materials[:, 4] > 0.04) & (np.abs(r["grough"]) > 0))[0]
    if live.size:
        gmax = np.abs(r["grough"][live]).max()
        cand = live[np.abs(r["grough"][live]) >= 1e-2 * gmax]
        for k in rng.choice(cand, size=min(8, cand.size), replace=False):
            checks.append(("rough", int(k), r["grough"][k]))
    if sd.albedo_map is not None:
        g = r["gmap"]
        cand = np.nonzero(np.abs(g) >= 1e-2 * np.abs(g).max())[0]
        for k in rng.choice(cand, size=min(32, cand.size), replace=False):
            checks.append(("map", int(k), g[k]))
    assert len(checks) >= 4
    # analytic FP64 host gradient (forward-mode duals through the same detached estimator)
    rough_ids = [k for which, k, _ in checks if which == "rough"]
    map_ids = [k for which, k, _ in checks if which == "map"]
    g64 = o.detached_grad(sd.views[0], ost, 0, spp, r["dLdI"], rough_ids, map_ids, with_score=True)
    g64v = o.detached_grad(sd.views[0], ost, 0, spp, r["dLdI"], rough_ids, map_ids, with_score=False)
    bad = []
    for j, (which, k, gdev) in enumerate(checks):
        # The device gradient is the pathwise derivative plus the sampling
        # scores; the FP64 duals compute both on the same paths. Central
        # differences of the detached estimator see the pathwise part only.
        gfd = _fd(o, sd, ost, spp, r["dLdI"], which, k)
        fd_ok = abs(g64v[j] - gfd) <= REL_TOL * max(abs(gfd), 1e-3 * abs(g64[j]))
        if abs(gdev - g64[j]) > REL_TOL * abs(g64[j]) or not fd_ok:
            bad.append((which, k, gdev, g64[j], g64v[j], gfd))
    assert not bad, f"{name}: {len(bad)}/{len(checks)} off (device, FP64 full, FP64 pathwise, FD): {bad[:6]}"


@pytest.mark.gpu
def test_backward_from_image_gradient_equals_loss_backward(gpu_lib):
    """ohao_pt_backward with dL/dI from the caller gives the gradients of
    ohao_pt_adjoint, and the torch.autograd wrapper gives the same."""
    import torch
    og = gpu_lib
    from ohao_engine_gb300 import diff
    sd = scenes.studio(freq=20, side=32)
    st = dict(max_bounces=3, sampler=1)
    r = _setup(og, sd, st, 2)
    pt, view = r["pt"], sd.views[0]
    g_img = torch.zeros((view.width * view.height, 4), dtype=torch.float32, device="cuda")
    g_img[:, :3] = torch.from_numpy(r["dLdI"].astype(np.float32)).cuda()
    gmap = torch.zeros(sd.albedo_map.size, dtype=torch.float32, device="cuda")
    grough = torch.zeros(sd.materials.shape[0], dtype=torch.float32, device="cuda")
    pt.backward([og.make_view(view)], r["settings"], [g_img], gmap, grough)
    torch.cuda.synchronize()
    scale = np.abs(r["gmap"]).max()
    assert np.allclose(gmap.cpu().numpy(), r["gmap"], rtol=1e-4, atol=1e-6 * scale)
    assert np.allclose(grough.cpu().numpy(), r["grough"], rtol=1e-4, atol=1e-6 * np.abs(r["grough"]).max())
    # autograd wrapper
    amap = torch.from_numpy(sd.albedo_map.copy()).cuda().requires_grad_(True)
    rough = torch.from_numpy(sd.materials[:, 4].copy()).cuda().requires_grad_(True)
    img = diff.render(amap, rough, pt, sd.materials, [view], r["settings"])
    tgt = r["target"][:, :3].reshape(1, view.height, view.width, 3)
    loss = diff.multi_view_mse(img, tgt)
    loss.backward()
    assert abs(loss.item() - r["loss"]) <= 1e-5 * r["loss"]
    assert np.allclose(amap.grad.cpu().numpy().reshape(-1), r["gmap"], rtol=1e-3, atol=1e-5 * scale)
    assert np.allclose(rough.grad.cpu().numpy(), r["grough"], rtol=1e-3, atol=1e-5 * np.abs(r["grough"]).max())


@pytest.mark.gpu
def test_backward_rejects_firefly_clamp_and_deep_paths(gpu_lib):
    import torch
    og = gpu_lib
    sd = scenes.studio(freq=10, side=16)
    pt = H.gpu_tracer(og, sd)
    view = sd.views[0]
    g = torch.zeros((view.width * view.height, 4), dtype=torch.float32, device="cuda")
    for kw in (dict(flags=og.FLAG_FIREFLY_CLAMP, clamp_luminance=4.0), dict(max_bounces=17),
               dict(flags=og.FLAG_GGX_VNDF)):
        with pytest.raises(og.OhaoError):
            pt.backward([og.make_view(view)], og.make_settings(spp=1, **kw), [g])


@pytest.mark.gpu
def test_adjoint_decorrelated_replay(gpu_lib, oracle):
    """With OHAO_PT_FLAG_ADJOINT_DECORRELATE the gradient replays the paths of
    sample indices spp..2spp-1 while the loss uses the rendered 0..spp-1."""
    import torch
    og = gpu_lib
    sd = scenes.studio(freq=20, side=32)
    st = dict(max_bounces=3, sampler=0)
    spp = 2
    pt = H.gpu_tracer(og, sd)
    v = sd.views[0]
    npix = v.width * v.height
    target = torch.full((npix, 4), 0.25, dtype=torch.float32, device="cuda")
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    gmap = torch.zeros(sd.albedo_map.size, dtype=torch.float32, device="cuda")
    grough = torch.zeros(sd.materials.shape[0], dtype=torch.float32, device="cuda")
    s = og.make_settings(spp=spp, flags=og.FLAG_ADJOINT_DECORRELATE, **st)
    pt.adjoint([og.make_view(v, accum=acc)], s, [target], gmap, grough)
    torch.cuda.synchronize()
    I = acc.cpu().numpy()[:, :3].astype(np.float64)
    dLdI = 2.0 * (I - 0.25) / (npix * 3)
    o = oracle.OracleScene(sd)
    ost = _oracle_settings(st)
    fwd = o.render_paths(v, ost, 0, spp, None, fp64=False).astype(np.float64).mean(axis=0)
    assert np.allclose(I, fwd, rtol=1e-5, atol=1e-6)
    g = gmap.cpu().numpy()
    map_ids = list(np.argsort(-np.abs(g))[:24])
    g64 = o.detached_grad(v, ost, spp, spp, dLdI, [0, 1, 2, 3], map_ids, with_score=True)
    dev = np.concatenate([grough.cpu().numpy()[:4], g[map_ids]]).astype(np.float64)
    assert np.allclose(dev, g64, rtol=1e-3, atol=1e-6 * np.abs(g64).max()), (dev, g64)


@pytest.mark.gpu
def test_display_space_loss_equals_chain_rule(gpu_lib):
    """OHAO_PT_FLAG_ADJOINT_LDR_LOSS (the lab's mseRGB on display values):
    loss and gradients equal ohao_pt_backward fed with dL/dI of the same loss
    computed here in float64 from the rendered image (chain rule through
    pow(ACES(x / 2), 1/2.2)), and the host-buffer call gives the same."""
    import torch
    og = gpu_lib
    sd = scenes.studio(freq=20, side=40)
    pt = H.gpu_tracer(og, sd)
    view = sd.views[0]
    npix = view.width * view.height
    st = og.make_settings(spp=2, max_bounces=3, flags=og.FLAG_ADJOINT_LDR_LOSS)
    rng = np.random.default_rng(3)
    tgt_np = rng.uniform(0.05, 0.95, (npix, 4)).astype(np.float32)
    target = torch.from_numpy(tgt_np).cuda()
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    gmap = torch.zeros(sd.albedo_map.size, dtype=torch.float32, device="cuda")
    grough = torch.zeros(sd.materials.shape[0], dtype=torch.float32, device="cuda")
    loss = pt.adjoint([og.make_view(view, accum=acc)], st, [target], gmap, grough)
    torch.cuda.synchronize()
    I = acc.cpu().numpy()[:, :3].astype(np.float64)
    u = 0.5 * I
    num, den = u * (2.51 * u + 0.03), u * (2.43 * u + 0.59) + 0.14
    a = num / den
    inside = (a > 0) & (a < 1)
    D = np.where(a >= 1, 1.0, np.where(inside, np.clip(a, 1e-30, 1) ** (1 / 2.2), 0.0))
    slope = np.where(inside, (1 / 2.2) * D / np.clip(a, 1e-30, 1)
                     * ((5.02 * u + 0.03) * den - num * (4.86 * u + 0.59)) / den ** 2 * 0.5, 0.0)
    E = D - tgt_np[:, :3]
    ref_loss = (E ** 2).sum() / (npix * 3)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    dLdI = np.zeros((npix, 4), np.float32)
    dLdI[:, :3] = 2.0 * E * slope / (npix * 3)
    gm2 = torch.zeros_like(gmap)
    gr2 = torch.zeros_like(grough)
    plain = og.make_settings(spp=2, max_bounces=3)
    pt.backward([og.make_view(view)], plain, [torch.from_numpy(dLdI).cuda()], gm2, gr2)
    torch.cuda.synchronize()
    g1 = np.concatenate([gmap.cpu().numpy(), grough.cpu().numpy()])
    g2 = np.concatenate([gm2.cpu().numpy(), gr2.cpu().numpy()])
    scale = np.abs(g2).max()
    assert scale > 0 and np.abs(g1 - g2).max() <= 1e-3 * scale
    hm = np.zeros(sd.albedo_map.size, np.float32)
    hr = np.zeros(sd.materials.shape[0], np.float32)
    hl = pt.adjoint_host([og.make_view(view)], st, [tgt_np], hm, hr)
    assert abs(hl - loss) <= 1e-6 * loss   # same render; sums in another atomic order
    assert np.abs(np.concatenate([hm, hr]) - g1).max() <= 1e-5 * scale
    pt.close()
