"""tcgen05 U-Net denoiser (include/ohao_dn.h) against the NumPy oracle
(oracle/dn_ref.py): every layer's forward output, weight/bias gradient and
data gradient from the device's own layer inputs, the whole network end to
end, and a short training run on path-traced pairs that must beat the noisy
input it denoises."""
import numpy as np
import pytest

import dn_ref as R


def _inputs(rng, n, h, w):
    import torch
    rad, aov, tgt = [], [], []
    for _ in range(n):
        r = np.zeros((h * w, 4), np.float32)
        r[:, :3] = rng.exponential(0.6, (h * w, 3)) * (rng.random((h * w, 1)) < 0.9)
        r[rng.random(h * w) < 0.02, :3] *= 40.0
        a = rng.random((h * w, 12)).astype(np.float32)
        a[:, 6] *= 8.0
        a[:, 7] = (rng.random(h * w) < 0.85).astype(np.float32)
        t = np.zeros((h * w, 4), np.float32)
        t[:, :3] = rng.exponential(0.5, (h * w, 3))
        rad.append(torch.from_numpy(r).cuda())
        aov.append(torch.from_numpy(a).cuda())
        tgt.append(torch.from_numpy(t).cuda())
    return rad, aov, tgt


def _device_state(dn, n, h, w):
    specs, tensors = R.layer_specs()
    T, G = [], []
    for i, (name, lvl, c8) in enumerate(tensors):
        a = dn.tensor(i).reshape(n, h >> lvl, w >> lvl, c8).astype(np.float64)
        T.append(a)
        G.append(dn.tensor(i, grad=True).reshape(n, h >> lvl, w >> lvl, c8).astype(np.float64) if i else None)
    return specs, tensors, T, G


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


# Forward kernels by row width: "narrow" runs every layer on the gather
# (rows < 96 pixels); "wide" (levels 0-2 >= 96 pixels) runs the
# warp-specialised kernel with 4-, 2- and 1-row tiles, two-source
# (upsampled + skip) layers and a layer split over its output channels;
# "wider" (every level >= 96 pixels) also the deep levels, split in two and
# four launches, and the neighbourhood and gather kernels of level 3.
@pytest.fixture(scope="module", params=[(2, 32, 48), (1, 16, 512), (1, 16, 1536)], ids=["narrow", "wide", "wider"])
def trained_step(gpu_lib, request):
    from ohao_engine_gb300.denoise import Denoiser
    n, h, w = request.param
    rng = np.random.default_rng(5)
    dn = Denoiser(max_pixels=n * h * w, seed=3)
    rad, aov, tgt = _inputs(rng, n, h, w)
    loss = dn.train_step(rad, aov, tgt, w, h, lr=0.0)
    return dn, (n, h, w), rad, aov, tgt, loss


@pytest.mark.gpu
def test_pack_and_loss(trained_step):
    dn, (n, h, w), rad, aov, tgt, loss = trained_step
    specs, tensors, T, G = _device_state(dn, n, h, w)
    for i in range(n):
        x = R.pack(rad[i].cpu().numpy().reshape(h, w, 4), aov[i].cpu().numpy().reshape(h, w, 12))
        # log1pf vs log1p may round to the other side of a BF16 boundary
        assert np.max(np.abs(T[0][i] - x)) <= np.max(np.abs(x)) * 2 ** -7
    out = T[-1]
    tg = np.stack([t.cpu().numpy().reshape(h, w, 4) for t in tgt])
    av = np.stack([a.cpu().numpy().reshape(h, w, 12) for a in aov])
    l_ref, g_ref = R.l1_loss_grad(out, tg[..., :3], av)
    assert abs(loss - l_ref) <= 1e-5 * l_ref
    # FP32 transcendental functions on the device: compare away from the
    # L1 kinks, within float rounding
    assert np.allclose(G[-1][..., :3], g_ref[..., :3], rtol=1e-4, atol=1e-6 * np.abs(g_ref).max())


@pytest.mark.gpu
def test_each_layer_forward(trained_step):
    """Each tensor-core convolution from the device's own inputs: BF16
    outputs within two BF16 rounding steps, the FP32 output layer within 1e-5."""
    dn, (n, h, w), *_ = trained_step
    specs, tensors, T, G = _device_state(dn, n, h, w)
    params = R.unflatten_params(dn.get_params())
    li = 0
    for s in specs:
        if s[0] == "pool":
            assert np.array_equal(T[s[9]], R.pool2(T[s[2]])), s[1]
            continue
        _, name, in0, in1, up0, cin, cin8, cout, relu, outi = s
        xin = R.up2(T[in0]) if up0 else T[in0]
        if in1 is not None:
            xin = np.concatenate([xin, T[in1]], axis=-1)
        W, b = params[li]
        li += 1
        y = R.conv3x3(xin, R.bf16(W), b)
        dev = T[outi][..., :cout]
        if relu:
            y = np.maximum(y, 0.0)
            err = np.abs(dev - R.bf16(y))
            assert np.all(err <= np.abs(y) * 2 ** -7 + 1e-6 * np.abs(y).max()), (name, err.max())
            assert np.mean(err > 0) < 0.01, name
        else:
            assert _rel(dev, y) < 1e-5, name


@pytest.mark.gpu
def test_each_layer_backward(trained_step):
    """Weight, bias and data gradients of every layer from the device's own
    upstream gradient dY (BF16 operands, FP32 accumulation on the device)."""
    dn, (n, h, w), *_ = trained_step
    specs, tensors, T, G = _device_state(dn, n, h, w)
    params = R.unflatten_params(dn.get_params())
    grads = R.unflatten_params(dn.get_grads())
    Gacc = [np.zeros_like(t) for t in T]
    convs = [s for s in specs if s[0] == "conv"]
    li = len(convs)
    for s in reversed(specs):
        if s[0] == "pool":
            Gacc[s[2]] += R.pool2_bwd(T[s[2]], G[s[9]])
            continue
        li -= 1
        _, name, in0, in1, up0, cin, cin8, cout, relu, outi = s
        W, b = params[li]
        dY = G[outi][..., :cout]
        dzf = dY * (T[outi][..., :cout] > 0) if relu else dY
        dz = R.bf16(dzf)
        xin = R.up2(T[in0]) if up0 else T[in0]
        if in1 is not None:
            xin = np.concatenate([xin, T[in1]], axis=-1)
        gW_dev, gb_dev = grads[li]
        assert _rel(gW_dev, R.conv3x3_wgrad(xin, dz, cin)) < 1e-4, name
        assert _rel(gb_dev, dzf.reshape(-1, cout).sum(axis=0)) < 1e-4, name
        if in0 != 0:
            dx = R.conv3x3_dgrad(dz, R.bf16(W), cin8)
            c0 = T[in0].shape[-1]
            Gacc[in0] += R.up2_bwd(dx[..., :c0]) if up0 else dx[..., :c0]
            if in1 is not None:
                Gacc[in1] += dx[..., c0:]
    for i in range(1, len(T) - 1):
        assert _rel(G[i], Gacc[i]) < 1e-4, tensors[i][0]


@pytest.mark.gpu
def test_network_end_to_end(trained_step):
    """The whole network against the oracle from the same packed input:
    output, loss and every parameter gradient."""
    dn, (n, h, w), rad, aov, tgt, loss = trained_step
    specs, tensors, T, G = _device_state(dn, n, h, w)
    params = R.unflatten_params(dn.get_params())
    Tr = R.forward(T[0], params)
    assert _rel(T[-1][..., :3], Tr[-1][..., :3]) < 1e-2
    tg = np.stack([t.cpu().numpy().reshape(h, w, 4) for t in tgt])
    av = np.stack([a.cpu().numpy().reshape(h, w, 12) for a in aov])
    l_ref, g_out = R.l1_loss_grad(Tr[-1], tg[..., :3], av)
    assert abs(loss - l_ref) <= 1e-2 * l_ref
    # backpropagate the device's own d loss / d output: the L1 sign flips
    # wherever the two outputs straddle the target, which is not under test
    gr, _ = R.backward(Tr, params, G[-1])
    gd = R.unflatten_params(dn.get_grads())
    for k, ((gW, gb), (dW, db)) in enumerate(zip(gr, gd)):
        # BF16 rounding and ReLU-mask differences accumulate over 19 layers; the
        # deepest levels sum over few pixels (the per-layer tests are the tight check)
        assert _rel(dW, gW) < 1e-1, k
        assert _rel(db, gb) < 1e-1, k


@pytest.mark.gpu
def test_infer_save_load_and_odd_sizes(gpu_lib, tmp_path):
    import torch
    from ohao_engine_gb300.denoise import Denoiser
    rng = np.random.default_rng(9)
    w, h = 40, 24   # padded to 48 x 32 inside
    dn = Denoiser(max_pixels=48 * 32, seed=4)
    rad, aov, _ = _inputs(rng, 1, h, w)
    out = torch.zeros((h * w, 4), dtype=torch.float32, device="cuda")
    dn.infer(rad, aov, [out], w, h)
    o1 = out.cpu().numpy()
    assert np.all(np.isfinite(o1)) and np.all(o1[:, 3] == 1.0)
    p = str(tmp_path / "dn.bin")
    dn.save(p)
    dn2 = Denoiser(max_pixels=48 * 32, seed=99)
    assert not np.array_equal(dn2.get_params(), dn.get_params())
    dn2.load(p)
    assert np.array_equal(dn2.get_params(), dn.get_params())
    out2 = torch.zeros_like(out)
    dn2.infer(rad, aov, [out2], w, h)
    assert torch.equal(out, out2)


@pytest.mark.gpu
def test_training_beats_the_noisy_input(gpu_lib):
    """Trained on the GPU with its own kernels on path-traced 1-spp / 256-spp
    pairs of four scenes, the network's output on a held-out scene is closer
    to that scene's reference than the 1-spp image it was given (the method
    without the network), in log radiance and after the display transform."""
    import torch
    og = gpu_lib
    from ohao_engine_gb300.denoise import Denoiser, render_pair, tonemap, training_scene
    side = 64
    data = []
    for seed in (11, 12, 13, 14, 99):
        sd = training_scene(seed, side=side, freq=24, env_size=(128, 64))
        pt = og.PathTracer()
        pt.load_scene(sd)
        pairs = [render_pair(pt, sd.views[0], side, side, 1, 256, seed_base=1000 * k) for k in range(3)]
        data.append(pairs)
        pt.close()
    train, held = data[:4], data[4]
    dn = Denoiser(max_pixels=4 * side * side, seed=7)
    rng = np.random.default_rng(0)
    losses = []
    for it in range(800):
        batch = [train[s][rng.integers(3)] for s in range(4)]
        losses.append(dn.train_step([b[0] for b in batch], [b[1] for b in batch], [b[2] for b in batch], side, side,
                                    lr=2e-3))
    assert np.all(np.isfinite(losses))
    assert np.mean(losses[-30:]) < 0.8 * np.mean(losses[:30]), (np.mean(losses[:30]), np.mean(losses[-30:]))
    noisy, aov, ref = held[0]
    out = torch.zeros_like(noisy)
    dn.infer([noisy], [aov], [out], side, side)
    n_, o_, r_ = (t.cpu().numpy()[:, :3].astype(np.float64) for t in (noisy, out, ref))
    l1 = lambda a: np.abs(np.log1p(np.maximum(a, 0)) - np.log1p(r_)).mean()
    rm = lambda a: np.sqrt(((tonemap(a) - tonemap(r_)) ** 2).mean())
    # the weight-gradient atomics make the run vary slightly from one GPU run
    # to the next; the margins hold with room on each
    assert l1(o_) < 0.9 * l1(n_), (l1(o_), l1(n_))
    assert rm(o_) < 0.8 * rm(n_), (rm(o_), rm(n_))
