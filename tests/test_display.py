"""The reference's display transform (pt_raygen.rgen:99-102, 1262-1269:
ldr = pow(ACES(acc * 0.5), 1/2.2) stored to an RGBA8 UNORM image, alpha 1):
the oracle's bytes against the formula in float64, and the device's bytes
(ohao_pt_view.display, ohao_pt_display, ohao_pt_render_host) against the
oracle's, bit for bit."""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes


def formula_bytes(x):
    x = np.asarray(x, np.float64) * 0.5
    y = np.clip((x * (2.51 * x + 0.03)) / (x * (2.43 * x + 0.59) + 0.14), 0.0, 1.0)
    return np.floor(255.0 * y ** (1.0 / 2.2) + 0.5)


def test_oracle_display_matches_formula(oracle):
    rng = np.random.default_rng(1)
    x = np.exp(rng.uniform(np.log(1e-5), np.log(1e3), (200000, 4))).astype(np.float32)
    x[:100] = 0.0
    b = oracle.display_rgba8(x)
    ref = formula_bytes(x[:, :3])
    d = np.abs(b[:, :3].astype(np.int64) - ref)
    assert d.max() <= 1                       # float ACES vs float64: only rounding-boundary cases differ
    assert (d == 0).mean() > 0.9999
    assert np.all(b[:, 3] == 255) and np.all(b[:100, :3] == 0)
    big = oracle.display_rgba8(np.full((1, 4), 1e6, np.float32))
    assert np.all(big[0] == 255)


@pytest.mark.gpu
def test_device_display_bit_exact(gpu_lib, oracle):
    import torch
    og = gpu_lib
    sd = scenes.cornell(40, 32, 4)
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    disp = torch.zeros((npix * 4,), dtype=torch.uint8, device="cuda")
    pt.render([og.make_view(v, accum=acc, display=disp)], og.make_settings(spp=4, max_bounces=4))
    torch.cuda.synchronize()
    a = acc.cpu().numpy()
    assert np.array_equal(disp.cpu().numpy().reshape(-1, 4), oracle.display_rgba8(a))
    # the standalone call over values spanning the whole curve (and NaN / negative / huge)
    rng = np.random.default_rng(2)
    x = np.exp(rng.uniform(np.log(1e-6), np.log(1e4), (1 << 20, 4))).astype(np.float32)
    x[:16] = [[0.0, -1.0, np.nan, 1e30]] * 16
    xd = torch.from_numpy(x).cuda()
    out = torch.zeros((x.shape[0] * 4,), dtype=torch.uint8, device="cuda")
    og.display(xd, x.shape[0], out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().reshape(-1, 4), oracle.display_rgba8(x))
    # render_host: display image read back into host memory with the accumulator
    host = np.zeros((npix, 4), np.float32)
    hdisp = np.zeros(npix * 4, np.uint8)
    pt.render_host([og.make_view(v, display=hdisp, display_host=True)], og.make_settings(spp=4, max_bounces=4),
                   [host])
    assert np.array_equal(host, a)
    assert np.array_equal(hdisp.reshape(-1, 4), oracle.display_rgba8(host))
    pt.close()
