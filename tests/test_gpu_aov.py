"""ohao_pt_aov: first-hit features averaged over camera samples. One sample
equals the record a render writes for that sample (bit for bit, flat and
textured scenes); several samples equal the mean of the single-sample
records (hit flag as a fraction, depth over the samples that hit)."""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pt_harness import gpu_tracer, small_env_scene

pytestmark = pytest.mark.gpu


def _render_aov(og, pt, v, base):
    import torch
    npix = v.width * v.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    aov = torch.zeros((npix, og.AOV_FLOATS), dtype=torch.float32, device="cuda")
    pt.render([og.make_view(v, accum=acc, aov=aov)], og.make_settings(spp=1, max_bounces=2, sample_index_base=base))
    return aov.cpu().numpy()


def _aov(og, pt, v, base, n):
    import torch
    out = torch.zeros((v.width * v.height, og.AOV_FLOATS), dtype=torch.float32, device="cuda")
    pt.aov(og.make_view(v), og.make_settings(spp=n, max_bounces=2, sample_index_base=base), out)
    return out.cpu().numpy()


@pytest.mark.parametrize("kind", ["env", "textured"])
def test_one_sample_is_the_render_record(gpu_lib, kind):
    og = gpu_lib
    sd = small_env_scene(freq=16) if kind == "env" else scenes.textured(48, 40)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    for base in (0, 7):
        assert np.array_equal(_aov(og, pt, v, base, 1), _render_aov(og, pt, v, base))


def test_mean_over_samples(gpu_lib):
    og = gpu_lib
    sd = small_env_scene(freq=16)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    n = 5
    recs = [_render_aov(og, pt, v, 11 + k) for k in range(n)]
    got = _aov(og, pt, v, 11, n)
    inv = np.float32(1.0) / np.float32(n)
    sums = np.zeros_like(recs[0])
    dsum = np.zeros(recs[0].shape[0], np.float32)
    hits = np.zeros(recs[0].shape[0], np.float32)
    for r in recs:   # the kernel's order of additions, in float32
        sums = (sums + r).astype(np.float32)
        dsum = (dsum + np.where(r[:, 7] > 0, r[:, 6], np.float32(0))).astype(np.float32)
        hits = (hits + r[:, 7]).astype(np.float32)
    want = (sums * inv).astype(np.float32)
    want[:, 6] = np.where(hits > 0, dsum / np.maximum(hits, np.float32(1)), np.float32(1e30))
    want[:, 10:] = 0.0
    assert np.allclose(got, want, rtol=1e-6, atol=1e-7)
    frac = got[:, 7]
    assert np.any((frac > 0) & (frac < 1)), "some pixels straddle an edge"
