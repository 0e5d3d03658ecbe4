"""Images of every workload against the FP64 host render of the same
samples (oracle in double precision, same seeds and sample indices): the
difference is the FP32 arithmetic of the device, not Monte Carlo noise.
Prints one line per workload (RMSE, relative RMSE, max relative error)."""
import numpy as np
import pytest

import pt_harness as H
from ohao_engine_gb300 import scenes


def _subset(rng, view, n):
    npix = view.width * view.height
    return np.sort(rng.choice(npix, min(n, npix), replace=False)).astype(np.uint32)


CASES = [
    # name, scene factory, spp, max_bounces, pixels (None = all)
    ("cornell 256x256 16spp", lambda: scenes.cornell(256, 256), 16, 4, None),
    ("sphere_1m 1920x1080", lambda: scenes.sphere_1m(), 2, 4, 3000),
    ("instanced view 0", lambda: scenes.instanced(n_instances=2000, n_views=1), 2, 4, 3000),
    ("studio view 0", lambda: scenes.studio(), 4, 3, 3000),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,spp,depth,npix", CASES, ids=[c[0].split()[0] for c in CASES])
def test_image_vs_fp64_host_render(gpu_lib, oracle, name, make, spp, depth, npix):
    og = gpu_lib
    sd = make()
    pt = H.gpu_tracer(og, sd)
    view = sd.views[0]
    paths, _, _ = H.render_paths_gpu(og, pt, view, spp, dict(max_bounces=depth, sampler=0))
    o = oracle.OracleScene(sd)
    rng = np.random.default_rng(1)
    pix = None if npix is None else _subset(rng, view, npix)
    ref = o.render_paths(view, dict(max_bounces=depth, sampler=0), 0, spp, pix, fp64=True)
    dev = paths if pix is None else paths[:, pix]
    img_dev = dev.astype(np.float64).mean(axis=0)
    img_ref = ref.mean(axis=0)
    rmse = float(np.sqrt(((img_dev - img_ref) ** 2).mean()))
    rel = rmse / max(float(np.sqrt((img_ref ** 2).mean())), 1e-30)
    mx = float((np.abs(img_dev - img_ref) / np.maximum(np.abs(img_ref), 1e-3)).max())
    print(f"\n[fp64] {name}: {img_ref.shape[0]} px x {spp} spp, RMSE {rmse:.3e}, relative RMSE {rel:.3e}, "
          f"max relative error {mx:.3e}")
    # Single paths may take the other branch in FP64 (Russian roulette, lobe
    # choice, grazing hits); one such path that reaches the sun moves a pixel
    # a lot, so the bound is on the whole image.
    assert rel < 1e-2
