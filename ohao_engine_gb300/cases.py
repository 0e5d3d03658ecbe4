"""Small self-contained runs of the library's GPU paths, for timing and for
profiler captures (one process, one GPU, a few GB at most):

    python -m ohao_engine_gb300.cases denoise_infer   # U-Net inference at 1920x1080 (13 calls)
    python -m ohao_engine_gb300.cases adjoint         # ohao_pt_adjoint, studio scene, 1 view 256^2, 4 spp (2 calls)
    python -m ohao_engine_gb300.cases instanced_view  # one 512^2 view of the instanced scene, 4 spp (3 calls)
    python -m ohao_engine_gb300.cases instanced_pool [launch shape]
                                              # 4 views 384^2 of the instanced scene, persistent pool (2 calls)

Each prints one line with its CUDA-event time per call.
"""
from __future__ import annotations

import sys

import numpy as np


def _timed(fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def denoise_infer():
    import torch
    from .denoise import Denoiser
    w, h = 1920, 1080
    rng = np.random.default_rng(0)
    rad = torch.from_numpy(rng.exponential(0.5, (w * h, 4)).astype(np.float32)).cuda()
    aov = torch.from_numpy(rng.random((w * h, 12)).astype(np.float32)).cuda()
    out = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    dn = Denoiser(max_pixels=1920 * 1088, seed=1)
    for _ in range(3):
        dn.infer([rad], [aov], [out], w, h)
    ms = _timed(lambda: dn.infer([rad], [aov], [out], w, h), 10)
    print(f"denoise_infer 1920x1080: {ms:.3f} ms per call")


def adjoint():
    import torch
    import ohao_engine_gb300 as og
    from . import scenes
    sd = scenes.studio(n_train=1, n_holdout=0, side=256)
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    tgt = torch.full((npix, 4), 0.3, device="cuda")
    acc = torch.zeros((npix, 4), device="cuda")
    gm = torch.zeros(sd.albedo_map.size, device="cuda")
    gr = torch.zeros(sd.materials.shape[0], device="cuda")
    s = og.make_settings(spp=4, max_bounces=3, flags=og.FLAG_ADJOINT_DECORRELATE)
    ms = _timed(lambda: pt.adjoint([og.make_view(v, accum=acc)], s, [tgt], gm, gr), 2)
    print(f"adjoint studio 256^2 x 4 spp: {ms:.3f} ms per call")


def instanced_view():
    import torch
    import ohao_engine_gb300 as og
    from . import scenes
    sd = scenes.instanced(n_views=1, side_range=(512, 512))
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    acc = torch.zeros((v.width * v.height, 4), device="cuda")
    s = og.make_settings(spp=4, max_bounces=4, mode=og.MODE_WAVEFRONT)
    ms = _timed(lambda: pt.render([og.make_view(v, accum=acc)], s), 3)
    print(f"instanced one 512^2 view x 4 spp: {ms:.3f} ms per call")


def instanced_pool():
    import torch
    import ohao_engine_gb300 as og
    from . import scenes
    sd = scenes.instanced(n_views=4, side_range=(384, 384))
    pt = og.PathTracer()
    pt.load_scene(sd)
    pt.launch_config = sys.argv[2] if len(sys.argv) > 2 else "pool_4M_unsorted_fetch4_chunk8"
    accs = [torch.zeros((v.width * v.height, 4), device="cuda") for v in sd.views]
    s = og.make_settings(spp=4, max_bounces=4, mode=og.MODE_PERSISTENT)
    ms = _timed(lambda: pt.render([og.make_view(v, accum=a) for v, a in zip(sd.views, accs)], s), 2)
    print(f"instanced 4 views 384^2 x 4 spp, {pt.launch_config}: {ms:.3f} ms per call")


CASES = {"denoise_infer": denoise_infer, "adjoint": adjoint, "instanced_view": instanced_view,
         "instanced_pool": instanced_pool}

if __name__ == "__main__":
    import ohao_engine_gb300 as og
    og.load_library()
    CASES[sys.argv[1]]()
