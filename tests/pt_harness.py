"""Shared harness for the GPU parity tests: runs the same seeded scene through
the CUDA library (C ABI) and the host oracle."""
from __future__ import annotations

import numpy as np

from ohao_engine_gb300 import scenes


def small_env_scene(freq=10, seed=1, width=40, height=24, env_peak=500.0, metal_mix=True):
    pos, nrm, uv, idx = scenes.displaced_sphere(freq, seed=seed)
    b = scenes._Builder()
    rng = np.random.default_rng(seed)
    nt = idx.shape[0]
    mats = scenes._random_materials(rng, nt + 1)
    if not metal_mix:
        mats[:, 5] = 0.0
    mats[nt] = scenes.material((0.5, 0.5, 0.5), rough=0.8)
    b.add(pos, nrm, uv, idx, np.arange(nt, dtype=np.uint32))
    scenes._ground(b, -1.05, 6.0, nt)
    P, N, U, I, M = b.arrays()
    env = scenes.sky_env(64, 32, seed=seed, peak=env_peak, radius_deg=3.0)
    view = scenes.look_at_view((0, 0.6, 3.2), (0, -0.1, 0), width=width, height=height)
    return scenes.SceneData("small_env", P, N, U, I, M, mats, np.zeros((0, 20), np.float32), env, 1.0,
                            [(0, I.size)], scenes.identity_instance(1), [view], spp=4, max_bounces=4)


def small_instanced(n_instances=80, seed=5, side=32):
    sd = scenes.instanced(n_instances=n_instances, n_views=2, freqs=(3, 6), side_range=(side, side), seed=seed)
    return sd


def gpu_tracer(og, sd, flatten_limit=0):
    pt = og.PathTracer(flatten_limit=flatten_limit)
    pt.load_scene(sd)
    return pt


def render_paths_gpu(og, pt, view, spp, settings_kw, history=0, accum=None, aov=False):
    import torch
    npix = view.width * view.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda") if accum is None else accum
    paths = torch.zeros((spp, npix, 4), dtype=torch.float32, device="cuda")
    aovt = torch.zeros((npix, og.AOV_FLOATS), dtype=torch.float32, device="cuda") if aov else None
    v = og.make_view(view, accum=acc, history=history, path_radiance=paths, aov=aovt)
    s = og.make_settings(spp=spp, **settings_kw)
    pt.render([v], s)
    torch.cuda.synchronize()
    out = paths.cpu().numpy()[:, :, :3]
    return out, acc, aovt


def trace_gpu(og, pt, rays, any_hit=False, stats=False):
    import torch
    n = rays.shape[0]
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    h = torch.zeros((n, 5), dtype=torch.int32, device="cuda")
    s = torch.zeros((n, 2), dtype=torch.int32, device="cuda") if stats else None
    pt.trace(r, n, h, any_hit=any_hit, stats_dev=s)
    torch.cuda.synchronize()
    hits = h.cpu().numpy().view(np.uint32)
    return (hits, s.cpu().numpy().view(np.uint32)) if stats else hits


def random_rays(rng, n, lo, hi, tmin=0.001, tmax=10000.0):
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)



def emitter_scene(width=40, height=24, lights=("area", "sphere"), env=False):
    """scenes.emitters at a test size."""
    return scenes.emitters(width=width, height=height, lights=lights, env=env)
