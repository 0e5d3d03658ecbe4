"""Differentiable rendering through ``torch.autograd``.

The GB300 counterpart of the reference's inverse-rendering hooks
(ohao/render/diff/diff_map.hpp: the tile albedo map read through diffuse
texture slot 0; ohao/render/diff/diff_vk_forward.hpp:80-93: the multi-view
image loss). The forward pass renders the views with ``ohao_pt_render``; the
backward pass replays the same paths with ``ohao_pt_backward`` and returns
d loss / d albedo map and d loss / d roughness per material. Sampling is
detached (see ``include/ohao_pt.h``): the gradient is that of the estimator
with the render's own random decisions held fixed.

torch is plumbing here (device buffers and autograd bookkeeping); every
path, traversal and gradient is computed by the CUDA kernels of
``libohao_pt.so``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import PathTracer, Settings, make_view


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo_map, roughness, tracer: PathTracer, materials: np.ndarray, views, settings: Settings):
        mats = np.array(materials, np.float32, copy=True).reshape(-1, 12)
        mats[:, 4] = roughness.detach().float().cpu().numpy()
        tracer.update_materials(mats)
        tracer.set_albedo_map(albedo_map.detach().float().cpu().numpy())
        dev = torch.device("cuda", tracer.device)
        accs = [torch.zeros((v.height, v.width, 4), dtype=torch.float32, device=dev) for v in views]
        tracer.render([make_view(v, accum=a) for v, a in zip(views, accs)], settings)
        ctx.tracer, ctx.views, ctx.settings = tracer, views, settings
        ctx.map_shape, ctx.map_device, ctx.nmats, ctx.rough_device = (tuple(albedo_map.shape), albedo_map.device,
                                                                      mats.shape[0], roughness.device)
        return torch.stack([a[..., :3] for a in accs])

    @staticmethod
    def backward(ctx, grad_out):
        tracer, views = ctx.tracer, ctx.views
        dev = torch.device("cuda", tracer.device)
        grads = []
        for k, v in enumerate(views):
            g = torch.zeros((v.height, v.width, 4), dtype=torch.float32, device=dev)
            g[..., :3] = grad_out[k].to(dev, torch.float32)
            grads.append(g)
        gmap = torch.zeros(ctx.map_shape, dtype=torch.float32, device=dev)
        grough = torch.zeros(ctx.nmats, dtype=torch.float32, device=dev)
        tracer.backward([make_view(v) for v in views], ctx.settings, grads, gmap, grough)
        torch.cuda.synchronize(dev)
        return gmap.to(ctx.map_device), grough.to(ctx.rough_device), None, None, None, None


def render(albedo_map: torch.Tensor, roughness: torch.Tensor, tracer: PathTracer, materials: np.ndarray, views,
           settings: Settings) -> torch.Tensor:
    """Images (n_views, H, W, 3) of the scene loaded in ``tracer`` with the
    given tile albedo map (h, w, 3) and per-material roughness (M,); the
    other material fields come from ``materials`` (M, 12). All views must
    share one size. Differentiable in ``albedo_map`` and ``roughness``; the
    firefly clamp must be off."""
    return _Render.apply(albedo_map, roughness, tracer, materials, views, settings)


def multi_view_mse(images: torch.Tensor, targets: torch.Tensor) -> torch.Tensor:
    """lossMulti on linear radiance: mean over views of the RGB MSE."""
    return ((images - targets) ** 2).mean(dim=(1, 2, 3)).mean()
