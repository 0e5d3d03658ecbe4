"""Inverse material fit driven by the path-replay adjoint.

Replaces the coordinate finite differences of the reference's fitter
(ohao/inverse/staged_fit.hpp:316-332 and ohao/inverse/diff_fit.hpp:177-200:
two renders of every view per parameter and iteration) with one
``ohao_pt_adjoint`` call per iteration, which renders the views, evaluates
lossMulti on linear radiance and returns the whole gradient (tile albedo map
and per-material roughness). The update is the reference's Adam
(ohao/inverse/optimizer.hpp:12-39: beta1 0.9, beta2 0.999, eps 1e-8, bias
correction, projection onto the parameter box after each step).
"""
from __future__ import annotations

import numpy as np

from . import FLAG_ADJOINT_DECORRELATE, PathTracer, Settings, make_settings, make_view


class Adam:
    """AdamState::step of ohao/inverse/optimizer.hpp:26-39 over a flat vector."""

    def __init__(self, n: int, beta1=0.9, beta2=0.999, eps=1e-8):
        self.m = np.zeros(n)
        self.v = np.zeros(n)
        self.t = 0
        self.beta1, self.beta2, self.eps = beta1, beta2, eps

    def step(self, values: np.ndarray, grad: np.ndarray, lr: float, lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
        self.t += 1
        b1t = 1.0 - self.beta1 ** self.t
        b2t = 1.0 - self.beta2 ** self.t
        self.m = self.beta1 * self.m + (1.0 - self.beta1) * grad
        self.v = self.beta2 * self.v + (1.0 - self.beta2) * grad * grad
        mhat = self.m / b1t
        vhat = self.v / b2t
        return np.clip(values - lr * mhat / (np.sqrt(vhat) + self.eps), lo, hi)


class AdjointFit:
    """Fits the tile albedo map and the roughness of ``rough_ids`` to target
    images. ``targets`` are device RGBA32F tensors, one per view; ``accums``
    device RGBA32F tensors receive each iteration's render."""

    def __init__(self, tracer: PathTracer, materials: np.ndarray, albedo_map: np.ndarray, views, targets,
                 spp: int = 16, max_bounces: int = 3, rough_ids=(), lr: float = 0.02, rough_bounds=(0.05, 1.0),
                 sampler: int = 0):
        import torch
        self.pt = tracer
        self.materials = np.array(materials, np.float32, copy=True).reshape(-1, 12)
        self.map_shape = albedo_map.shape
        self.rough_ids = np.asarray(rough_ids, np.int64)
        self.views = views
        self.targets = targets
        self.spp, self.max_bounces, self.sampler, self.lr = spp, max_bounces, sampler, lr
        n_map = int(np.prod(albedo_map.shape))
        self.theta = np.concatenate([np.asarray(albedo_map, np.float64).reshape(-1),
                                     self.materials[self.rough_ids, 4].astype(np.float64)])
        self.lo = np.concatenate([np.zeros(n_map), np.full(self.rough_ids.size, rough_bounds[0])])
        self.hi = np.concatenate([np.ones(n_map), np.full(self.rough_ids.size, rough_bounds[1])])
        self.n_map = n_map
        self.adam = Adam(self.theta.size)
        dev = torch.device("cuda", tracer.device)
        self.accums = [torch.zeros((v.height * v.width, 4), dtype=torch.float32, device=dev) for v in views]
        self.gmap = torch.zeros(n_map, dtype=torch.float32, device=dev)
        self.grough = torch.zeros(self.materials.shape[0], dtype=torch.float32, device=dev)
        self.iteration = 0
        self._upload()

    def _upload(self):
        self.pt.set_albedo_map(self.theta[:self.n_map].astype(np.float32).reshape(self.map_shape))
        self.materials[self.rough_ids, 4] = self.theta[self.n_map:].astype(np.float32)
        self.pt.update_materials(self.materials)

    def settings(self, sample_base: int) -> Settings:
        # decorrelated replay: the gradient of the loss of the expected image
        return make_settings(spp=self.spp, max_bounces=self.max_bounces, sample_index_base=sample_base,
                             sampler=self.sampler, flags=FLAG_ADJOINT_DECORRELATE)

    def gradient(self, sample_base: int):
        """(loss, d loss / d theta) at the current parameters; one adjoint call."""
        vs = [make_view(v, accum=a) for v, a in zip(self.views, self.accums)]
        loss = self.pt.adjoint(vs, self.settings(sample_base), self.targets, self.gmap, self.grough)
        g = np.concatenate([self.gmap.cpu().numpy().astype(np.float64),
                            self.grough.cpu().numpy().astype(np.float64)[self.rough_ids]])
        return loss, g

    def step(self) -> float:
        """One Adam iteration with fresh samples; returns the loss before it."""
        loss, g = self.gradient(sample_base=2 * self.iteration * self.spp)
        self.theta = self.adam.step(self.theta, g, self.lr, self.lo, self.hi)
        self._upload()
        self.iteration += 1
        return loss

    @property
    def albedo_map(self) -> np.ndarray:
        return self.theta[:self.n_map].reshape(self.map_shape)

    @property
    def roughness(self) -> np.ndarray:
        return self.theta[self.n_map:]
