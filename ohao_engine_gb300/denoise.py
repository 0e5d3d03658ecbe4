"""Learned denoiser (``include/ohao_dn.h``): ctypes binding and the training
data pipeline that renders noisy / reference pairs with the path tracer.

The GB300 replacement of the reference's OIDN pass
(ohao/render/rt/oidn_denoise.cpp:10-29). Every convolution of the U-Net runs
on tcgen05 tensor cores inside ``libohao_pt.so``; this module only moves
device pointers (torch tensors) across the C ABI and drives the loops.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import AOV_FLOATS, OhaoError, OK, _buffer, _ptr, load_library, make_settings, make_view

EXPORTED_SYMBOLS = [
    "ohao_dn_create", "ohao_dn_destroy", "ohao_dn_last_error", "ohao_dn_param_count", "ohao_dn_get_params",
    "ohao_dn_set_params", "ohao_dn_save", "ohao_dn_load", "ohao_dn_infer", "ohao_dn_train_step",
    "ohao_dn_get_grads", "ohao_dn_tensor", "ohao_dn_wait_selftest",
]


class _DnDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("seed", C.c_uint32), ("max_pixels", C.c_uint64)]


def _bind(L):
    if getattr(L, "_dn_bound", False):
        return L
    vp, u32, i32, u64, f32 = C.c_void_p, C.c_uint32, C.c_int32, C.c_uint64, C.c_float
    sigs = {
        "ohao_dn_create": ([C.POINTER(_DnDesc), C.POINTER(vp)], i32),
        "ohao_dn_destroy": ([vp], None),
        "ohao_dn_last_error": ([vp], C.c_char_p),
        "ohao_dn_param_count": ([vp], u64),
        "ohao_dn_get_params": ([vp, vp, u64], i32),
        "ohao_dn_set_params": ([vp, vp, u64], i32),
        "ohao_dn_save": ([vp, C.c_char_p], i32),
        "ohao_dn_load": ([vp, C.c_char_p], i32),
        "ohao_dn_infer": ([vp, C.POINTER(vp), C.POINTER(vp), u32, u32, u32, C.POINTER(vp), vp], i32),
        "ohao_dn_train_step": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), u32, u32, u32, f32,
                                C.POINTER(f32), vp], i32),
        "ohao_dn_get_grads": ([vp, vp, u64], i32),
        "ohao_dn_tensor": ([vp, i32, i32, vp, u64, C.POINTER(u32), C.POINTER(u64)], i32),
        "ohao_dn_wait_selftest": ([vp, u32, vp], i32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    L._dn_bound = True
    return L


def _frames(items, n: int, elems: int, what: str):
    """Pointer array of n device buffers of at least ``elems`` floats each
    (checked: the kernels read and write them without bounds)."""
    if len(items) != n:
        raise ValueError(f"{what}: {n} buffers expected, got {len(items)}")
    return (C.c_void_p * n)(*[_buffer(t, elems, what) for t in items])


class Denoiser:
    """One network on one GPU. Inputs are device tensors: radiance RGBA32F
    [h*w, 4] (an accumulator), AOV [h*w, 12] (ohao_pt_view.aov)."""

    def __init__(self, max_pixels: int, device: int = 0, seed: int = 1):
        self._L = _bind(load_library())
        d = _DnDesc(device, seed, max_pixels)
        h = C.c_void_p()
        st = self._L.ohao_dn_create(C.byref(d), C.byref(h))
        if st != OK:
            raise OhaoError(st, "ohao_dn_create failed")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self._L.ohao_dn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st != OK:
            raise OhaoError(st, f"{what}: {self._L.ohao_dn_last_error(self.h).decode()}")

    @property
    def param_count(self) -> int:
        return int(self._L.ohao_dn_param_count(self.h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count, np.float32)
        self._ck(self._L.ohao_dn_get_params(self.h, _ptr(p), p.size), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self._L.ohao_dn_set_params(self.h, _ptr(p), p.size), "set_params")

    def get_grads(self) -> np.ndarray:
        p = np.zeros(self.param_count, np.float32)
        self._ck(self._L.ohao_dn_get_grads(self.h, _ptr(p), p.size), "get_grads")
        return p

    def save(self, path: str):
        self._ck(self._L.ohao_dn_save(self.h, path.encode()), "save")

    def load(self, path: str):
        self._ck(self._L.ohao_dn_load(self.h, path.encode()), "load")

    def infer(self, radiance, aov, out, width: int, height: int, stream=None):
        n, npix = len(radiance), width * height
        self._ck(self._L.ohao_dn_infer(self.h, _frames(radiance, n, npix * 4, "radiance"),
                                       _frames(aov, n, npix * AOV_FLOATS, "aov"), n, width, height,
                                       _frames(out, n, npix * 4, "out"),
                                       _ptr(stream) if stream is not None else None), "infer")

    def train_step(self, radiance, aov, target, width: int, height: int, lr: float, stream=None) -> float:
        loss = C.c_float()
        n, npix = len(radiance), width * height
        self._ck(self._L.ohao_dn_train_step(self.h, _frames(radiance, n, npix * 4, "radiance"),
                                            _frames(aov, n, npix * AOV_FLOATS, "aov"),
                                            _frames(target, n, npix * 4, "target"), n,
                                            width, height, lr, C.byref(loss),
                                            _ptr(stream) if stream is not None else None), "train_step")
        return loss.value

    def wait_selftest(self, spin_limit: int = 1024, stream=None) -> int:
        """Status of ohao_dn_wait_selftest: a bounded tensor-core pipeline
        wait that is made to run out (OHAO_ERR_TIMEOUT, -4, expected)."""
        return int(self._L.ohao_dn_wait_selftest(self.h, spin_limit, _ptr(stream) if stream is not None else None))

    def tensor(self, index: int, grad: bool = False) -> np.ndarray:
        ch, px = C.c_uint32(), C.c_uint64()
        self._ck(self._L.ohao_dn_tensor(self.h, index, int(grad), None, 0, C.byref(ch), C.byref(px)), "tensor")
        out = np.zeros((px.value, ch.value), np.float32)
        self._ck(self._L.ohao_dn_tensor(self.h, index, int(grad), _ptr(out), out.size, C.byref(ch), C.byref(px)),
                 "tensor")
        return out


def training_scene(seed: int, side: int = 256, freq: int = 64, env_size=(512, 256)):
    """A scene of the single-object family: displaced geodesic sphere with
    per-triangle GGX materials on a plane under a sky + sun environment, seen
    from a seeded camera."""
    import math
    from . import scenes
    sd = scenes.sphere_1m(width=side, height=side, freq=freq, seed=seed, env_size=env_size)
    rng = np.random.default_rng(seed + 7919)
    az, el, dist = rng.uniform(0, 2 * math.pi), rng.uniform(0.05, 0.6), rng.uniform(2.4, 4.2)
    eye = (dist * math.cos(az) * math.cos(el), 0.1 + dist * math.sin(el), dist * math.sin(az) * math.cos(el))
    sd.views = [scenes.look_at_view(eye, (0.0, -0.1, 0.0), fov_y_deg=float(rng.uniform(30, 50)), width=side,
                                    height=side)]
    return sd


def tonemap(rgb):
    """The reference's display transform: pow(ACES(x * 0.5), 1/2.2) with
    ACES(x) = clamp(x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14), 0, 1)
    (pt_raygen.rgen:99-102, 1263-1264)."""
    x = np.maximum(np.asarray(rgb, np.float64), 0.0) * 0.5
    y = np.clip((x * (2.51 * x + 0.03)) / (x * (2.43 * x + 0.59) + 0.14), 0.0, 1.0)
    return y ** (1.0 / 2.2)


def render_pair(pt, view, width, height, spp_noisy, spp_ref, seed_base, max_bounces=4, aov_spp=1):
    """(noisy accum, aov, reference accum) device tensors of one view: the
    noisy image at spp_noisy, its first-hit AOVs (the render's record of its
    last sample, or with aov_spp > 1 the mean over aov_spp camera samples of
    their own, ohao_pt_aov) and an independent reference at spp_ref."""
    import torch
    npix = width * height
    noisy = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    aov = torch.zeros((npix, AOV_FLOATS), dtype=torch.float32, device="cuda")
    ref = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    pt.render([make_view(view, accum=noisy, aov=aov if aov_spp <= 1 else None)],
              make_settings(spp=spp_noisy, max_bounces=max_bounces, sample_index_base=seed_base))
    if aov_spp > 1:
        pt.aov(make_view(view), make_settings(spp=aov_spp, max_bounces=max_bounces,
                                              sample_index_base=seed_base + (1 << 19)), aov)
    pt.render([make_view(view, accum=ref)],
              make_settings(spp=spp_ref, max_bounces=max_bounces, sample_index_base=seed_base + (1 << 20)))
    return noisy, aov, ref
