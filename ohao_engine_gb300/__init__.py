"""GB300-native path-tracing hot path of the OHAO engine (Python host mirror).

This package loads ``_lib/libohao_pt.so`` -- the C ABI declared in
``include/ohao_pt.h`` -- and mirrors the reference's host objects around it:

* :class:`PathTracer` -- PathTracer's inputs and render call
  (``ohao/render/rt/path_tracer.hpp:61-194``) plus RTAccelerationStructure's
  createBLAS / addInstance / buildTLAS (``rt_acceleration_structure.hpp:73-107``);
* :class:`EnvCDF` -- ``ohao/render/rt/env_cdf.hpp:12-43``.

Failures raise :class:`OhaoError` carrying the ABI status and message. There
is no CPU fallback: without the compiled library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import scenes  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libohao_pt.so")

OK = 0
STATUS_NAMES = {0: "OK", -1: "INVALID_ARG", -2: "OOM", -3: "CUDA_ERROR", -4: "TIMEOUT", -5: "NOT_BUILT",
                -6: "UNSUPPORTED", -7: "DEVICE_CHECK"}
SAMPLER_PCG, SAMPLER_SOBOL = 0, 1
FLAG_FIREFLY_CLAMP = 1 << 2
FLAG_ENV_FIXED_V = 1 << 8
FLAG_ALPHA_TEST = 1 << 10     # non-opaque rays: alpha test on OHAO_BLAS_FLAG_NO_OPAQUE geometry
FLAG_SORT_MATERIAL = 1 << 11  # shade each ray queue in material order (same image)
FLAG_SORT_RAYS = 1 << 12      # trace each bounce's rays grouped by direction and origin (same image)
BLAS_FLAG_NO_OPAQUE = 1
FLAG_GGX_VNDF = 1 << 9        # VNDF sampling of the first specular bounce (not the offline estimator)
FLAG_EMITTER_MIS = 1 << 13     # emissive triangles in the light NEE, sphere / area lights hit by BSDF rays, MIS
FLAG_PROFILE = 1 << 16
FLAG_ADJOINT_DECORRELATE = 1 << 17
FLAG_ADJOINT_LDR_LOSS = 1 << 18   # loss on display values (the reference's mseRGB), targets in [0, 1]
MODE_AUTO, MODE_WAVEFRONT, MODE_PERSISTENT = 0, 1, 2
AOV_FLOATS = 12   # OHAO_PT_AOV_FLOATS: first-hit record per pixel (ohao_pt_view.aov)

EXPORTED_SYMBOLS = [
    "ohao_pt_create", "ohao_pt_destroy", "ohao_pt_last_error", "ohao_pt_version", "ohao_pt_set_geometry",
    "ohao_pt_create_blas", "ohao_pt_set_instances", "ohao_pt_build", "ohao_pt_is_two_level",
    "ohao_pt_set_materials", "ohao_pt_update_materials", "ohao_pt_set_lights", "ohao_pt_set_env",
    "ohao_pt_set_albedo_map", "ohao_env_cdf_build", "ohao_pt_render", "ohao_pt_render_host",
    "ohao_pt_get_profile", "ohao_pt_trace", "ohao_pt_bvh_info", "ohao_pt_bvh_download", "ohao_bvh_build_noalloc",
    "ohao_pt_autotune", "ohao_pt_launch_config", "ohao_pt_launch_config_at", "ohao_pt_set_launch_config",
    "ohao_pt_backward", "ohao_pt_adjoint", "ohao_pt_display", "ohao_pt_set_geometry_device",
    "ohao_pt_adjoint_host", "ohao_pt_set_textures", "ohao_pt_set_blas_flags", "ohao_pt_aov",
]


class OhaoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class _Desc(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32), ("flatten_limit", C.c_uint64)]


class View(C.Structure):
    """ohao_pt_view"""
    _fields_ = [("inv_view", C.c_float * 16), ("inv_proj", C.c_float * 16), ("width", C.c_uint32),
                ("height", C.c_uint32), ("history", C.c_uint32), ("reserved", C.c_uint32),
                ("accum", C.c_void_p), ("path_radiance", C.c_void_p), ("aov", C.c_void_p),
                ("display", C.c_void_p)]


class Settings(C.Structure):
    """ohao_pt_settings"""
    _fields_ = [("spp", C.c_uint32), ("max_bounces", C.c_uint32), ("sample_index_base", C.c_uint32),
                ("sampler", C.c_uint32), ("flags", C.c_uint32), ("clamp_luminance", C.c_float),
                ("aniso_strength", C.c_float), ("aniso_rotation", C.c_float), ("mode", C.c_uint32),
                ("trace_stack_limit", C.c_uint32), ("wavefront_refill", C.c_uint32), ("reserved", C.c_uint32 * 5)]


class Texture(C.Structure):
    """ohao_pt_texture"""
    _fields_ = [("rgba8", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32)]


class Profile(C.Structure):
    _fields_ = [("extend_ms", C.c_float), ("shadow_ms", C.c_float), ("shade_ms", C.c_float),
                ("other_ms", C.c_float), ("total_ms", C.c_float), ("extend_launches", C.c_uint32),
                ("shadow_launches", C.c_uint32), ("shade_launches", C.c_uint32), ("other_launches", C.c_uint32),
                ("rays_closest", C.c_uint64), ("rays_shadow", C.c_uint64), ("nodes_closest", C.c_uint64),
                ("tris_closest", C.c_uint64), ("nodes_shadow", C.c_uint64), ("tris_shadow", C.c_uint64),
                ("lanes", C.c_uint32), ("reserved", C.c_uint32)]


_lib = None


def load_library(path: str | None = None):
    """Load libohao_pt.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OhaoError(-5, f"{p} not built; run __graft_entry__.build() or python -m ohao_engine_gb300._build")
    L = C.CDLL(p)
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int32, C.c_float
    sigs = {
        "ohao_pt_create": ([C.POINTER(_Desc), C.POINTER(vp)], i32),
        "ohao_pt_destroy": ([vp], None),
        "ohao_pt_last_error": ([vp], C.c_char_p),
        "ohao_pt_version": ([], C.c_char_p),
        "ohao_pt_set_geometry": ([vp, vp, u32, u32, vp, vp, vp, u32, vp], i32),
        "ohao_pt_create_blas": ([vp, u32, u32, C.POINTER(u32)], i32),
        "ohao_pt_set_instances": ([vp, vp, u32], i32),
        "ohao_pt_build": ([vp, vp], i32),
        "ohao_pt_is_two_level": ([vp], i32),
        "ohao_pt_set_materials": ([vp, vp, u32], i32),
        "ohao_pt_update_materials": ([vp, vp, u32, u32], i32),
        "ohao_pt_set_lights": ([vp, vp, u32], i32),
        "ohao_pt_set_env": ([vp, vp, u32, u32, vp, vp, f32, f32], i32),
        "ohao_pt_set_albedo_map": ([vp, vp, u32, u32], i32),
        "ohao_env_cdf_build": ([vp, i32, i32, vp, vp, vp], i32),
        "ohao_pt_render": ([vp, C.POINTER(View), u32, C.POINTER(Settings), vp], i32),
        "ohao_pt_render_host": ([vp, C.POINTER(View), u32, C.POINTER(Settings), C.POINTER(vp), vp], i32),
        "ohao_pt_get_profile": ([vp, C.POINTER(Profile)], i32),
        "ohao_pt_trace": ([vp, vp, u32, vp, i32, vp, vp], i32),
        "ohao_pt_bvh_info": ([vp, i32, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)], i32),
        "ohao_pt_bvh_download": ([vp, i32, vp, vp], i32),
        "ohao_bvh_build_noalloc": ([vp, u32, vp, vp, vp, C.POINTER(u32), C.POINTER(u32), vp], i32),
        "ohao_pt_autotune": ([vp, C.POINTER(View), u32, C.POINTER(Settings), C.POINTER(f32), vp], i32),
        "ohao_pt_launch_config": ([vp], C.c_char_p),
        "ohao_pt_launch_config_at": ([u32], C.c_char_p),
        "ohao_pt_set_launch_config": ([vp, C.c_char_p], i32),
        "ohao_pt_backward": ([vp, C.POINTER(View), u32, C.POINTER(Settings), C.POINTER(vp), vp, vp, vp], i32),
        "ohao_pt_adjoint": ([vp, C.POINTER(View), u32, C.POINTER(Settings), C.POINTER(vp), vp, vp,
                                   C.POINTER(f32), vp], i32),
        "ohao_pt_display": ([vp, u32, vp, vp], i32),
        "ohao_pt_aov": ([vp, C.POINTER(View), C.POINTER(Settings), vp, vp], i32),
        "ohao_pt_set_textures": ([vp, vp, u32], i32),
        "ohao_pt_set_blas_flags": ([vp, u32, u32], i32),
        "ohao_pt_adjoint_host": ([vp, C.POINTER(View), u32, C.POINTER(Settings), C.POINTER(vp), vp, vp,
                                  C.POINTER(f32), vp], i32),
        "ohao_pt_set_geometry_device": ([vp, vp, u32, u32, vp, vp, vp, u32, vp, vp], i32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(int(a))


class EnvCDF:
    """ohao::EnvCDF -- marginal + conditional luminance CDFs of an RGBA32F map."""

    def __init__(self):
        self.width = self.height = 0
        self.integral = 0.0
        self.marginal = np.zeros(0, np.float32)
        self.conditional = np.zeros(0, np.float32)

    def build(self, pixels: np.ndarray, width: int | None = None, height: int | None = None) -> "EnvCDF":
        px = np.ascontiguousarray(pixels, np.float32)
        h = height or px.shape[0]
        w = width or px.shape[1]
        self.marginal = np.zeros(h, np.float32)
        self.conditional = np.zeros(w * h, np.float32)
        integ = np.zeros(1, np.float32)
        st = load_library().ohao_env_cdf_build(_ptr(px), w, h, _ptr(self.marginal), _ptr(self.conditional), _ptr(integ))
        if st != OK:
            raise OhaoError(st, "ohao_env_cdf_build failed")
        self.width, self.height, self.integral = w, h, float(integ[0])
        return self

    def valid(self) -> bool:
        return self.width > 0 and self.height > 0 and self.marginal.size > 0


def _buffer(a, elems: int, what: str, host: bool = False, floats: bool = True):
    """Pointer value of a buffer that the kernels (or, with ``host``, the
    library's copies) use without bounds checks: a contiguous array or tensor
    of 4-byte elements (float32 unless ``floats`` is False), at least
    ``elems`` long, on a CUDA device (in host memory with ``host``). A wrong
    buffer raises ValueError here instead of faulting the device; raw integer
    pointers pass unchecked."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not host:
            raise ValueError(f"{what}: a host array where a CUDA device buffer is needed")
        ok = (a.flags.c_contiguous and a.flags.writeable and a.itemsize == 4
              and (a.dtype == np.float32 or not floats) and a.size >= elems)
        if not ok:
            raise ValueError(f"{what}: needs a writable C-contiguous float32 array of at least {elems} elements "
                             f"(got {a.shape} {a.dtype})")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        ok = (a.element_size() == 4 and (a.is_floating_point() or not floats) and a.is_contiguous()
              and a.numel() >= elems)
        if not ok:
            raise ValueError(f"{what}: needs a contiguous {'float32' if floats else '4-byte'} tensor of at least "
                             f"{elems} elements (got {tuple(a.shape)} {a.dtype})")
        if bool(a.is_cuda) == host:
            raise ValueError(f"{what}: needs a {'host' if host else 'CUDA device'} tensor (got one on {a.device})")
        return a.data_ptr()
    return int(a)


def _bytes(a, nbytes: int, what: str, host: bool):
    """Pointer value of a uint8 buffer of at least nbytes (device memory, or
    host memory with ``host``); a wrong buffer raises ValueError."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not host:
            raise ValueError(f"{what}: a host array where a CUDA device buffer is needed")
        if not (a.flags.c_contiguous and a.flags.writeable and a.dtype == np.uint8 and a.size >= nbytes):
            raise ValueError(f"{what}: needs a writable C-contiguous uint8 array of at least {nbytes} bytes")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not (a.element_size() == 1 and a.is_contiguous() and a.numel() >= nbytes):
            raise ValueError(f"{what}: needs a contiguous uint8 tensor of at least {nbytes} bytes")
        if bool(a.is_cuda) == host:
            raise ValueError(f"{what}: needs a {'host' if host else 'CUDA device'} tensor (got one on {a.device})")
        return a.data_ptr()
    return int(a)


def display(rgba32f, npix: int, out_rgba8, stream=None):
    """ohao_pt_display: RGBA8 display image of npix device RGBA32F texels."""
    st = load_library().ohao_pt_display(_ptr(_buffer(rgba32f, npix * 4, "rgba32f")), npix,
                                        _ptr(_bytes(out_rgba8, npix * 4, "rgba8", False)),
                                        _ptr(stream) if stream is not None else None)
    if st != OK:
        raise OhaoError(st, "ohao_pt_display failed")


def make_view(view, accum=None, history: int = 0, path_radiance=None, aov=None, display=None,
              display_host: bool = False) -> View:
    """One ``ohao_pt_view``. accum: RGBA32F per pixel; path_radiance: RGBA32F
    per sample and pixel ([spp][pixel][4], for up to as many samples per call
    as it holds); aov: AOV_FLOATS per pixel; all on the device. display:
    RGBA8 per pixel (uint8, 4 per pixel), on the device, or in host memory
    with display_host for render_host."""
    v = View()
    v.inv_view[:] = [float(x) for x in np.asarray(view.inv_view, np.float32)]
    v.inv_proj[:] = [float(x) for x in np.asarray(view.inv_proj, np.float32)]
    v.width, v.height, v.history = int(view.width), int(view.height), int(history)
    npix = v.width * v.height
    v.accum = _buffer(accum, npix * 4, "accum")
    v.path_radiance = _buffer(path_radiance, npix * 4, "path_radiance")
    v.aov = _buffer(aov, npix * AOV_FLOATS, "aov")
    v.display = _bytes(display, npix * 4, "display", display_host)
    if path_radiance is not None and hasattr(path_radiance, "numel") and npix:
        v._path_samples = path_radiance.numel() // (npix * 4)
    return v


def _view_array(views, settings: "Settings"):
    """ctypes array of the views, after checking that every per-sample
    radiance buffer holds the call's samples."""
    for v in views:
        ns = getattr(v, "_path_samples", None)
        if ns is not None and settings.spp > ns:
            raise ValueError(f"path_radiance holds {ns} samples per pixel, the call renders {settings.spp}")
    return (View * len(views))(*views)


def make_settings(spp=1, max_bounces=4, sample_index_base=0, sampler=SAMPLER_PCG, flags=0, clamp_luminance=0.0,
                  aniso_strength=0.0, aniso_rotation=0.0, mode=MODE_AUTO, trace_stack_limit=0,
                  wavefront_refill=0) -> Settings:
    s = Settings()
    s.trace_stack_limit = trace_stack_limit
    s.wavefront_refill = wavefront_refill
    s.spp, s.max_bounces, s.sample_index_base, s.sampler = spp, max_bounces, sample_index_base, sampler
    s.flags, s.clamp_luminance, s.aniso_strength, s.aniso_rotation, s.mode = (flags, clamp_luminance,
                                                                             aniso_strength, aniso_rotation, mode)
    return s


class PathTracer:
    """Context wrapper: scene inputs, LBVH/TLAS build and render on one GPU."""

    def __init__(self, device: int = 0, flatten_limit: int = 0):
        self._L = load_library()
        d = _Desc(device, 0, flatten_limit)
        h = C.c_void_p()
        st = self._L.ohao_pt_create(C.byref(d), C.byref(h))
        if st != OK:
            raise OhaoError(st, "ohao_pt_create failed")
        self.h = h
        self.device = device
        self._keep = {}
        self._nmats = 0        # material table size (gradient buffer bounds)
        self._map_floats = 0   # tile albedo map floats (gradient buffer bounds)

    def close(self):
        if getattr(self, "h", None):
            self._L.ohao_pt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st: int, what: str):
        if st != OK:
            msg = self._L.ohao_pt_last_error(self.h)
            raise OhaoError(st, f"{what}: {msg.decode() if msg else ''}")

    # -- inputs --------------------------------------------------------------
    def set_geometry(self, pos, normals, uvs, indices, mat_ids, pos_stride_bytes: int = 12):
        pos = np.ascontiguousarray(pos, np.float32)
        nrm = np.ascontiguousarray(normals, np.float32)
        uv = None if uvs is None else np.ascontiguousarray(uvs, np.float32)
        idx = np.ascontiguousarray(indices, np.uint32)
        mid = np.ascontiguousarray(mat_ids, np.uint32)
        nverts = pos.size * 4 // pos_stride_bytes
        self._ck(self._L.ohao_pt_set_geometry(self.h, _ptr(pos), pos_stride_bytes, nverts, _ptr(nrm), _ptr(uv),
                                              _ptr(idx), idx.size // 3, _ptr(mid)), "set_geometry")

    def set_geometry_device(self, pos, normals, uvs, indices, mat_ids, nverts: int, ntris: int,
                            pos_stride_bytes: int = 12, stream=None):
        """ohao_pt_set_geometry_device: the geometry from CUDA tensors
        (positions at pos_stride_bytes, float4 normals, float2 UVs or None,
        uint32 indices and material ids), ordered on `stream`."""
        pf = pos_stride_bytes // 4
        p = _buffer(pos, max(nverts - 1, 0) * pf + 3 if nverts else 0, "pos")
        n = _buffer(normals, nverts * 4, "normals")
        u = _buffer(uvs, nverts * 2, "uvs")
        i = _buffer(indices, ntris * 3, "indices", floats=False)
        m = _buffer(mat_ids, ntris, "mat_ids", floats=False)
        self._ck(self._L.ohao_pt_set_geometry_device(self.h, p, pos_stride_bytes, nverts, n, u, i, ntris, m,
                                                     _ptr(stream) if stream is not None else None),
                 "set_geometry_device")

    def create_blas(self, first_index: int, index_count: int) -> int:
        out = C.c_uint32()
        self._ck(self._L.ohao_pt_create_blas(self.h, first_index, index_count, C.byref(out)), "create_blas")
        return out.value

    def set_instances(self, inst: np.ndarray):
        inst = np.ascontiguousarray(inst, scenes.INSTANCE_DTYPE)
        self._ck(self._L.ohao_pt_set_instances(self.h, _ptr(inst), inst.size), "set_instances")

    def build(self, stream=None):
        self._ck(self._L.ohao_pt_build(self.h, _ptr(stream) if stream is not None else None), "build")

    @property
    def two_level(self) -> bool:
        return bool(self._L.ohao_pt_is_two_level(self.h))

    def set_materials(self, mats):
        m = np.ascontiguousarray(mats, np.float32).reshape(-1, 12)
        self._ck(self._L.ohao_pt_set_materials(self.h, _ptr(m), m.shape[0]), "set_materials")
        self._nmats = m.shape[0]

    def update_materials(self, mats, first: int = 0):
        m = np.ascontiguousarray(mats, np.float32).reshape(-1, 12)
        self._ck(self._L.ohao_pt_update_materials(self.h, _ptr(m), first, m.shape[0]), "update_materials")

    def set_lights(self, lights):
        l = np.ascontiguousarray(lights, np.float32).reshape(-1, 20)
        self._ck(self._L.ohao_pt_set_lights(self.h, _ptr(l), l.shape[0]), "set_lights")

    def set_textures(self, textures):
        """Bindless RGBA8 textures, each a (h, w, 4) uint8 array."""
        arrs = [np.ascontiguousarray(t, np.uint8) for t in textures]
        for a in arrs:
            if a.ndim != 3 or a.shape[2] != 4:
                raise ValueError("set_textures: each texture is a (height, width, 4) uint8 array")
        tex = (Texture * max(len(arrs), 1))(*[Texture(a.ctypes.data, a.shape[1], a.shape[0]) for a in arrs])
        self._ck(self._L.ohao_pt_set_textures(self.h, tex, len(arrs)), "set_textures")

    def set_blas_flags(self, blas: int, flags: int):
        self._ck(self._L.ohao_pt_set_blas_flags(self.h, blas, flags), "set_blas_flags")

    def set_env(self, rgba, cdf: EnvCDF | None = None, intensity: float = 1.0, importance_sampling: bool = True):
        if rgba is None:
            self._ck(self._L.ohao_pt_set_env(self.h, None, 0, 0, None, None, 0.0, 0.0), "set_env")
            return
        env = np.ascontiguousarray(rgba, np.float32)
        h, w = env.shape[:2]
        if importance_sampling and cdf is None:
            cdf = EnvCDF().build(env)
        self._keep["env"] = (env, cdf)
        self._ck(self._L.ohao_pt_set_env(self.h, _ptr(env), w, h, _ptr(cdf.marginal) if cdf else None,
                                         _ptr(cdf.conditional) if cdf else None, cdf.integral if cdf else 0.0,
                                         intensity), "set_env")

    def set_albedo_map(self, rgb):
        m = np.ascontiguousarray(rgb, np.float32)
        self._ck(self._L.ohao_pt_set_albedo_map(self.h, _ptr(m), m.shape[1], m.shape[0]), "set_albedo_map")
        self._map_floats = m.shape[0] * m.shape[1] * 3

    def load_scene(self, sd, build: bool = True):
        """Upload a :class:`scenes.SceneData` and build its BVH."""
        self.set_geometry(sd.pos, sd.normals, sd.uvs, sd.indices, sd.mat_ids)
        for k, (fi, ic) in enumerate(sd.blas):
            b = self.create_blas(fi, ic)
            if sd.blas_flags:
                self.set_blas_flags(b, int(sd.blas_flags[k]))
        if sd.textures:
            self.set_textures(sd.textures)
        self.set_instances(sd.instances)
        self.set_materials(sd.materials)
        if sd.lights is not None and len(sd.lights):
            self.set_lights(sd.lights)
        if sd.env is not None:
            self.set_env(sd.env, intensity=sd.env_intensity)
        if sd.albedo_map is not None:
            self.set_albedo_map(sd.albedo_map)
        if build:
            self.build()

    # -- render --------------------------------------------------------------
    def render(self, views, settings: Settings, stream=None):
        arr = _view_array(views, settings)
        self._ck(self._L.ohao_pt_render(self.h, arr, len(views), C.byref(settings),
                                        _ptr(stream) if stream is not None else None), "render")

    def render_host(self, views, settings: Settings, host_accum, stream=None):
        arr = _view_array(views, settings)
        if len(host_accum) != len(views):
            raise ValueError("render_host: one host accumulator per view")
        ptrs = (C.c_void_p * len(views))(*[_buffer(a, v.width * v.height * 4, "host_accum", host=True)
                                           for a, v in zip(host_accum, views)])
        self._ck(self._L.ohao_pt_render_host(self.h, arr, len(views), C.byref(settings), ptrs,
                                             _ptr(stream) if stream is not None else None), "render_host")

    def aov(self, view, settings: Settings, out, stream=None):
        """ohao_pt_aov: first-hit features of `view` averaged over
        settings.spp camera samples into the device buffer `out`
        (AOV_FLOATS per pixel)."""
        arr = _view_array([view], settings)
        self._ck(self._L.ohao_pt_aov(self.h, arr, C.byref(settings),
                                     _ptr(_buffer(out, view.width * view.height * AOV_FLOATS, "aov")),
                                     _ptr(stream) if stream is not None else None), "aov")

    def autotune(self, views, settings: Settings, stream=None) -> float:
        arr = _view_array(views, settings)
        ms = C.c_float()
        self._ck(self._L.ohao_pt_autotune(self.h, arr, len(views), C.byref(settings), C.byref(ms),
                                          _ptr(stream) if stream is not None else None), "autotune")
        return ms.value

    # -- gradients -----------------------------------------------------------
    def backward(self, views, settings: Settings, grad_images, grad_map=None, grad_rough=None, stream=None):
        """d loss / d (albedo map, roughness) from per-view d loss / d image
        (device RGBA32F); writes the device buffers grad_map / grad_rough."""
        arr = _view_array(views, settings)
        ptrs = self._image_ptrs(views, grad_images, "grad_images")
        gm, gr = self._grad_ptrs(grad_map, grad_rough)
        self._ck(self._L.ohao_pt_backward(self.h, arr, len(views), C.byref(settings), ptrs, gm, gr,
                                          _ptr(stream) if stream is not None else None), "backward")

    def adjoint(self, views, settings: Settings, targets, grad_map=None, grad_rough=None, stream=None) -> float:
        """Renders the views (history 0), returns the multi-view RGB MSE against
        the device RGBA32F targets and writes its gradients."""
        arr = _view_array(views, settings)
        ptrs = self._image_ptrs(views, targets, "targets")
        gm, gr = self._grad_ptrs(grad_map, grad_rough)
        loss = C.c_float()
        self._ck(self._L.ohao_pt_adjoint(self.h, arr, len(views), C.byref(settings), ptrs, gm, gr, C.byref(loss),
                                         _ptr(stream) if stream is not None else None), "adjoint")
        return loss.value

    def adjoint_host(self, views, settings: Settings, host_targets, grad_map=None, grad_rough=None) -> float:
        """ohao_pt_adjoint_host: targets and gradients in host (numpy) memory."""
        arr = _view_array(views, settings)
        if len(host_targets) != len(views):
            raise ValueError("adjoint_host: one host target per view")
        tp = (C.c_void_p * len(views))(*[_buffer(t, v.width * v.height * 4, "host_targets", host=True)
                                         for t, v in zip(host_targets, views)])
        gm = _buffer(grad_map, self._map_floats, "grad_map", host=True)
        gr = _buffer(grad_rough, self._nmats, "grad_rough", host=True)
        loss = C.c_float()
        self._ck(self._L.ohao_pt_adjoint_host(self.h, arr, len(views), C.byref(settings), tp, gm, gr, C.byref(loss),
                                              None), "adjoint_host")
        return loss.value

    @staticmethod
    def _image_ptrs(views, images, what):
        if len(images) != len(views):
            raise ValueError(f"{what}: one RGBA32F image per view")
        return (C.c_void_p * len(views))(*[_buffer(g, v.width * v.height * 4, what) for g, v in zip(images, views)])

    def _grad_ptrs(self, grad_map, grad_rough):
        return (_buffer(grad_map, self._map_floats, "grad_map"),
                _buffer(grad_rough, self._nmats, "grad_rough"))

    @property
    def launch_config(self) -> str:
        return self._L.ohao_pt_launch_config(self.h).decode()

    @launch_config.setter
    def launch_config(self, name: str) -> None:
        self._ck(self._L.ohao_pt_set_launch_config(self.h, name.encode()), "set_launch_config")

    def launch_configs(self) -> list:
        """Names of the compiled persistent launch shapes."""
        out, i = [], 0
        while True:
            n = self._L.ohao_pt_launch_config_at(i)
            if n is None:
                return out
            out.append(n.decode())
            i += 1

    def profile(self) -> Profile:
        p = Profile()
        self._ck(self._L.ohao_pt_get_profile(self.h, C.byref(p)), "get_profile")
        return p

    def trace(self, rays_dev, n: int, hits_dev, any_hit: bool = False, stats_dev=None, stream=None,
              alpha: bool = False):
        rays = _buffer(rays_dev, 8 * n, "rays")
        hits = _buffer(hits_dev, 5 * n, "hits", floats=False)
        stats = _buffer(stats_dev, 2 * n, "stats", floats=False)
        self._ck(self._L.ohao_pt_trace(self.h, rays, n, hits, int(any_hit) | (2 if alpha else 0), stats,
                                       _ptr(stream) if stream is not None else None), "trace")

    def bvh(self, which: int = -1):
        nn, npr, hh = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._ck(self._L.ohao_pt_bvh_info(self.h, which, C.byref(nn), C.byref(npr), C.byref(hh)), "bvh_info")
        nodes = np.zeros(nn.value * 80, np.uint8)
        pb = 4 if (which < 0 and self.two_level) else 48
        prims = np.zeros(npr.value * pb, np.uint8)
        self._ck(self._L.ohao_pt_bvh_download(self.h, which, _ptr(nodes), _ptr(prims)), "bvh_download")
        return nodes, prims, hh.value


def version() -> str:
    return load_library().ohao_pt_version().decode()
