"""ctypes binding of the host oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU-baseline
leg, always as the checker or the timed CPU baseline, never as part of the
product path. ``build()`` compiles ``oracle/_build/liboracle.so`` with the
Makefile beside this file.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libohao_ref.so")
GLSL_PATH = os.path.join(HERE, "_ref", "libohao_glsl.so")
REF_ROOT = os.environ.get("OHAO_REFERENCE_ROOT", "/root/reference")   # the reference checkout, where present

_lib = None


def build(ref: bool | None = None) -> None:
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_ROOT, "ohao"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True)
        import glsl_pin
        if glsl_pin.available(REF_ROOT):
            glsl_pin.build(REF_ROOT)
        if glsl_pin.pt_available(REF_ROOT):
            glsl_pin.build_pt(REF_ROOT)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        vp, u32, i32, f32, u64 = C.c_void_p, C.c_uint32, C.c_int, C.c_float, C.c_uint64
        L.orc_scene_create.restype = vp
        L.orc_scene_destroy.argtypes = [vp]
        L.orc_scene_set_geometry.argtypes = [vp, vp, u32, u32, vp, vp, vp, u32, vp]
        L.orc_scene_set_materials.argtypes = [vp, vp, u32]
        L.orc_scene_set_lights.argtypes = [vp, vp, u32]
        L.orc_scene_set_env.argtypes = [vp, vp, u32, u32, vp, vp, f32, f32]
        L.orc_scene_set_albedo_map.argtypes = [vp, vp, u32, u32]
        L.orc_scene_set_textures.argtypes = [vp, vp, vp, u32]
        L.orc_scene_set_blas_flags.argtypes = [vp, u32, u32]
        L.orc_alpha_accept.argtypes = [vp, vp, vp, vp, u32, vp]
        L.orc_emitter_table.argtypes = [vp, vp, vp]
        L.orc_emitter_table.restype = u32
        L.orc_light_samples.argtypes = [vp, u32, vp, vp, u32, u32, vp]
        L.orc_scene_add_blas.argtypes = [vp, u32, u32]
        L.orc_scene_add_blas.restype = u32
        L.orc_scene_set_instances.argtypes = [vp, vp, u32]
        L.orc_scene_build.argtypes = [vp, u64, i32]
        L.orc_scene_two_level.argtypes = [vp]
        L.orc_scene_two_level.restype = i32
        L.orc_bvh_sizes.argtypes = [vp, i32, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]
        L.orc_bvh_copy.argtypes = [vp, i32, vp, vp]
        L.orc_trace.argtypes = [vp, vp, u32, vp, i32, vp, i32]
        L.orc_render_paths.argtypes = [vp, vp, vp, u32, u32, vp, u32, u32, vp, u32, vp, i32, i32, vp]
        L.orc_accumulate.argtypes = [vp, u32, u32, vp, u32]
        L.orc_detached_paths.argtypes = [vp, vp, vp, u32, u32, vp, u32, u32, vp, u32, vp, vp, vp, i32]
        L.orc_detached_grad.argtypes = [vp, vp, vp, u32, u32, vp, u32, u32, vp, vp, u32, vp, u32, i32, vp, i32]
        L.orc_detached_grad.restype = i32
        L.orc_env_cdf_build.argtypes = [vp, i32, i32, vp, vp, vp]
        L.orc_sobol_sample1d.argtypes = [u32, u32]
        L.orc_sobol_sample1d.restype = f32
        L.orc_owen_scramble.argtypes = [u32, u32]
        L.orc_owen_scramble.restype = u32
        L.orc_sampler_stream.argtypes = [u32, u32, u32, u32, u32, vp]
        L.orc_math.argtypes = [i32, vp, u32, vp]
        L.orc_num_threads.restype = i32
        L.orc_display_rgba8.argtypes = [vp, u64, vp]
        L.orc_pow_def.argtypes = [vp, u64, f32, vp]
        L.orc_glsl_helper.argtypes = [i32, vp, u32, vp]
        L.orc_glsl_helper.restype = i32
        L.orc_glsl_env.argtypes = [i32, vp, vp, u32, u32, vp, u32, vp]
        L.orc_glsl_env.restype = i32
        _lib = L
    return _lib


def ref_lib():
    """The reference's own helpers (only where the reference tree exists)."""
    if not os.path.exists(REF_PATH):
        return None
    L = C.CDLL(REF_PATH)
    L.ref_env_cdf_build.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_sobol_sample1d.argtypes = [C.c_uint32, C.c_uint32]
    L.ref_sobol_sample1d.restype = C.c_float
    L.ref_owen_scramble.argtypes = [C.c_uint32, C.c_uint32]
    L.ref_owen_scramble.restype = C.c_uint32
    L.ref_sobol_dirs.restype = C.POINTER(C.c_uint32)
    return L


def glsl_lib():
    """The reference's GLSL helper includes compiled as C++ (glsl_pin.py; only
    where the reference tree exists)."""
    if not os.path.exists(GLSL_PATH):
        return None
    L = C.CDLL(GLSL_PATH)
    L.gref_helper.argtypes = [C.c_int, C.c_void_p, C.c_uint32, C.c_void_p]
    L.gref_helper.restype = C.c_int
    L.gref_env.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
    L.gref_env.restype = C.c_int
    return L


def glsl_pt_lib(variant: str = "base"):
    """The reference's raygen ("base": pt_raygen.rgen, "offline":
    pt_raygen_offline.rgen) with its closest-hit and miss shaders compiled as
    C++ over the oracle's scenes (glsl_pin.py; only where the reference tree
    exists)."""
    import glsl_pin
    path = glsl_pin.pt_lib_path(variant)
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    vp, u32 = C.c_void_p, C.c_uint32
    L.gpt_render_paths.argtypes = [vp, vp, vp, u32, u32, vp, u32, u32, vp, u32, vp]
    L.gpt_anyhit.argtypes = [vp, vp, vp, vp, u32, vp]
    return L


def shader_paths(glsl_lib_, scene: "OracleScene", view, settings: dict, sample_base: int, spp: int,
                 pixels=None) -> np.ndarray:
    """Per-path radiance [spp, npix, 3] from the reference's shaders, traced
    through the oracle's BVH; the layout of OracleScene.render_paths."""
    st = np.zeros(1, SETTINGS_DTYPE)
    for k in SETTINGS_DTYPE.names:
        st[k] = settings.get(k, 0)
    pix = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
    npix = view.width * view.height if pix is None else pix.size
    out = np.zeros((spp, npix, 3), np.float32)
    glsl_lib_.gpt_render_paths(scene.h, _p(view.inv_view), _p(view.inv_proj), view.width, view.height, _p(st),
                               sample_base, spp, _p(pix), npix, _p(out))
    return out


def shader_anyhit(glsl_pt_lib_, scene: "OracleScene", inst, prim, uv) -> np.ndarray:
    """The reference's any-hit shader (pt_anyhit.rahit, compiled as C++) on
    candidate hits: 1 accepted, 0 ignored."""
    inst = np.ascontiguousarray(inst, np.uint32)
    prim = np.ascontiguousarray(prim, np.uint32)
    uv = np.ascontiguousarray(uv, np.float32)
    out = np.zeros(inst.size, np.uint32)
    glsl_pt_lib_.gpt_anyhit(scene.h, _p(inst), _p(prim), _p(uv), inst.size, _p(out))
    return out


def glsl_eval(lib_, prefix: str, fn: int, x: np.ndarray, n_out: int, env=None) -> np.ndarray:
    """Runs helper (env=None) or env function ``fn`` of the oracle
    (prefix "orc_glsl_") or of the compiled reference GLSL ("gref_") on the
    records x; env = (marg, cond, w, h)."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((x.shape[0], n_out), np.float32)
    if env is None:
        st = getattr(lib_, prefix + "helper")(fn, _p(x), x.shape[0], _p(out))
    else:
        m, c, w, h = env
        m = np.ascontiguousarray(m, np.float32)
        c = np.ascontiguousarray(c, np.float32)
        st = getattr(lib_, prefix + "env")(fn, _p(m), _p(c), w, h, _p(x), x.shape[0], _p(out))
    assert st == 0, f"{prefix} fn {fn}: status {st}"
    return out


def env_cdf(env: np.ndarray):
    h, w = env.shape[:2]
    e = np.ascontiguousarray(env, np.float32)
    marg = np.zeros(h, np.float32)
    cond = np.zeros(w * h, np.float32)
    integ = np.zeros(1, np.float32)
    lib().orc_env_cdf_build(_p(e), w, h, _p(marg), _p(cond), _p(integ))
    return marg, cond, float(integ[0])


SETTINGS_DTYPE = np.dtype([("max_bounces", "<u4"), ("sampler", "<u4"), ("flags", "<u4"),
                           ("clamp_lum", "<f4"), ("aniso", "<f4"), ("aniso_rot", "<f4")])


class OracleScene:
    """Host oracle scene built from a :class:`ohao_engine_gb300.scenes.SceneData`."""

    def __init__(self, sd, flatten_limit: int = 1 << 25, force_mode: int = 0, env_cdf_arrays=None):
        L = lib()
        self.sd = sd
        self.h = L.orc_scene_create()
        self._keep = []
        pos = np.ascontiguousarray(sd.pos, np.float32)
        nrm = np.ascontiguousarray(sd.normals, np.float32)
        uv = np.ascontiguousarray(sd.uvs, np.float32)
        idx = np.ascontiguousarray(sd.indices, np.uint32)
        mid = np.ascontiguousarray(sd.mat_ids, np.uint32)
        L.orc_scene_set_geometry(self.h, _p(pos), 12, pos.shape[0], _p(nrm), _p(uv), _p(idx), idx.size // 3, _p(mid))
        mats = np.ascontiguousarray(sd.materials, np.float32)
        L.orc_scene_set_materials(self.h, _p(mats), mats.shape[0])
        lights = np.ascontiguousarray(sd.lights, np.float32)
        L.orc_scene_set_lights(self.h, _p(lights), lights.shape[0])
        if sd.env is not None:
            env = np.ascontiguousarray(sd.env, np.float32)
            marg, cond, integ = env_cdf_arrays if env_cdf_arrays is not None else env_cdf(env)
            L.orc_scene_set_env(self.h, _p(env), env.shape[1], env.shape[0], _p(marg), _p(cond), integ,
                                sd.env_intensity)
        if sd.albedo_map is not None:
            self.set_albedo_map(sd.albedo_map)
        if getattr(sd, "textures", None):
            texels = np.ascontiguousarray(np.concatenate([np.asarray(t, np.uint8).reshape(-1) for t in sd.textures]))
            sizes = np.array([[t.shape[1], t.shape[0]] for t in sd.textures], np.uint32)
            self._keep.append(texels)
            L.orc_scene_set_textures(self.h, _p(texels), _p(sizes), len(sd.textures))
        for k, (fi, ic) in enumerate(sd.blas):
            L.orc_scene_add_blas(self.h, fi, ic)
            flags = getattr(sd, "blas_flags", None)
            if flags:
                L.orc_scene_set_blas_flags(self.h, k, int(flags[k]))
        inst = np.ascontiguousarray(sd.instances)
        L.orc_scene_set_instances(self.h, _p(inst), inst.size)
        L.orc_scene_build(self.h, flatten_limit, force_mode)

    def set_albedo_map(self, amap):
        amap = np.ascontiguousarray(amap, np.float32)
        lib().orc_scene_set_albedo_map(self.h, _p(amap), amap.shape[1], amap.shape[0])

    def __del__(self):
        try:
            lib().orc_scene_destroy(self.h)
        except Exception:
            pass

    @property
    def two_level(self) -> bool:
        return bool(lib().orc_scene_two_level(self.h))

    def bvh(self, which: int = -1):
        nn, npr, hh = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().orc_bvh_sizes(self.h, which, C.byref(nn), C.byref(npr), C.byref(hh))
        nodes = np.zeros(nn.value * 80, np.uint8)
        prim_bytes = 4 if (which < 0 and self.two_level) else 48
        prims = np.zeros(npr.value * prim_bytes, np.uint8)
        lib().orc_bvh_copy(self.h, which, _p(nodes), _p(prims))
        return nodes, prims, hh.value

    def trace(self, rays: np.ndarray, mode: int = 0, stats: bool = False, nthreads: int = 0, alpha: bool = False):
        """mode 0 closest hit, 1 any hit, 2 brute-force closest hit; alpha:
        non-opaque rays (the any-hit alpha test)."""
        mode = mode | (4 if alpha else 0)
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        hits = np.zeros((n, 5), np.uint32)
        st = np.zeros((n, 2), np.uint32) if stats else None
        lib().orc_trace(self.h, _p(rays), n, _p(hits), mode, _p(st), nthreads)
        return (hits, st) if stats else hits

    def alpha_accept(self, inst, prim, uv) -> np.ndarray:
        """The oracle's any-hit alpha test on candidate hits (uint32 0/1)."""
        inst = np.ascontiguousarray(inst, np.uint32)
        prim = np.ascontiguousarray(prim, np.uint32)
        uv = np.ascontiguousarray(uv, np.float32)
        out = np.zeros(inst.size, np.uint32)
        lib().orc_alpha_accept(self.h, _p(inst), _p(prim), _p(uv), inst.size, _p(out))
        return out

    def render_paths(self, view, settings: dict, sample_base: int, spp: int, pixels=None, fp64=False,
                     nthreads: int = 0, stats: bool = False):
        st = np.zeros(1, SETTINGS_DTYPE)
        for k in SETTINGS_DTYPE.names:
            st[k] = settings.get(k, 0)
        pix = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        npix = view.width * view.height if pix is None else pix.size
        out = np.zeros((spp, npix, 3), np.float64 if fp64 else np.float32)
        s = np.zeros(3, np.uint64) if stats else None
        lib().orc_render_paths(self.h, _p(view.inv_view), _p(view.inv_proj), view.width, view.height, _p(st),
                               sample_base, spp, _p(pix), npix, _p(out), int(fp64), nthreads, _p(s))
        return (out, s) if stats else out

    def emitter_table(self):
        """Emitter-MIS table: (entries [n, 12] float32: p0, pdf per area,
        p1 - p0, instance bits, p2 - p0, prim bits; CDF [n])."""
        L = lib()
        n = L.orc_emitter_table(self.h, None, None)
        tri = np.zeros((n, 12), np.float32)
        cdf = np.zeros(n, np.float32)
        if n:
            L.orc_emitter_table(self.h, _p(tri), _p(cdf))
        return tri, cdf

    def light_samples(self, flags: int, P, N, n: int, seed: int = 0):
        """n light-NEE draws at P (normal N): [n, 15] float32 = L, Le,
        weight, choices, mis_pdf, valid, the emissive-table pdf at the
        closest hit along L from P, the weighted sphere / area light radiance
        along it (BSDF pdf 1), that hit's distance (-1: none)."""
        out = np.zeros((n, 15), np.float32)
        P = np.ascontiguousarray(P, np.float32)
        N = np.ascontiguousarray(N, np.float32)
        lib().orc_light_samples(self.h, flags, _p(P), _p(N), n, seed, _p(out))
        return out

    def detached_paths(self, view, settings: dict, sample_base: int, spp: int, pixels=None, materials=None,
                       albedo_map=None, nthreads: int = 0):
        """FP64 radiance of the detached-sampling estimator: sampling with the
        scene's own parameters, values with ``materials`` (M,12) and
        ``albedo_map`` (h,w,3); both default to the scene's. [spp, npix, 3]."""
        st = np.zeros(1, SETTINGS_DTYPE)
        for k in SETTINGS_DTYPE.names:
            st[k] = settings.get(k, 0)
        pix = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        npix = view.width * view.height if pix is None else pix.size
        mats = np.ascontiguousarray(self.sd.materials if materials is None else materials, np.float32)
        amap = self.sd.albedo_map if albedo_map is None else albedo_map
        amap = None if amap is None else np.ascontiguousarray(amap, np.float32)
        out = np.zeros((spp, npix, 3), np.float64)
        lib().orc_detached_paths(self.h, _p(view.inv_view), _p(view.inv_proj), view.width, view.height, _p(st),
                                 sample_base, spp, _p(pix), npix, _p(mats), _p(amap), _p(out), nthreads)
        return out

    def detached_grad(self, view, settings: dict, sample_base: int, spp: int, dLdI, rough_ids=(), map_ids=(),
                      with_score: bool = True, nthreads: int = 0):
        """Analytic FP64 gradient (forward-mode duals) of sum_p dLdI_p . I_p,
        I_p the mean of the pixel's detached paths, w.r.t. the roughness of
        materials ``rough_ids`` then the map entries ``map_ids`` (texel*3+c);
        at most 40 parameters. with_score adds the sampling-score terms (the
        device adjoint's full estimator); without, it is the derivative of
        :meth:`detached_paths`."""
        st = np.zeros(1, SETTINGS_DTYPE)
        for k in SETTINGS_DTYPE.names:
            st[k] = settings.get(k, 0)
        g = np.ascontiguousarray(dLdI, np.float64).reshape(-1, 3)
        assert g.shape[0] == view.width * view.height
        r = np.ascontiguousarray(rough_ids, np.int32)
        m = np.ascontiguousarray(map_ids, np.int32)
        out = np.zeros(r.size + m.size, np.float64)
        rc = lib().orc_detached_grad(self.h, _p(view.inv_view), _p(view.inv_proj), view.width, view.height, _p(st),
                                     sample_base, spp, _p(g), _p(r), r.size, _p(m), m.size, int(with_score), _p(out),
                                     nthreads)
        if rc != 0:
            raise ValueError("detached_grad: too many parameters")
        return out


def pow_def(x: np.ndarray, y: float) -> np.ndarray:
    """The pow(x, y) definition that the oracle and the kernels share."""
    a = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(a)
    lib().orc_pow_def(_p(a), a.size, float(y), _p(out))
    return out


def display_rgba8(rgba: np.ndarray) -> np.ndarray:
    """RGBA8 display image of RGBA32F texels (n, 4): the reference's
    pow(ACES(x * 0.5), 1/2.2) to UNORM8, alpha 255."""
    a = np.ascontiguousarray(rgba, np.float32).reshape(-1, 4)
    out = np.zeros((a.shape[0], 4), np.uint8)
    lib().orc_display_rgba8(_p(a), a.shape[0], _p(out))
    return out


def accumulate(paths: np.ndarray, accum: np.ndarray | None = None, history: int = 0):
    spp, npix, _ = paths.shape
    if accum is None:
        accum = np.zeros((npix, 4), np.float32)
    p = np.ascontiguousarray(paths, np.float32)
    lib().orc_accumulate(_p(p), npix, spp, _p(accum), history)
    return accum
