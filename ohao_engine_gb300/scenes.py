"""Seeded synthetic scenes for the path-tracing workloads.

Each builder returns a :class:`SceneData` holding arrays in the layout the C
ABI takes (the layout OHAO's RT scene packer uploads, ``rt_build.cpp:27-310``):
global float3 positions, float4 normals, float2 UVs, global uint32 indices,
per-triangle material ids, 3 x vec4 material records (``layout_meta.hpp:20-58``),
80-byte lights (``gpu_light.hpp:10-16``), an RGBA32F environment, BLAS index
ranges and 64-byte instance records.

Workloads (all seeds fixed):

* ``cornell``     -- Cornell box, 36 triangles, one area light, 256x256.
* ``cornell_example`` -- the reference example's Cornell box (five walls,
  two primitive spheres, twelve sphere lights) at 1920x1080, the scene of
  its golden image; a parity case, not a benchmark workload.
* ``sphere_1m``   -- geodesic sphere of frequency 224 (1,003,520 triangles)
  displaced by 5% value noise plus a 2-triangle ground plane, per-triangle
  GGX materials, 1024x512 sky + sun environment, 1920x1080.
* ``instanced``   -- 10,000 instances of 5 displaced geodesic spheres
  (2,000 / 9,680 / 50,000 / 100,820 / 200,000 triangles) and 64 views with
  log-uniform sides in [256, 1024].
* ``studio``      -- 200,000-triangle displaced sphere on a plane, 64x64 tile
  albedo map (texture slot 0) and 4 roughness regions; 10 views of 512x512.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NO_TEX = 0xFFFFFFFF
INSTANCE_DTYPE = np.dtype([("blas", "<u4"), ("xform", "<f4", (12,)), ("custom_index", "<u4"),
                           ("mask", "<u4"), ("sbt_offset", "<u4")])
assert INSTANCE_DTYPE.itemsize == 64


@dataclass
class View:
    inv_view: np.ndarray   # float32[16], column-major
    inv_proj: np.ndarray   # float32[16], column-major
    width: int
    height: int


@dataclass
class SceneData:
    name: str
    pos: np.ndarray          # (V,3) f32
    normals: np.ndarray      # (V,4) f32
    uvs: np.ndarray          # (V,2) f32
    indices: np.ndarray      # (3T,) u32
    mat_ids: np.ndarray      # (T,) u32
    materials: np.ndarray    # (M,12) f32
    lights: np.ndarray       # (L,20) f32
    env: np.ndarray | None   # (H,W,4) f32
    env_intensity: float
    blas: list               # [(first_index, index_count)]
    instances: np.ndarray    # INSTANCE_DTYPE
    views: list = field(default_factory=list)
    albedo_map: np.ndarray | None = None   # (h,w,3) f32
    spp: int = 1
    max_bounces: int = 4
    textures: list | None = None           # bindless RGBA8 textures, each (h,w,4) u8
    blas_flags: list | None = None         # per BLAS: OHAO_BLAS_FLAG_* (1 = non-opaque, alpha-tested)

    @property
    def ntris(self) -> int:
        return int(self.indices.size // 3)


# ---------------------------------------------------------------------------
# camera
# ---------------------------------------------------------------------------
def look_at_view(eye, target, up=(0.0, 1.0, 0.0), fov_y_deg=40.0, width=256, height=256) -> View:
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    up = np.asarray(up, np.float64)
    if abs(np.dot(f, up)) > 0.999:
        up = np.array([0.0, 0.0, 1.0])
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    inv_view = np.eye(4)
    inv_view[:3, 0] = r
    inv_view[:3, 1] = u
    inv_view[:3, 2] = -f
    inv_view[:3, 3] = eye
    t = math.tan(math.radians(fov_y_deg) * 0.5)
    aspect = width / height
    near, far = 0.01, 1000.0
    proj = np.zeros((4, 4))
    proj[0, 0] = 1.0 / (aspect * t)
    proj[1, 1] = -1.0 / t          # Vulkan y flip
    proj[2, 2] = far / (near - far)
    proj[2, 3] = far * near / (near - far)
    proj[3, 2] = -1.0
    inv_proj = np.linalg.inv(proj)
    # column-major flatten (glm memory layout)
    return View(inv_view.T.reshape(-1).astype(np.float32), inv_proj.T.reshape(-1).astype(np.float32),
                int(width), int(height))


def identity_instance(n=1):
    inst = np.zeros(n, INSTANCE_DTYPE)
    inst["xform"][:] = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    inst["mask"] = 0xFF
    return inst


def material(albedo, rough=1.0, metal=0.0, emissive=(0.0, 0.0, 0.0), diffuse_tex=NO_TEX):
    m = np.zeros(12, np.float32)
    m[0:3] = albedo
    m[3:4] = np.array([diffuse_tex], np.uint32).view(np.float32)
    m[4] = rough
    m[5] = metal
    m[6:8] = np.array([NO_TEX, NO_TEX], np.uint32).view(np.float32)
    m[8:9] = np.array([NO_TEX], np.uint32).view(np.float32)
    m[9:12] = emissive
    return m


# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------
_ICO_V = None


def _icosahedron():
    p = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p],
                  [0, -1, -p], [0, 1, -p], [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def geodesic_sphere(freq: int):
    """Class-I geodesic sphere: each icosahedron face split into freq^2 triangles."""
    v, f = _icosahedron()
    n = int(freq)
    ii, jj = [], []
    for i in range(n + 1):
        for j in range(n + 1 - i):
            ii.append(i)
            jj.append(j)
    ii = np.array(ii)
    jj = np.array(jj)
    lut = -np.ones((n + 1, n + 1), np.int64)
    lut[ii, jj] = np.arange(ii.size)
    tris = []
    for i in range(n):
        for j in range(n - i):
            tris.append((lut[i, j], lut[i + 1, j], lut[i, j + 1]))
            if j < n - i - 1:
                tris.append((lut[i + 1, j], lut[i + 1, j + 1], lut[i, j + 1]))
    tris = np.array(tris, np.int64)
    npf = ii.size
    A, B, C = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    wa = (n - ii - jj) / n
    wb = ii / n
    wc = jj / n
    pts = (A[:, None, :] * wa[None, :, None] + B[:, None, :] * wb[None, :, None] + C[:, None, :] * wc[None, :, None])
    pts = pts.reshape(-1, 3)
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    idx = (tris[None, :, :] + (np.arange(20) * npf)[:, None, None]).reshape(-1, 3)
    key = np.round(pts * 1e6).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    verts = pts[first]
    idx = inv.reshape(-1)[idx]
    return verts, idx


def value_noise3(p: np.ndarray, seed: int, freq: float = 4.0) -> np.ndarray:
    """Seeded 3-D value noise in [0,1]: lattice values, smoothstep trilinear."""
    rng = np.random.default_rng(seed)
    g = 64
    lat = rng.random((g, g, g))
    q = p * freq + 17.0
    i0 = np.floor(q).astype(np.int64)
    t = q - i0
    t = t * t * (3.0 - 2.0 * t)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (t[:, 0] if dx else 1 - t[:, 0]) * (t[:, 1] if dy else 1 - t[:, 1]) * (t[:, 2] if dz else 1 - t[:, 2])
                out += w * lat[(i0[:, 0] + dx) % g, (i0[:, 1] + dy) % g, (i0[:, 2] + dz) % g]
    return out


def vertex_normals(verts: np.ndarray, idx: np.ndarray) -> np.ndarray:
    a, b, c = verts[idx[:, 0]], verts[idx[:, 1]], verts[idx[:, 2]]
    fn = np.cross(b - a, c - a)
    vn = np.zeros_like(verts)
    for k in range(3):
        for comp in range(3):
            vn[:, comp] += np.bincount(idx[:, k], weights=fn[:, comp], minlength=verts.shape[0])
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-20)
    return vn


def displaced_sphere(freq: int, seed: int, amp: float = 0.05, radius: float = 1.0, center=(0, 0, 0)):
    verts, idx = geodesic_sphere(freq)
    nz = value_noise3(verts, seed)
    r = radius * (1.0 + amp * (2.0 * nz - 1.0))
    pos = verts * r[:, None] + np.asarray(center, np.float64)
    nrm = vertex_normals(pos, idx)
    u = np.arctan2(verts[:, 2], verts[:, 0]) / (2 * np.pi) + 0.5
    v = np.arccos(np.clip(verts[:, 1], -1, 1)) / np.pi
    uv = np.stack([u, v], 1)
    return pos, nrm, uv, idx


class _Builder:
    def __init__(self):
        self.pos, self.nrm, self.uv, self.idx, self.mid = [], [], [], [], []
        self.nv = 0
        self.ntri = 0

    def add(self, pos, nrm, uv, idx, mat_ids):
        first_index = self.ntri * 3
        self.pos.append(np.asarray(pos, np.float32))
        n4 = np.zeros((len(pos), 4), np.float32)
        n4[:, :3] = nrm
        self.nrm.append(n4)
        self.uv.append(np.asarray(uv, np.float32))
        self.idx.append((np.asarray(idx, np.int64) + self.nv).astype(np.uint32).reshape(-1))
        self.mid.append(np.broadcast_to(np.asarray(mat_ids, np.uint32), (len(idx),)).astype(np.uint32))
        self.nv += len(pos)
        self.ntri += len(idx)
        return first_index, len(idx) * 3

    def quad(self, a, b, c, d, normal, mat):
        pos = np.array([a, b, c, d], np.float64)
        nrm = np.tile(np.asarray(normal, np.float64), (4, 1))
        uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64)
        return self.add(pos, nrm, uv, [[0, 1, 2], [0, 2, 3]], mat)

    def arrays(self):
        return (np.concatenate(self.pos), np.concatenate(self.nrm), np.concatenate(self.uv),
                np.concatenate(self.idx), np.concatenate(self.mid))


def _box(b: _Builder, center, size, angle_deg, mat):
    cx, cy, cz = center
    sx, sy, sz = size
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)

    def P(x, y, z):
        x0, z0 = x * sx * 0.5, z * sz * 0.5
        return (cx + ca * x0 + sa * z0, cy + y * sy, cz - sa * x0 + ca * z0)

    def N(x, y, z):
        return (ca * x + sa * z, y, -sa * x + ca * z)

    b.quad(P(-1, 1, -1), P(-1, 1, 1), P(1, 1, 1), P(1, 1, -1), N(0, 1, 0), mat)      # top
    b.quad(P(-1, 0, -1), P(1, 0, -1), P(1, 0, 1), P(-1, 0, 1), N(0, -1, 0), mat)     # bottom
    b.quad(P(-1, 0, 1), P(1, 0, 1), P(1, 1, 1), P(-1, 1, 1), N(0, 0, 1), mat)        # front
    b.quad(P(1, 0, -1), P(-1, 0, -1), P(-1, 1, -1), P(1, 1, -1), N(0, 0, -1), mat)   # back
    b.quad(P(-1, 0, -1), P(-1, 0, 1), P(-1, 1, 1), P(-1, 1, -1), N(-1, 0, 0), mat)   # left
    b.quad(P(1, 0, 1), P(1, 0, -1), P(1, 1, -1), P(1, 1, 1), N(1, 0, 0), mat)        # right


def area_light(corner, e1, e2, intensity, color=(1.0, 1.0, 1.0)):
    """type-3 GPULight whose Le = color*intensity (radius 1/sqrt(4*pi) makes
    the reference's 4*pi*r^2 normalisation equal to 1)."""
    L = np.zeros(20, np.float32)
    e1 = np.asarray(e1, np.float64)
    e2 = np.asarray(e2, np.float64)
    L[0:3] = corner
    L[3] = 3.0
    L[4:7] = color
    L[7] = intensity
    L[8:11] = (0.0, -1.0, 0.0)
    L[11] = 1.0 / math.sqrt(4.0 * math.pi)
    L[12:15] = e1
    L[16:19] = e2
    L[19] = float(np.linalg.norm(np.cross(e1, e2)))
    return L


def sky_env(width=1024, height=512, seed=1, sky=0.5, peak=5e4, radius_deg=0.5):
    """Constant sky plus a Gaussian sun; row 0 is +Y (the CDF convention)."""
    rng = np.random.default_rng(seed)
    az = rng.uniform(-math.pi, math.pi)
    el = rng.uniform(math.radians(20), math.radians(70))
    sun = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    y, x = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    u = (x + 0.5) / width
    v = (y + 0.5) / height
    phi = (u - 0.5) * 2 * math.pi
    theta = v * math.pi
    d = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], -1)
    ang = np.arccos(np.clip(d @ sun, -1, 1))
    s = peak * np.exp(-0.5 * (ang / math.radians(radius_deg)) ** 2)
    env = np.zeros((height, width, 4), np.float32)
    env[..., 0] = sky + s
    env[..., 1] = sky + s * 0.95
    env[..., 2] = sky + s * 0.85
    env[..., 3] = 1.0
    return env


def _ground(b: _Builder, y, half, mat):
    return b.quad((-half, y, -half), (-half, y, half), (half, y, half), (half, y, -half), (0, 1, 0), mat)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def cornell(width=256, height=256, spp=16) -> SceneData:
    b = _Builder()
    white, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    mats = [material(white), material(red), material(green), material(white),
            material((0.78, 0.78, 0.78), emissive=(15.0, 15.0, 15.0))]
    h = 0.5
    b.quad((-h, 0, -h), (h, 0, -h), (h, 1, -h), (-h, 1, -h), (0, 0, 1), 0)       # back
    b.quad((-h, 0, -h), (-h, 1, -h), (-h, 1, h), (-h, 0, h), (1, 0, 0), 1)       # left (red)
    b.quad((h, 0, -h), (h, 0, h), (h, 1, h), (h, 1, -h), (-1, 0, 0), 2)          # right (green)
    b.quad((-h, 0, -h), (-h, 0, h), (h, 0, h), (h, 0, -h), (0, 1, 0), 3)         # floor
    b.quad((-h, 1, -h), (h, 1, -h), (h, 1, h), (-h, 1, h), (0, -1, 0), 3)        # ceiling
    _box(b, (-0.17, 0.0, -0.12), (0.28, 0.6, 0.28), 15.0, 0)                     # tall box
    _box(b, (0.18, 0.0, 0.16), (0.28, 0.3, 0.28), -18.0, 0)                      # short box
    ly = 0.999
    b.quad((-0.12, ly, -0.1), (0.12, ly, -0.1), (0.12, ly, 0.1), (-0.12, ly, 0.1), (0, -1, 0), 4)  # light
    pos, nrm, uv, idx, mid = b.arrays()
    lights = area_light((-0.12, 0.998, -0.1), (0.24, 0, 0), (0, 0, 0.2), 15.0)[None, :]
    inst = identity_instance(1)
    view = look_at_view((0.0, 0.5, 1.94), (0.0, 0.5, 0.0), fov_y_deg=40.0, width=width, height=height)
    return SceneData("cornell", pos, nrm, uv, idx, mid, np.stack(mats), lights, None, 1.0,
                     [(0, idx.size)], inst, [view], spp=spp, max_bounces=4)


def _random_materials(rng, n):
    m = np.zeros((n, 12), np.float32)
    m[:, 0:3] = rng.uniform(0.1, 0.9, (n, 3))
    m[:, 3] = np.array([NO_TEX], np.uint32).view(np.float32)[0]
    m[:, 4] = rng.uniform(0.05, 1.0, n)
    m[:, 5] = (rng.random(n) < 0.5).astype(np.float32)
    m[:, 6:9] = np.array([NO_TEX] * 3, np.uint32).view(np.float32)
    return m


def sphere_1m(width=1920, height=1080, freq=224, seed=1, env_size=(1024, 512)) -> SceneData:
    rng = np.random.default_rng(seed)
    b = _Builder()
    pos, nrm, uv, idx = displaced_sphere(freq, seed)
    nt = idx.shape[0]
    mats = _random_materials(rng, nt + 1)
    mats[nt] = material((0.5, 0.5, 0.5), rough=0.8)
    b.add(pos, nrm, uv, idx, np.arange(nt, dtype=np.uint32))
    _ground(b, -1.05, 6.0, nt)
    P, N, U, I, M = b.arrays()
    env = sky_env(env_size[0], env_size[1], seed=seed)
    inst = identity_instance(1)
    view = look_at_view((0.0, 0.6, 3.2), (0.0, -0.1, 0.0), fov_y_deg=40.0, width=width, height=height)
    return SceneData("sphere_1m", P, N, U, I, M, mats, np.zeros((0, 20), np.float32), env, 1.0,
                     [(0, I.size)], inst, [view], spp=1, max_bounces=4)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def instanced(n_instances=10000, n_views=64, seed=1, freqs=(10, 22, 50, 71, 100), side_range=(256, 1024),
              spp=4) -> SceneData:
    rng = np.random.default_rng(seed)
    b = _Builder()
    blas = []
    mat_base = 0
    mats = []
    for k, f in enumerate(freqs):
        pos, nrm, uv, idx = displaced_sphere(f, seed + 7 * k)
        nt = idx.shape[0]
        mats.append(_random_materials(rng, nt))
        blas.append(b.add(pos, nrm, uv, idx, np.arange(nt, dtype=np.uint32) + mat_base))
        mat_base += nt
    P, N, U, I, M = b.arrays()
    inst = np.zeros(n_instances, INSTANCE_DTYPE)
    for i in range(n_instances):
        k = int(rng.integers(0, len(freqs)))
        R = _random_rotation(rng) * rng.uniform(0.5, 2.0)
        t = rng.uniform(-50, 50, 3)
        x = np.zeros((3, 4))
        x[:, :3] = R
        x[:, 3] = t
        inst[i]["blas"] = k
        inst[i]["xform"] = x.reshape(-1).astype(np.float32)
        inst[i]["custom_index"] = blas[k][0] // 3
        inst[i]["mask"] = 0xFF
    views = []
    lo, hi = math.log(side_range[0]), math.log(side_range[1])
    for _ in range(n_views):
        side = int(round(math.exp(rng.uniform(lo, hi))))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        eye = d * 75.0
        target = rng.uniform(-20, 20, 3)
        views.append(look_at_view(eye, target, fov_y_deg=45.0, width=side, height=side))
    env = sky_env(seed=seed)
    return SceneData("instanced", P, N, U, I, M, np.concatenate(mats), np.zeros((0, 20), np.float32), env, 1.0,
                     [(fi, ic) for fi, ic in blas], inst, views, spp=spp, max_bounces=4)


def studio(freq=100, seed=1, side=512, n_train=8, n_holdout=2, map_size=64, albedo_map=None,
           roughness=(0.3, 0.5, 0.7, 0.9)) -> SceneData:
    """Displaced sphere (4 roughness regions, texture slot 0) on a plane."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    pos, nrm, uv, idx = displaced_sphere(freq, seed)
    tri_uv = uv[idx].mean(axis=1)
    region = (tri_uv[:, 0] >= 0.5).astype(np.uint32) + 2 * (tri_uv[:, 1] >= 0.5).astype(np.uint32)
    b.add(pos, nrm, uv, idx, region)
    _ground(b, -1.05, 6.0, 4)
    P, N, U, I, M = b.arrays()
    mats = [material((1.0, 1.0, 1.0), rough=r, metal=0.0, diffuse_tex=0) for r in roughness]
    mats.append(material((0.6, 0.6, 0.6), rough=0.9))
    if albedo_map is None:
        albedo_map = rng.uniform(0.1, 0.9, (map_size, map_size, 3)).astype(np.float32)
    env = sky_env(256, 128, seed=seed, peak=500.0, radius_deg=3.0)
    views = []
    for k in range(n_train + n_holdout):
        a = 2 * math.pi * k / (n_train + n_holdout)
        eye = (3.0 * math.cos(a), 0.8 + 0.3 * math.sin(3 * a), 3.0 * math.sin(a))
        views.append(look_at_view(eye, (0, -0.1, 0), fov_y_deg=40.0, width=side, height=side))
    return SceneData("studio", P, N, U, I, M, np.stack(mats), np.zeros((0, 20), np.float32), env, 1.0,
                     [(0, I.size)], identity_instance(1), views, albedo_map=np.asarray(albedo_map, np.float32),
                     spp=16, max_bounces=3)


def material_tex(albedo, rough=1.0, metal=0.0, diffuse_tex=NO_TEX, normal_tex=NO_TEX, emissive_tex=NO_TEX,
                 rough_metal_tex=NO_TEX, emissive=(0.0, 0.0, 0.0)):
    """A 48-byte material record with every bindless texture slot
    (layout_meta.hpp:32-56): diffuse [3], normal [6], emissive [7],
    roughness-metal [8]."""
    m = material(albedo, rough=rough, metal=metal, emissive=emissive, diffuse_tex=diffuse_tex)
    m[6:7] = np.array([normal_tex], np.uint32).view(np.float32)
    m[7:8] = np.array([emissive_tex], np.uint32).view(np.float32)
    m[8:9] = np.array([rough_metal_tex], np.uint32).view(np.float32)
    return m


def _textures(rng, size=64):
    """Seeded RGBA8 textures: 0 checker albedo, 1 bump normal map, 2 ORM
    (R ao, G roughness, B metallic), 3 noise albedo, 4 emissive pattern, 5
    albedo with an alpha cut-out (alpha 0, 255 and a soft edge band)."""
    y, x = np.meshgrid(np.arange(size), np.arange(size), indexing="ij")
    u, v = (x + 0.5) / size, (y + 0.5) / size
    tex = []
    chk = ((x // 8 + y // 8) % 2).astype(np.float64)
    a = np.stack([0.2 + 0.7 * chk, 0.3 + 0.5 * (1 - chk), 0.6 * np.ones_like(chk), np.ones_like(chk)], -1)
    tex.append(a)
    h = 0.5 * np.sin(2 * math.pi * 3 * u) * np.cos(2 * math.pi * 2 * v)
    nx, ny = -np.gradient(h, axis=1) * 4, -np.gradient(h, axis=0) * 4
    n = np.stack([nx, ny, np.ones_like(nx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    tex.append(np.concatenate([n * 0.5 + 0.5, np.ones_like(nx)[..., None]], -1))
    tex.append(np.stack([0.8 + 0.2 * rng.random((size, size)), 0.2 + 0.8 * rng.random((size, size)),
                         (rng.random((size, size)) > 0.5).astype(np.float64), np.ones((size, size))], -1))
    tex.append(np.concatenate([rng.random((size, size, 3)), np.ones((size, size, 1))], -1))
    e = ((np.sin(2 * math.pi * 4 * u) > 0.3) & (np.cos(2 * math.pi * 4 * v) > 0.0)).astype(np.float64)
    tex.append(np.stack([e, 0.8 * e, 0.3 * e, np.ones_like(e)], -1))
    r = np.hypot(u - 0.5, v - 0.5)
    alpha = np.clip((0.42 - r) / 0.04, 0.0, 1.0) * ((x // 6 + y // 6) % 3 != 0)
    tex.append(np.stack([0.3 + 0.2 * u, 0.6 * np.ones_like(u), 0.2 + 0.3 * v, alpha], -1))
    return [np.clip(np.rint(t * 255.0), 0, 255).astype(np.uint8) for t in tex]


def textured(width=48, height=32, seed=3, freq=12) -> SceneData:
    """Bindless-texture scene: a tiled floor (checker albedo, normal map,
    ORM), a displaced sphere (noise albedo, ORM, metallic), an emissive
    texture panel, and a curtain of alpha cut-out leaves in a non-opaque
    BLAS, under a sky with a sun and one sphere light."""
    rng = np.random.default_rng(seed)
    texs = _textures(rng)
    b = _Builder()
    mats = [material_tex((1.0, 1.0, 1.0), rough=0.9, diffuse_tex=0, normal_tex=1, rough_metal_tex=2),
            material_tex((0.9, 0.9, 0.9), rough=0.7, metal=1.0, diffuse_tex=3, rough_metal_tex=2),
            material_tex((0.0, 0.0, 0.0), rough=1.0, emissive_tex=4),
            material_tex((1.0, 1.0, 1.0), rough=0.8, diffuse_tex=5, normal_tex=1)]
    half = 3.0
    pos = np.array([(-half, -1.0, -half), (-half, -1.0, half), (half, -1.0, half), (half, -1.0, -half)], np.float64)
    b.add(pos, np.tile([0.0, 1.0, 0.0], (4, 1)), np.array([[0, 0], [0, 3], [3, 3], [3, 0]], np.float64),
          [[0, 1, 2], [0, 2, 3]], 0)
    sp, sn, su, si = displaced_sphere(freq, seed, amp=0.05, radius=0.7, center=(0.3, -0.25, 0.0))
    b.add(sp, sn, su * 2.0, si, 1)
    b.quad((-1.6, -0.6, -1.2), (-1.6, -0.6, -0.4), (-1.6, 0.4, -0.4), (-1.6, 0.4, -1.2), (1, 0, 0), 2)
    opaque_count = b.ntri * 3
    for k in range(5):     # leaves: the non-opaque BLAS
        x0 = -1.2 + 0.55 * k
        z0 = 0.9 + 0.15 * math.sin(k)
        b.quad((x0, -0.9, z0), (x0 + 0.5, -0.9, z0 + 0.1), (x0 + 0.5, 0.2, z0 + 0.1), (x0, 0.2, z0),
               (-0.2, 0.0, 1.0), 3)
    P, N, U, I, M = b.arrays()
    env = sky_env(64, 32, seed=seed, peak=300.0, radius_deg=4.0)
    light = np.zeros(20, np.float32)
    light[0:4] = (1.2, 1.5, 1.5, 0.0)         # sphere light
    light[4:8] = (1.0, 0.9, 0.8, 6.0)
    light[11] = 0.15
    inst = identity_instance(2)
    inst[1]["blas"] = 1
    inst[1]["custom_index"] = opaque_count // 3
    view = look_at_view((0.6, 0.9, 3.6), (0.0, -0.4, 0.0), fov_y_deg=45.0, width=width, height=height)
    return SceneData("textured", P, N, U, I, M, np.stack(mats), light[None, :], env, 1.0,
                     [(0, opaque_count), (opaque_count, I.size - opaque_count)], inst, [view], spp=4, max_bounces=4,
                     textures=texs, blas_flags=[0, 1])


def emitters(width=256, height=160, lights=("area", "sphere"), env=False, floor_rough=0.9) -> SceneData:
    """Emitter-MIS scene: a floor, a metal box, a near-mirror panel, two
    emissive quads (small and bright overhead, large and dim on a wall) in
    BLAS 0; one emissive triangle in BLAS 1, instanced scaled and moved,
    and again masked out; the same triangle in BLAS 2, non-opaque. Optional
    area and sphere GPULights and an environment. The emitter-MIS workload
    (OHAO_PT_FLAG_EMITTER_MIS): small bright and large dim emitters, glossy
    and near-mirror surfaces."""
    b = _Builder()
    mats = [material((0.7, 0.7, 0.7), rough=floor_rough),
            material((0.6, 0.3, 0.2), rough=0.3, metal=1.0),
            material((0.8, 0.8, 0.8), emissive=(40.0, 30.0, 20.0)),
            material((0.5, 0.5, 0.5), emissive=(1.0, 1.5, 2.0)),
            material((0.2, 0.6, 0.3), rough=0.02),
            material((0.9, 0.9, 0.9), emissive=(5.0, 4.0, 6.0))]
    h = 3.0
    b.quad((-h, -1, -h), (-h, -1, h), (h, -1, h), (h, -1, -h), (0, 1, 0), 0)
    _box(b, (0.6, -1.0, -0.3), (0.6, 0.8, 0.6), 20.0, 1)
    b.quad((1.6, -1.0, 0.8), (1.6, -1.0, -0.8), (1.6, 0.4, -0.8), (1.6, 0.4, 0.8), (-1, 0, 0), 4)
    b.quad((-0.3, 1.2, 0.2), (0.3, 1.2, 0.2), (0.3, 1.2, -0.2), (-0.3, 1.2, -0.2), (0, -1, 0), 2)
    b.quad((-2.5, -1.0, -1.5), (-2.5, -1.0, 1.5), (-2.5, 1.0, 1.5), (-2.5, 1.0, -1.5), (1, 0, 0), 3)
    n0 = b.ntri * 3
    b.add(np.array([(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0)]), np.tile([0.0, -1.0, 0.0], (3, 1)),
          np.array([(0, 0), (1, 0), (0, 1)], np.float64), [[0, 1, 2]], 5)
    P, N, U, I, M = b.arrays()
    inst = identity_instance(4)
    x = np.zeros((3, 4), np.float32)
    x[:, :3] = np.diag([0.8, 1.0, 0.6])
    x[:, 3] = (-1.2, 0.9, 0.6)
    for k in (1, 2, 3):
        inst[k]["blas"] = 1 if k < 3 else 2
        inst[k]["custom_index"] = n0 // 3
        inst[k]["xform"] = x.reshape(-1)
    inst[2]["mask"] = 0
    inst[3]["xform"][3] = 1.5      # the non-opaque copy elsewhere
    ls = []
    if "area" in lights:
        ls.append(area_light((0.9, 1.1, 0.9), (0.0, 0.0, -0.3), (0.4, 0.0, 0.0), 12.0, (1.0, 0.9, 0.7)))
    if "sphere" in lights:
        L = np.zeros(20, np.float32)
        L[0:4] = (-0.8, 0.6, 1.2, 0.0)
        L[4:8] = (0.7, 0.8, 1.0, 8.0)
        L[11] = 0.2
        ls.append(L)
    lights_arr = np.stack(ls) if ls else np.zeros((0, 20), np.float32)
    envmap = sky_env(64, 32, seed=4, peak=200.0, radius_deg=4.0) if env else None
    view = look_at_view((0.2, 0.6, 4.0), (0.0, -0.2, 0.0), fov_y_deg=50.0, width=width, height=height)
    return SceneData("emitters", P, N, U, I, M, np.stack(mats), lights_arr, envmap, 1.0,
                            [(0, n0), (n0, 3), (n0, 3)], inst, [view], spp=4, max_bounces=4, blas_flags=[0, 0, 1])


WORKLOADS = {"cornell": cornell, "sphere_1m": sphere_1m, "instanced": instanced, "studio": studio}


def _f32(x):
    return np.float32(x)


def _glm_sphere_mesh(radius=0.5, sectors=32, stacks=16):
    """The primitive sphere of ``ComponentFactory::generateSphereMesh``
    (``scene/component/component_factory.cpp:347-395``): a UV sphere of
    radius 0.5, 32 sectors x 16 stacks, angles and products in float32,
    sin/cos of the float angle evaluated in double and rounded (the C
    library's double sin/cos), unit normals = the unscaled positions."""
    pi = _f32(math.pi)
    pos, nrm, uv = [], [], []
    for i in range(stacks + 1):
        phi = _f32(_f32(pi * _f32(i)) / _f32(stacks))
        sp, cp = _f32(math.sin(float(phi))), _f32(math.cos(float(phi)))
        for j in range(sectors + 1):
            theta = _f32(_f32(_f32(2.0) * pi * _f32(j)) / _f32(sectors))
            st, ct = _f32(math.sin(float(theta))), _f32(math.cos(float(theta)))
            x, y, z = _f32(ct * sp), cp, _f32(st * sp)
            r = _f32(radius)
            pos.append((x * r, y * r, z * r))
            nrm.append((x, y, z))
            uv.append((_f32(j) / _f32(sectors), _f32(i) / _f32(stacks)))
    idx = []
    for i in range(stacks):
        for j in range(sectors):
            first = i * (sectors + 1) + j
            second = first + sectors + 1
            idx.append((first, second, first + 1))
            idx.append((second, second + 1, first + 1))
    return (np.array(pos, np.float32), np.array(nrm, np.float32), np.array(uv, np.float32), idx)


def _glm_look_at_inverse(eye, yaw_deg, pitch_deg):
    """Inverse view matrix (column-major) of OHAO's camera
    (``render/camera/camera.cpp:25-42``: front from yaw/pitch, right/up by
    cross products, ``glm::lookAt``), built in float32 and inverted in double."""
    rad = _f32(0.017453292519943295)
    yaw, pitch = _f32(_f32(yaw_deg) * rad), _f32(_f32(pitch_deg) * rad)
    cy, sy = _f32(math.cos(float(yaw))), _f32(math.sin(float(yaw)))
    cpi, spi = _f32(math.cos(float(pitch))), _f32(math.sin(float(pitch)))
    front = np.array([cy * cpi, spi, sy * cpi], np.float32)

    def normalize(v):
        return (v * _f32(1.0 / math.sqrt(float(np.dot(v, v))))).astype(np.float32)

    front = normalize(front)
    right = normalize(np.cross(front, np.array([0, 1, 0], np.float32)).astype(np.float32))
    up = normalize(np.cross(right, front).astype(np.float32))
    eye = np.asarray(eye, np.float32)
    f = normalize((eye + front).astype(np.float32) - eye)
    s = normalize(np.cross(f, up).astype(np.float32))
    u = np.cross(s, f).astype(np.float32)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[0, 3], view[1, 3], view[2, 3] = -np.dot(s, eye), -np.dot(u, eye), np.dot(f, eye)
    return np.linalg.inv(view.astype(np.float32).astype(np.float64)).T.reshape(-1).astype(np.float32)


# light colours and positions of the reference example's 12 sphere lights
_EXAMPLE_LIGHT_COLORS = [(1.0, 0.3, 0.2), (0.2, 1.0, 0.3), (0.3, 0.4, 1.0), (1.0, 0.9, 0.3), (1.0, 0.5, 0.0),
                         (0.8, 0.2, 1.0), (0.0, 1.0, 1.0), (1.0, 0.0, 0.5), (1.0, 1.0, 1.0), (0.5, 1.0, 0.5),
                         (1.0, 0.7, 0.5), (0.5, 0.7, 1.0)]
_EXAMPLE_LIGHT_POS = [(-3, 4, -3), (0, 4, -3), (3, 4, -3), (-3, 4, 0), (0, 4, 0), (3, 4, 0),
                      (-3, 4, 3), (0, 4, 3), (3, 4, 3), (-4, 0, 0), (4, 0, 0), (0, 0, -4)]
# Upload order of the 12 lights. The engine walks its actor table, an
# std::unordered_map keyed by sequential actor ids (the root actor is 1, the
# five walls 2-6, the two spheres 7-8, the lights 9-20); libstdc++ iterates
# those 20 keys as 20, 19, ..., 14, 1, 2, ..., 13, so the light records go
# out as lights 11..5 followed by lights 0..4.
EXAMPLE_LIGHT_ORDER = (11, 10, 9, 8, 7, 6, 5, 0, 1, 2, 3, 4)


def cornell_example(width=1920, height=1080, spp=16, light_order=EXAMPLE_LIGHT_ORDER) -> SceneData:
    """The reference's ``examples/cornell_box.cpp`` scene as its renderer
    uploads it, the scene of its golden image ``tests/golden/cornell_box.png``:
    five 10x10 walls (white 0.73, red, green; roughness 0.95), a metal sphere
    (radius 1 at (-2, -3, 0), roughness 0.05) and a dielectric one (radius 0.9
    at (2.5, -3.2, 1.5), roughness 0.02), both the 32x16 primitive UV sphere
    as instances of their own BLAS; twelve coloured sphere lights (intensity
    5, radius 0.3); no environment (misses are black); camera at (0, 0, 13),
    yaw -90, 38 degree vertical field of view. Actors are packed in the
    engine's order (walls Back, Left, Right, Floor, Ceiling, then the two
    spheres), one BLAS and one material per actor, instance custom index =
    the actor's first global triangle (``gpu/vulkan/rt_build.cpp:825-900``,
    ``scene_upload.cpp:20-80``)."""
    S = 5.0
    white, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    LBB, RBB, LTB, RTB = (-S, -S, -S), (S, -S, -S), (-S, S, -S), (S, S, -S)
    LBF, RBF, LTF, RTF = (-S, -S, S), (S, -S, S), (-S, S, S), (S, S, S)
    walls = [((LBB, RBB, RTB, LTB), (0, 0, 1), white), ((LBB, LTB, LTF, LBF), (1, 0, 0), red),
             ((RBB, RBF, RTF, RTB), (-1, 0, 0), green), ((LBB, LBF, RBF, RBB), (0, 1, 0), white),
             ((LTB, RTB, RTF, LTF), (0, -1, 0), white)]
    b = _Builder()
    blas, mats, xforms = [], [], []
    ident = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    for k, (quad, n, col) in enumerate(walls):
        pos = np.array(quad, np.float32)
        uv = np.zeros((4, 2), np.float32)
        blas.append(b.add(pos, np.tile(np.array(n, np.float32), (4, 1)), uv, [[0, 1, 2], [0, 2, 3]], k))
        mats.append(material(col, rough=0.95))
        xforms.append(ident)
    spos, snrm, suv, sidx = _glm_sphere_mesh()
    spheres = [((-2.0, -S + 2.0, 0.0), 2.0, (0.95, 0.93, 0.88), 0.05, 1.0),
               ((2.5, -S + 1.8, 1.5), 1.8, (0.9, 0.95, 1.0), 0.02, 0.0)]
    for k, (c, scale, col, rough, metal) in enumerate(spheres):
        blas.append(b.add(spos, snrm, suv, sidx, len(walls) + k))
        mats.append(material(col, rough=rough, metal=metal))
        c = np.array(c, np.float32)
        sc = _f32(scale)
        xforms.append(np.array([sc, 0, 0, c[0], 0, sc, 0, c[1], 0, 0, sc, c[2]], np.float32))
    pos, nrm, uv, idx, mid = b.arrays()
    inst = np.zeros(len(blas), INSTANCE_DTYPE)
    tri0 = 0
    for k, (first, count) in enumerate(blas):
        inst[k]["blas"] = k
        inst[k]["xform"] = xforms[k]
        inst[k]["custom_index"] = tri0
        inst[k]["mask"] = 0xFF
        tri0 += count // 3
    lights = []
    for i in light_order:
        L = np.zeros(20, np.float32)
        L[0:3] = _EXAMPLE_LIGHT_POS[i]
        L[3] = 0.0
        L[4:7] = _EXAMPLE_LIGHT_COLORS[i]
        L[7] = 5.0
        L[8:11] = (-0.3, -1.0, -0.2) / np.float32(np.linalg.norm((-0.3, -1.0, -0.2)))
        L[11] = 0.3
        lights.append(L)
    inv_view = _glm_look_at_inverse((0.0, 0.0, 13.0), -90.0, 0.0)
    t = np.float32(math.tan(float(_f32(_f32(38.0) * _f32(0.017453292519943295)) / _f32(2.0))))
    # inverse of glm::perspective(fov, aspect, 0.1, 1000) (OpenGL depth range),
    # column-major; the raygen reads only |[1][1]| = tan(fov / 2)
    inv_proj = np.zeros(16, np.float32)
    aspect = _f32(_f32(width) / _f32(height))
    inv_proj[0] = _f32(1.0) / _f32(_f32(1.0) / _f32(aspect * t))
    inv_proj[5] = _f32(1.0) / _f32(_f32(1.0) / t)
    inv_proj[11], inv_proj[14], inv_proj[15] = -4.9995, -1.0, 5.0005
    view = View(inv_view, inv_proj, int(width), int(height))
    return SceneData("cornell_example", pos, nrm, uv, idx, mid, np.stack(mats), np.stack(lights), None, 1.0,
                     blas, inst, [view], spp=spp, max_bounces=4)
