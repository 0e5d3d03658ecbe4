"""Host-oracle self checks: traversal vs brute force, BVH invariants, math,
FP32 vs FP64 integrator agreement. CPU only."""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes


def random_rays(rng, n, lo, hi, tmin=0.001, tmax=10000.0):
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def decode_nodes(nodes):
    rec = np.dtype([("origin", "<f4", 3), ("exps", "i1", 3), ("imask", "u1"), ("child_base", "<u4"),
                    ("tri_base", "<u4"), ("meta", "u1", 8), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
    assert rec.itemsize == 80
    return nodes.view(rec)


def check_bvh_invariants(nodes_u8, tris_u8, nprims):
    n = decode_nodes(nodes_u8)
    tri = tris_u8.view(np.float32).reshape(-1, 12)
    seen = np.zeros(nprims, np.int32)
    for k in range(len(n)):
        nd = n[k]
        scale = np.ldexp(1.0, nd["exps"].astype(np.int64))
        for i in range(8):
            m = int(nd["meta"][i])
            if m == 0:
                continue
            lo = nd["origin"].astype(np.float64) + nd["qlo"][:, i] * scale
            hi = nd["origin"].astype(np.float64) + nd["qhi"][:, i] * scale
            if nd["imask"] >> i & 1:
                assert m & 0x80
                c = n[int(nd["child_base"]) + (m & 7)]
                # child's quantized grid origin lies inside the parent's box for that slot
                assert np.all(c["origin"] >= lo - 1e-6 * np.abs(lo) - 1e-30)
            else:
                cnt, off = m >> 5, m & 31
                assert 1 <= cnt <= 3
                for q in range(cnt):
                    j = int(nd["tri_base"]) + off + q
                    seen[j] += 1
                    v = tri[j].reshape(3, 4)[:, :3].astype(np.float64)
                    assert np.all(v >= lo[None, :]) and np.all(v <= hi[None, :]), "quantized leaf box not conservative"
    assert np.all(seen == 1), "every primitive in exactly one leaf"


def test_oracle_math_accuracy(oracle):
    L = oracle.lib()
    x = np.linspace(-7.0, 7.0, 20001).astype(np.float32)
    for op, ref in ((0, np.sin), (1, np.cos)):
        out = np.zeros_like(x)
        L.orc_math(op, x.ctypes.data, x.size, out.ctypes.data)
        assert np.max(np.abs(out - ref(x.astype(np.float64)))) < 2e-7
    yx = np.random.default_rng(0).normal(size=(5000, 2)).astype(np.float32)
    out = np.zeros(5000, np.float32)
    L.orc_math(2, yx.ctypes.data, 5000, out.ctypes.data)
    assert np.max(np.abs(out - np.arctan2(yx[:, 0], yx[:, 1]).astype(np.float64))) < 4e-7
    u = np.linspace(-1, 1, 4001).astype(np.float32)
    for op, ref in ((3, np.arcsin), (4, np.arccos)):
        o2 = np.zeros_like(u)
        L.orc_math(op, u.ctypes.data, u.size, o2.ctypes.data)
        assert np.max(np.abs(o2 - ref(u.astype(np.float64)))) < 2e-6


def test_flat_bvh_matches_brute_force(oracle):
    sd = scenes.cornell(32, 32, 1)
    sc = oracle.OracleScene(sd)
    rng = np.random.default_rng(1)
    rays = random_rays(rng, 20000, -0.45, 0.45)
    rays[:, 1] = rng.uniform(0.02, 0.98, rays.shape[0])
    assert np.array_equal(sc.trace(rays, 0), sc.trace(rays, 2))
    nodes, tris, _ = sc.bvh()
    check_bvh_invariants(nodes, tris, sd.ntris)


def test_displaced_sphere_bvh_matches_brute_force(oracle):
    pos, nrm, uv, idx = scenes.displaced_sphere(12, seed=3)
    b = scenes._Builder()
    b.add(pos, nrm, uv, idx, 0)
    P, N, U, I, M = b.arrays()
    sd = scenes.SceneData("s", P, N, U, I, M, np.stack([scenes.material((0.5, 0.5, 0.5))]),
                          np.zeros((0, 20), np.float32), None, 1.0, [(0, I.size)], scenes.identity_instance(1), [])
    sc = oracle.OracleScene(sd)
    rng = np.random.default_rng(2)
    rays = random_rays(rng, 4000, -1.5, 1.5)
    h_bvh, st = sc.trace(rays, 0, stats=True)
    h_bf = sc.trace(rays, 2)
    assert np.array_equal(h_bvh, h_bf)
    assert (h_bvh[:, 4] != 0xFFFFFFFF).mean() > 0.15
    nodes, tris, height = sc.bvh()
    check_bvh_invariants(nodes, tris, sd.ntris)
    # any-hit agrees with closest-hit existence
    occ = sc.trace(rays, 1)
    assert np.array_equal(occ[:, 0] == 1, h_bf[:, 4] != 0xFFFFFFFF)


def test_two_level_matches_flat(oracle):
    sd = scenes.instanced(n_instances=60, n_views=2, freqs=(3, 5), side_range=(16, 32), seed=5)
    flat = oracle.OracleScene(sd, force_mode=1)
    two = oracle.OracleScene(sd, force_mode=2)
    assert two.two_level and not flat.two_level
    rng = np.random.default_rng(4)
    rays = random_rays(rng, 3000, -60, 60)
    ht, hf = two.trace(rays, 0), flat.trace(rays, 0)
    hb = two.trace(rays, 2)
    assert np.array_equal(ht, hb)
    # flat and two-level agree on what was hit (t may differ in the last bits:
    # the triangle test runs in world vs object space)
    same = (ht[:, 3] == hf[:, 3]) & (ht[:, 4] == hf[:, 4])
    assert same.mean() > 0.999
    assert np.array_equal(two.trace(rays, 1)[:, 0], flat.trace(rays, 1)[:, 0]) or \
        (two.trace(rays, 1)[:, 0] != flat.trace(rays, 1)[:, 0]).mean() < 1e-3


def test_fp32_fp64_integrator_agree_cornell(oracle):
    sd = scenes.cornell(32, 32, 4)
    sc = oracle.OracleScene(sd)
    v = sd.views[0]
    st = dict(max_bounces=4, sampler=0)
    p32 = sc.render_paths(v, st, 0, 4)
    p64 = sc.render_paths(v, st, 0, 4, fp64=True)
    rel = np.abs(p32 - p64) / np.maximum(np.abs(p64), 1e-3)
    assert np.isfinite(p32).all()
    assert np.mean(rel < 1e-3) > 0.99
    assert abs(p32.mean() - p64.mean()) / p64.mean() < 1e-3


def test_fp32_fp64_agree_vndf_mode(oracle):
    """The VNDF stage-B mode in FP32 and FP64 on a scene of smooth and rough
    metals and dielectrics; the flag changes the estimator."""
    pos, nrm, uv, idx = scenes.displaced_sphere(8, seed=2)
    b = scenes._Builder()
    rng = np.random.default_rng(3)
    nt = idx.shape[0]
    mats = scenes._random_materials(rng, nt + 1)
    mats[nt] = scenes.material((0.5, 0.5, 0.5), rough=0.3)
    b.add(pos, nrm, uv, idx, np.arange(nt, dtype=np.uint32))
    scenes._ground(b, -1.05, 6.0, nt)
    P, N, U, I, M = b.arrays()
    env = scenes.sky_env(64, 32, seed=2, peak=50.0, radius_deg=3.0)
    view = scenes.look_at_view((0, 0.6, 3.2), (0, -0.1, 0), width=24, height=16)
    sd = scenes.SceneData("vndf", P, N, U, I, M, mats, np.zeros((0, 20), np.float32), env, 1.0, [(0, I.size)],
                          scenes.identity_instance(1), [view], spp=4, max_bounces=3)
    sc = oracle.OracleScene(sd)
    st = dict(max_bounces=3, sampler=1, flags=1 << 9)
    p32 = sc.render_paths(view, st, 0, 4)
    p64 = sc.render_paths(view, st, 0, 4, fp64=True)
    assert np.isfinite(p32).all() and (p32 >= 0).all()
    rel = np.abs(p32 - p64) / np.maximum(np.abs(p64), 1e-3)
    assert np.mean(rel < 1e-3) > 0.98
    assert abs(p32.mean() - p64.mean()) / p64.mean() < 2e-3
    assert not np.array_equal(p32, sc.render_paths(view, dict(max_bounces=3, sampler=1), 0, 4))


@pytest.mark.parametrize("sampler", [0, 1])
def test_oracle_render_env_scene(oracle, sampler):
    pos, nrm, uv, idx = scenes.displaced_sphere(8, seed=1)
    b = scenes._Builder()
    rng = np.random.default_rng(0)
    nt = idx.shape[0]
    mats = scenes._random_materials(rng, nt + 1)
    mats[nt] = scenes.material((0.5, 0.5, 0.5), rough=0.8)
    b.add(pos, nrm, uv, idx, np.arange(nt, dtype=np.uint32))
    scenes._ground(b, -1.05, 6.0, nt)
    P, N, U, I, M = b.arrays()
    env = scenes.sky_env(64, 32, seed=1, peak=500.0, radius_deg=3.0)
    view = scenes.look_at_view((0, 0.6, 3.2), (0, -0.1, 0), width=24, height=16)
    sd = scenes.SceneData("t", P, N, U, I, M, mats, np.zeros((0, 20), np.float32), env, 1.0, [(0, I.size)],
                          scenes.identity_instance(1), [view])
    sc = oracle.OracleScene(sd)
    p = sc.render_paths(view, dict(max_bounces=4, sampler=sampler), 0, 2)
    assert np.isfinite(p).all() and p.mean() > 0.05


def _empty_scene(env):
    v = scenes.look_at_view((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), width=8, height=4)
    return scenes.SceneData("empty", np.zeros((0, 3), np.float32), np.zeros((0, 4), np.float32),
                            np.zeros((0, 2), np.float32), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                            scenes.material((0.5, 0.5, 0.5))[None], np.zeros((0, 20), np.float32), env, 1.0,
                            [(0, 0)], scenes.identity_instance(1), [v])


@pytest.mark.parametrize("kind", ["no_triangles", "all_masked"])
def test_scene_without_visible_geometry(oracle, kind):
    """No triangles, or every instance masked out: every ray misses and every
    path is the environment seen by its camera ray (the sky is 0.5 away from
    the sun)."""
    env = scenes.sky_env(64, 32, seed=1)
    if kind == "no_triangles":
        sd = _empty_scene(env)
    else:
        sd = scenes.cornell(8, 4, 1)
        sd.env, sd.env_intensity = env, 1.0
        sd.lights = np.zeros((0, 20), np.float32)
        sd.instances = sd.instances.copy()
        sd.instances["mask"] = 0
    orc = oracle.OracleScene(sd)
    rng = np.random.default_rng(2)
    rays = random_rays(rng, 256, -1.0, 1.0)
    for mode in (0, 1, 2):
        h = orc.trace(rays, mode)
        assert np.all(h[:, 3:5] == 0xFFFFFFFF), f"mode {mode}: a hit in a scene without geometry"
    p = orc.render_paths(sd.views[0], dict(max_bounces=4, sampler=0), 0, 2)
    assert p.shape == (2, 32, 3) and np.all(p == np.float32(0.5))


@pytest.mark.parametrize("flatten_limit", [1 << 25, 1])
def test_zero_scale_instance_equals_masked(oracle, flatten_limit):
    """A singular instance transform (zero scale) has no inverse; the build
    treats the instance as masked out, flat and two-level alike."""
    from pt_harness import small_instanced
    sd = small_instanced(side=8)
    sd.instances = sd.instances.copy()
    x = sd.instances[5]["xform"].reshape(3, 4).copy()
    x[:, :3] = 0.0
    sd.instances[5]["xform"] = x.reshape(-1)
    m = small_instanced(side=8)
    m.instances = m.instances.copy()
    m.instances["mask"][5] = 0
    a = oracle.OracleScene(sd, flatten_limit=flatten_limit)
    b = oracle.OracleScene(m, flatten_limit=flatten_limit)
    rng = np.random.default_rng(3)
    rays = random_rays(rng, 4000, -60, 60)
    ha = a.trace(rays, 0)
    assert np.array_equal(ha, b.trace(rays, 0))
    assert np.all(np.isfinite(ha[:, 0].view(np.float32)))
    assert np.array_equal(a.render_paths(sd.views[0], dict(max_bounces=3), 0, 1),
                          b.render_paths(m.views[0], dict(max_bounces=3), 0, 1))


def test_pow_definition_accuracy(oracle):
    """The pow shared by the oracle and the kernels (exp2(y log2 x), both
    defined from their series) against float64 pow: within 1e-5 relative
    (float exp2 of a float exponent of magnitude up to ~44 here; GLSL allows
    pow the error of exp2(y * log2(x)), several ulp)."""
    import ctypes as C
    rng = np.random.default_rng(8)
    x = np.exp(rng.uniform(np.log(1e-6), 0.0, 200000)).astype(np.float32)
    for y in (2.2, 1.0 / 2.2, 0.7, 3.0):
        got = oracle.pow_def(x, np.float32(y))
        ref = x.astype(np.float64) ** np.float64(np.float32(y))
        rel = np.abs(got - ref) / ref
        assert rel.max() < 1e-5, (y, rel.max())
    assert oracle.pow_def(np.array([0.0, 1.0], np.float32), np.float32(2.2)).tolist() == [0.0, 1.0]


def test_alpha_test_bvh_equals_brute_force(oracle):
    sd = scenes.textured()
    for fl in (1 << 25, 1):
        orc = oracle.OracleScene(sd, flatten_limit=fl)
        rng = np.random.default_rng(5)
        rays = random_rays(rng, 6000, -1.5, 1.5)
        for alpha in (False, True):
            assert np.array_equal(orc.trace(rays, 0, alpha=alpha), orc.trace(rays, 2, alpha=alpha))
        assert not np.array_equal(orc.trace(rays, 0), orc.trace(rays, 0, alpha=True))
