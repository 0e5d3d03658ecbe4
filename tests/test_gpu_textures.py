"""Bindless textures and the alpha test on the GPU against the oracle:
diffuse (sRGB-decoded), normal (Frisvad basis), roughness-metal and
emissive textures in closest-hit shading (pt_closesthit.rchit:108-157) and
the any-hit alpha test (pt_anyhit.rahit:17-50) for non-opaque geometry and
rays, flat and two-level, per path within 1e-4 (observed: bit-identical),
hits bit-exact."""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pt_harness import gpu_tracer, random_rays, rel_err, render_paths_gpu, trace_gpu

pytestmark = pytest.mark.gpu

RTOL = 1e-4
ALPHA = 1 << 10


def assert_paths_match(gpu, ref, what):
    assert gpu.shape == ref.shape
    assert np.isfinite(gpu).all(), what
    err = rel_err(gpu, ref, floor=1e-3)
    bad = np.argwhere(err > RTOL)
    assert bad.size == 0, f"{what}: {len(bad)} components beyond {RTOL} (first {bad[:5].tolist()})"


@pytest.mark.parametrize("two_level", [False, True])
@pytest.mark.parametrize("alpha", [False, True])
@pytest.mark.parametrize("sampler", [0, 1])
def test_textured_paths(gpu_lib, oracle, two_level, alpha, sampler):
    og = gpu_lib
    sd = scenes.textured()
    fl = 1 if two_level else 0
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    assert pt.two_level == two_level
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    v = sd.views[0]
    flags = ALPHA if alpha else 0
    g, acc, _ = render_paths_gpu(og, pt, v, 4, dict(max_bounces=4, sampler=sampler, flags=flags, sample_index_base=1))
    o = orc.render_paths(v, dict(max_bounces=4, sampler=sampler, flags=flags), 1, 4)
    assert_paths_match(g, o, f"textured two_level={two_level} alpha={alpha}")
    assert np.array_equal(acc.cpu().numpy(), oracle.accumulate(o))


def test_textures_change_the_image(oracle):
    """Each texture kind matters on this scene (the parity above would also
    hold for a shader that ignored them)."""
    sd = scenes.textured()
    v = sd.views[0]
    base = oracle.OracleScene(sd).render_paths(v, dict(max_bounces=3, flags=ALPHA), 0, 2)
    for slot in (3, 6, 7, 8):
        s2 = scenes.textured()
        s2.materials = s2.materials.copy()
        s2.materials[:, slot] = np.array([0xFFFFFFFF], np.uint32).view(np.float32)[0]
        assert not np.array_equal(oracle.OracleScene(s2).render_paths(v, dict(max_bounces=3, flags=ALPHA), 0, 2),
                                  base), f"texture slot {slot} has no effect"
    assert not np.array_equal(oracle.OracleScene(sd).render_paths(v, dict(max_bounces=3), 0, 2), base)


@pytest.mark.parametrize("two_level", [False, True])
def test_alpha_trace_bit_exact(gpu_lib, oracle, two_level):
    """Closest and any hit of non-opaque rays through the alpha-tested
    leaves: equal to the oracle's BVH walk and to brute force."""
    og = gpu_lib
    sd = scenes.textured()
    fl = 1 if two_level else 0
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    rng = np.random.default_rng(12)
    rays = random_rays(rng, 20000, -1.5, 1.5)
    rays[:, 0:3] = rng.uniform((-1.5, -0.8, 2.0), (1.5, 0.2, 3.0), (20000, 3))   # in front of the leaves
    rays[:, 4:7] = np.array([0.0, 0.0, -1.0]) + rng.normal(scale=0.3, size=(20000, 3))
    rays[:, 4:7] /= np.linalg.norm(rays[:, 4:7], axis=1, keepdims=True)
    import torch
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    for alpha in (False, True):
        h = torch.zeros((20000, 5), dtype=torch.int32, device="cuda")
        pt.trace(r, 20000, h, alpha=alpha)
        torch.cuda.synchronize()
        gh = h.cpu().numpy().view(np.uint32)
        assert np.array_equal(gh, orc.trace(rays, 0, alpha=alpha)), f"closest alpha={alpha}"
        assert np.array_equal(gh, orc.trace(rays, 2, alpha=alpha)), f"brute force alpha={alpha}"
        h.zero_()
        pt.trace(r, 20000, h, any_hit=True, alpha=alpha)
        torch.cuda.synchronize()
        assert np.array_equal(h.cpu().numpy().view(np.uint32)[:, 0], orc.trace(rays, 1, alpha=alpha)[:, 0])
    # the cut-outs let rays through: some hits move behind the leaves
    opaque = orc.trace(rays, 0)
    cut = orc.trace(rays, 0, alpha=True)
    assert (opaque[:, 4] != cut[:, 4]).mean() > 0.05


def test_textured_pool_equals_wavefront(gpu_lib):
    import torch
    og = gpu_lib
    sd = scenes.textured()
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    ref = None
    for mode in (og.MODE_WAVEFRONT, og.MODE_PERSISTENT):
        for name in (["default"] if mode == og.MODE_WAVEFRONT else pt.launch_configs()):
            if name != "default":
                pt.launch_config = name
            acc = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
            pt.render([og.make_view(v, accum=acc)], og.make_settings(spp=3, max_bounces=4, flags=ALPHA, mode=mode))
            torch.cuda.synchronize()
            if ref is None:
                ref = acc.clone()
            assert torch.equal(acc, ref), name


def test_texture_errors(gpu_lib):
    import torch
    og = gpu_lib
    sd = scenes.textured()
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    acc = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
    pt.set_textures(sd.textures[:3])           # materials name textures 3..5: nothing renders
    with pytest.raises(og.OhaoError) as e:
        pt.render([og.make_view(v, accum=acc)], og.make_settings())
    assert e.value.status == -1
    pt.set_textures(sd.textures)
    pt.render([og.make_view(v, accum=acc)], og.make_settings())
    gm = torch.zeros(1, device="cuda")
    gr = torch.zeros(sd.materials.shape[0], device="cuda")
    with pytest.raises(og.OhaoError) as e:    # the adjoint does not differentiate bindless textures
        pt.adjoint([og.make_view(v, accum=acc)], og.make_settings(), [acc.clone()], None, gr)
    assert e.value.status == -6
    bad = sd.materials.copy()
    bad[0, 6] = np.array([70000], np.uint32).view(np.float32)[0]
    with pytest.raises(og.OhaoError):
        pt.set_materials(bad)
    with pytest.raises(og.OhaoError):
        pt.set_blas_flags(7, 1)
    pt.close()
