"""GPU parity on the scene kinds the base parity tests leave out: the four
analytic light types of stage A's next-event estimation
(pt_raygen.rgen:305-435: sphere, directional, spot, area), scenes without
visible geometry (no triangles; every instance masked; a zero-scale
instance), the full instanced benchmark scene (10,000 instances, two-level)
on a seeded pixel subset, and the device-side checks that must return a
status instead of faulting (the traversal stack limit, the denoiser's
bounded tensor-core waits).

Bars as in test_gpu_parity: per-path radiance within 1e-4 relative of the
host oracle (FP32), accumulation and hits bit-exact.
"""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pin_cases import CASES
from pt_harness import gpu_tracer, random_rays, rel_err, render_paths_gpu, small_instanced, trace_gpu

pytestmark = pytest.mark.gpu

RTOL = 1e-4
DEVICE_CHECK = -7
TIMEOUT = -4


def assert_paths_match(gpu, ref, what):
    assert gpu.shape == ref.shape
    assert np.isfinite(gpu).all(), what
    err = rel_err(gpu, ref, floor=1e-3)
    bad = np.argwhere(err > RTOL)
    assert bad.size == 0, f"{what}: {len(bad)} components beyond {RTOL} (first {bad[:5].tolist()})"


@pytest.mark.parametrize("case", ["cornell_area_pcg", "cornell_4_types_sobol", "env_lights_sobol"])
def test_light_types_paths(gpu_lib, oracle, case):
    """Sphere, directional, spot and area GPULights (with and without an
    environment), per path against the oracle, whose paths equal the
    reference shaders' on these scenes (tests/golden/glsl_kats.json)."""
    maker, st, fl = CASES[case]
    sd = maker()
    assert len(sd.lights) >= 1
    pt = gpu_tracer(gpu_lib, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl)
    v = sd.views[0]
    kw = dict(max_bounces=st["max_bounces"], sampler=st["sampler"], sample_index_base=3)
    g, acc, _ = render_paths_gpu(gpu_lib, pt, v, 4, kw)
    o = orc.render_paths(v, st, 3, 4)
    assert_paths_match(g, o, case)
    assert np.array_equal(acc.cpu().numpy(), oracle.accumulate(o))


def _empty_scene(env):
    v = scenes.look_at_view((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), width=16, height=8)
    return scenes.SceneData("empty", np.zeros((0, 3), np.float32), np.zeros((0, 4), np.float32),
                            np.zeros((0, 2), np.float32), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                            scenes.material((0.5, 0.5, 0.5))[None], np.zeros((0, 20), np.float32), env, 1.0,
                            [(0, 0)], scenes.identity_instance(1), [v])


@pytest.mark.parametrize("kind", ["no_triangles", "all_masked"])
def test_scene_without_visible_geometry(gpu_lib, oracle, kind):
    """No triangles, or every instance masked out (no visible triangle, so
    the build is flat whatever the flatten limit): every ray misses, every
    path is the environment seen by its camera ray; the device agrees with
    the oracle path by path and hit by hit, in the wavefront and the pool."""
    import torch
    og = gpu_lib
    env = scenes.sky_env(64, 32, seed=1)
    fl = 0
    if kind == "no_triangles":
        sd = _empty_scene(env)
    else:
        sd = scenes.cornell(16, 8, 1)
        sd.env, sd.env_intensity = env, 1.0
        sd.lights = np.zeros((0, 20), np.float32)
        sd.instances = sd.instances.copy()
        sd.instances["mask"] = 0
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    rng = np.random.default_rng(2)
    rays = random_rays(rng, 2048, -1.0, 1.0)
    h = trace_gpu(og, pt, rays)
    assert np.all(h[:, 3:5] == 0xFFFFFFFF)
    assert np.array_equal(h, orc.trace(rays, 0))
    assert not trace_gpu(og, pt, rays, any_hit=True)[:, 0].any()
    v = sd.views[0]
    g, acc, _ = render_paths_gpu(og, pt, v, 2, dict(max_bounces=4, sampler=0))
    o = orc.render_paths(v, dict(max_bounces=4, sampler=0), 0, 2)
    assert_paths_match(g, o, kind)
    assert np.all(g == np.float32(0.5))
    acc2 = torch.zeros_like(acc)
    pt.render([og.make_view(v, accum=acc2), og.make_view(v, accum=torch.zeros_like(acc))],
              og.make_settings(spp=2, max_bounces=4, mode=og.MODE_PERSISTENT))
    torch.cuda.synchronize()
    assert torch.equal(acc2, acc)


@pytest.mark.parametrize("two_level", [False, True])
def test_zero_scale_instance_is_masked(gpu_lib, oracle, two_level):
    """An instance with a singular transform (scale 0, often used to hide an
    instance) has no inverse: the build treats it as masked out, on the
    device and in the oracle, instead of tracing with inf/NaN matrices."""
    og = gpu_lib
    sd = small_instanced(side=16)
    sd.instances = sd.instances.copy()
    hidden = [3, 17, 40]
    for i in hidden:
        x = sd.instances[i]["xform"].reshape(3, 4).copy()
        x[:, :3] = 0.0
        sd.instances[i]["xform"] = x.reshape(-1)
    fl = 1 if two_level else 0
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    masked = small_instanced(side=16)
    masked.instances = masked.instances.copy()
    masked.instances["mask"][hidden] = 0
    orc_m = oracle.OracleScene(masked, flatten_limit=fl if fl else 1 << 25)
    rng = np.random.default_rng(4)
    rays = random_rays(rng, 20000, -60, 60)
    gh = trace_gpu(og, pt, rays)
    assert np.array_equal(gh, orc.trace(rays, 0))
    assert np.array_equal(gh, orc_m.trace(rays, 0)), "a zero-scale instance differs from a masked one"
    assert not np.isin(gh[:, 3], hidden).any()
    v = sd.views[0]
    g, _, _ = render_paths_gpu(og, pt, v, 2, dict(max_bounces=4, sampler=0))
    assert_paths_match(g, orc.render_paths(v, dict(max_bounces=4, sampler=0), 0, 2), "zero-scale instance")


def test_full_instanced_scene_subset(gpu_lib, oracle):
    """The full instanced benchmark scene (10,000 instances of 5 meshes,
    362,500 base triangles, two-level): per-path radiance on 4,000 seeded
    pixels of its largest view, through the per-view wavefront and the
    persistent pool."""
    import torch
    og = gpu_lib
    sd = scenes.instanced()
    pt = gpu_tracer(og, sd)
    assert pt.two_level
    orc = oracle.OracleScene(sd)
    assert orc.two_level
    v = max(sd.views, key=lambda x: x.width * x.height)
    npix = v.width * v.height
    g, acc, _ = render_paths_gpu(og, pt, v, 1, dict(max_bounces=4, sampler=0, sample_index_base=1))
    rng = np.random.default_rng(11)
    pix = np.sort(rng.choice(npix, 4000, replace=False)).astype(np.uint32)
    o = orc.render_paths(v, dict(max_bounces=4, sampler=0), 1, 1, pixels=pix)
    assert_paths_match(g[:, pix], o, "instanced 10k subset")
    acc2 = torch.zeros_like(acc)
    pt.launch_config = "pool_4M_unsorted_fetch4_chunk8"
    pt.render([og.make_view(v, accum=acc2)], og.make_settings(spp=1, max_bounces=4, sample_index_base=1,
                                                              mode=og.MODE_PERSISTENT))
    torch.cuda.synchronize()
    assert torch.equal(acc2, acc)
    rays = random_rays(rng, 20000, -60, 60)
    assert np.array_equal(trace_gpu(og, pt, rays), orc.trace(rays, 0))


def test_stack_limit_returns_device_check(gpu_lib, oracle):
    """A traversal that needs more stack than the per-ray limit stops with
    OHAO_ERR_DEVICE_CHECK (no write past the stack, no fault), and the next
    render on the same context, with the full stack, is correct."""
    import torch
    og = gpu_lib
    from pt_harness import small_env_scene
    sd = small_env_scene(freq=24)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    acc = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
    for mode in (og.MODE_WAVEFRONT, og.MODE_PERSISTENT):
        with pytest.raises(og.OhaoError) as e:
            pt.render([og.make_view(v, accum=acc)], og.make_settings(spp=1, max_bounces=2, trace_stack_limit=1,
                                                                     mode=mode))
        assert e.value.status == DEVICE_CHECK
    g, acc, _ = render_paths_gpu(og, pt, v, 2, dict(max_bounces=4, sampler=0))
    orc = oracle.OracleScene(sd)
    assert_paths_match(g, orc.render_paths(v, dict(max_bounces=4, sampler=0), 0, 2), "after the stack check")


def test_denoiser_wait_timeout_is_a_status(gpu_lib):
    """The tensor-core pipeline's bounded wait, made to run out on an
    mbarrier that nothing arrives on, reaches the ABI as OHAO_ERR_TIMEOUT;
    the denoiser context stays usable."""
    import torch
    from ohao_engine_gb300.denoise import Denoiser
    og = gpu_lib
    dn = Denoiser(max_pixels=32 * 32, seed=1)
    assert dn.wait_selftest(256) == TIMEOUT
    assert dn.wait_selftest(4096) == TIMEOUT
    rad = torch.rand((32 * 32, 4), device="cuda")
    aov = torch.rand((32 * 32, og.AOV_FLOATS), device="cuda")
    out = torch.zeros_like(rad)
    dn.infer([rad], [aov], [out], 32, 32)
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    dn.close()


@pytest.mark.parametrize("stride", [12, 100])
def test_device_geometry_upload(gpu_lib, stride):
    """ohao_pt_set_geometry_device (device buffers, a stream, OHAO's 100-byte
    Vertex stride) builds the same BVH and renders the same image as the
    host-array upload; an out-of-range index is rejected on the device."""
    import torch
    og = gpu_lib
    sd = small_instanced(side=16)
    ref = gpu_tracer(og, sd)
    v = sd.views[0]
    npix = v.width * v.height
    acc_ref = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    ref.render([og.make_view(v, accum=acc_ref)], og.make_settings(spp=2, max_bounces=4))
    nv, nt = sd.pos.shape[0], sd.ntris
    packed = np.zeros((nv, stride // 4), np.float32)
    packed[:, :3] = sd.pos
    packed[:, 3:] = 7.0   # other vertex attributes the stride skips
    stream = torch.cuda.Stream()
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in
         (packed, sd.normals, sd.uvs, sd.indices.astype(np.int32), sd.mat_ids.astype(np.int32))]
    pt = og.PathTracer()
    pt.set_geometry_device(d[0], d[1], d[2], d[3], d[4], nv, nt, pos_stride_bytes=stride, stream=stream.cuda_stream)
    for fi, ic in sd.blas:
        pt.create_blas(fi, ic)
    pt.set_instances(sd.instances)
    pt.set_materials(sd.materials)
    pt.set_env(sd.env, intensity=sd.env_intensity)
    pt.build()
    for which in (-1,):
        a, b = pt.bvh(which), ref.bvh(which)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    acc = torch.zeros_like(acc_ref)
    pt.render([og.make_view(v, accum=acc)], og.make_settings(spp=2, max_bounces=4))
    torch.cuda.synchronize()
    assert torch.equal(acc, acc_ref)
    bad = d[3].clone()
    bad[5] = nv
    with pytest.raises(og.OhaoError) as e:
        pt.set_geometry_device(d[0], d[1], d[2], bad, d[4], nv, nt, pos_stride_bytes=stride)
    assert e.value.status == -1
    pt.close()
    ref.close()
