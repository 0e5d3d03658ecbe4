"""GPU parity: the CUDA path (through the C ABI) against the host oracle.

Bars: BVH nodes and triangle records bit-exact; closest-hit (t, u, v,
instance, primitive) and any-hit bit-exact; per-path radiance within 1e-4
relative in FP32 (the kernels follow the oracle's operation order, so the
expected and observed result is bit equality); accumulation bit-exact.
"""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pt_harness import (gpu_tracer, random_rays, rel_err, render_paths_gpu, small_env_scene, small_instanced,
                        trace_gpu)

pytestmark = pytest.mark.gpu

RTOL = 1e-4   # per-path radiance tolerance (FP32)


def assert_paths_match(gpu, ref, what):
    assert gpu.shape == ref.shape
    assert np.isfinite(gpu).all(), what
    err = rel_err(gpu, ref, floor=1e-3)
    bad = np.argwhere(err > RTOL)
    assert bad.size == 0, f"{what}: {len(bad)} components beyond {RTOL} (first {bad[:5].tolist()})"


@pytest.mark.parametrize("maker", ["cornell", "small_env"])
def test_bvh_bit_exact_flat(gpu_lib, oracle, maker):
    sd = scenes.cornell(16, 16, 1) if maker == "cornell" else small_env_scene(freq=24)
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    assert not pt.two_level
    gn, gt, gh = pt.bvh()
    on, ot, oh = orc.bvh()
    assert gh == oh
    assert np.array_equal(gn, on), "node bytes differ"
    assert np.array_equal(gt, ot), "triangle records differ"


def test_bvh_bit_exact_two_level(gpu_lib, oracle):
    sd = small_instanced()
    pt = gpu_tracer(gpu_lib, sd, flatten_limit=1)
    orc = oracle.OracleScene(sd, flatten_limit=1)
    assert pt.two_level and orc.two_level
    gn, gi, _ = pt.bvh(-1)
    on, oi, _ = orc.bvh(-1)
    assert np.array_equal(gn, on) and np.array_equal(gi, oi)
    for b in range(len(sd.blas)):
        gn, gt, _ = pt.bvh(b)
        on, ot, _ = orc.bvh(b)
        assert np.array_equal(gn, on) and np.array_equal(gt, ot), f"BLAS {b}"


@pytest.mark.parametrize("two_level", [False, True])
def test_trace_bit_exact(gpu_lib, oracle, two_level):
    if two_level:
        sd = small_instanced()
        lo, hi = -60, 60
    else:
        sd = small_env_scene(freq=24)
        lo, hi = -2, 2
    fl = 1 if two_level else 0
    pt = gpu_tracer(gpu_lib, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    rng = np.random.default_rng(7)
    rays = random_rays(rng, 20000, lo, hi)
    gh, gs = trace_gpu(gpu_lib, pt, rays, stats=True)
    oh, os_ = orc.trace(rays, 0, stats=True)
    assert np.array_equal(gh, oh), f"{int((gh != oh).any(axis=1).sum())} rays differ"
    assert np.array_equal(gs, os_), "node/triangle visit counts differ"
    assert np.array_equal(gh, orc.trace(rays, 2)), "BVH result differs from brute force"
    ga = trace_gpu(gpu_lib, pt, rays, any_hit=True)
    oa = orc.trace(rays, 1)
    assert np.array_equal(ga[:, 0], oa[:, 0])


@pytest.mark.parametrize("sampler", [0, 1])
def test_render_cornell_paths(gpu_lib, oracle, sampler):
    sd = scenes.cornell(48, 40, 4)
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    v = sd.views[0]
    kw = dict(max_bounces=4, sampler=sampler, sample_index_base=3)
    g, acc, _ = render_paths_gpu(gpu_lib, pt, v, 4, kw)
    o = orc.render_paths(v, dict(max_bounces=4, sampler=sampler), 3, 4)
    assert_paths_match(g, o, "cornell")
    ref_acc = oracle.accumulate(o)
    assert np.array_equal(acc.cpu().numpy(), ref_acc)


@pytest.mark.parametrize("sampler", [0, 1])
def test_render_env_paths(gpu_lib, oracle, sampler):
    sd = small_env_scene(freq=16)
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    v = sd.views[0]
    g, acc, _ = render_paths_gpu(gpu_lib, pt, v, 3, dict(max_bounces=4, sampler=sampler))
    o = orc.render_paths(v, dict(max_bounces=4, sampler=sampler), 0, 3)
    assert_paths_match(g, o, "env sphere")
    assert np.array_equal(acc.cpu().numpy(), oracle.accumulate(o))


@pytest.mark.parametrize("sampler", [0, 1])
def test_render_vndf_mode_paths(gpu_lib, oracle, sampler):
    """The VNDF stage-B estimator mode (OHAO_PT_FLAG_GGX_VNDF) per path
    against the oracle, on a scene with smooth and rough metals and
    dielectrics under an environment with a sun."""
    sd = small_env_scene(freq=16)
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    v = sd.views[0]
    fl = gpu_lib.FLAG_GGX_VNDF
    g, acc, _ = render_paths_gpu(gpu_lib, pt, v, 3, dict(max_bounces=4, sampler=sampler, flags=fl))
    o = orc.render_paths(v, dict(max_bounces=4, sampler=sampler, flags=fl), 0, 3)
    assert_paths_match(g, o, "vndf")
    assert np.array_equal(acc.cpu().numpy(), oracle.accumulate(o))
    plain = orc.render_paths(v, dict(max_bounces=4, sampler=sampler), 0, 3)
    assert not np.array_equal(plain, o)   # the flag changes the estimator


def test_render_two_level_paths(gpu_lib, oracle):
    sd = small_instanced(side=24)
    pt = gpu_tracer(gpu_lib, sd, flatten_limit=1)
    orc = oracle.OracleScene(sd, flatten_limit=1)
    for v in sd.views[:2]:
        g, _, _ = render_paths_gpu(gpu_lib, pt, v, 2, dict(max_bounces=4, sampler=0))
        o = orc.render_paths(v, dict(max_bounces=4, sampler=0), 0, 2)
        assert_paths_match(g, o, "instanced")


def test_firefly_clamp_and_depth(gpu_lib, oracle):
    sd = small_env_scene(freq=12, env_peak=5e4)
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    v = sd.views[0]
    for mb, flags in ((2, 1 << 2), (0, 0), (1, 1 << 2)):
        kw = dict(max_bounces=mb, sampler=1, flags=flags, clamp_luminance=5.0)
        g, _, _ = render_paths_gpu(gpu_lib, pt, v, 2, kw)
        o = orc.render_paths(v, dict(max_bounces=mb, sampler=1, flags=flags, clamp_lum=5.0), 0, 2)
        assert_paths_match(g, o, f"depth {mb} flags {flags}")


def test_progressive_accumulation_and_host_path(gpu_lib, oracle):
    import torch
    sd = scenes.cornell(24, 24, 1)
    pt = gpu_tracer(gpu_lib, sd)
    v = sd.views[0]
    acc = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
    g1, _, _ = render_paths_gpu(gpu_lib, pt, v, 2, dict(max_bounces=4, sample_index_base=0), history=0, accum=acc)
    g2, _, _ = render_paths_gpu(gpu_lib, pt, v, 3, dict(max_bounces=4, sample_index_base=2), history=2, accum=acc)
    ref = oracle.accumulate(np.concatenate([g1, g2]))
    assert np.array_equal(acc.cpu().numpy(), ref)
    host = np.zeros((v.width * v.height, 4), np.float32)
    pt.render_host([gpu_lib.make_view(v)], gpu_lib.make_settings(spp=5, max_bounces=4), [host])
    assert np.array_equal(host, ref)


@pytest.mark.parametrize("mode", ["wavefront", "persistent"])
def test_host_path_with_history(gpu_lib, oracle, mode):
    """ohao_pt_render_host continuing a host accumulator (history > 0): its
    upload overlaps the render on another stream, and the result equals the
    device-buffer render of the same samples bit for bit; on a small frame
    it equals the oracle's accumulation, on a 1024^2 frame (an upload long
    enough to still be in flight) the device path."""
    import torch
    og = gpu_lib
    m = og.MODE_WAVEFRONT if mode == "wavefront" else og.MODE_PERSISTENT
    sd = scenes.cornell(24, 24, 1)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    g1, _, _ = render_paths_gpu(og, pt, v, 2, dict(max_bounces=4, sample_index_base=0), history=0)
    g2, _, _ = render_paths_gpu(og, pt, v, 3, dict(max_bounces=4, sample_index_base=2), history=2)
    host = oracle.accumulate(g1).astype(np.float32)
    pt.render_host([og.make_view(v, history=2)], og.make_settings(spp=3, max_bounces=4, sample_index_base=2, mode=m),
                   [host])
    assert np.array_equal(host, oracle.accumulate(np.concatenate([g1, g2])))
    big = scenes.cornell(1024, 1024, 1)
    pt2 = gpu_tracer(og, big)
    vb = big.views[0]
    n = vb.width * vb.height
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    pt2.render([og.make_view(vb, accum=acc)], og.make_settings(spp=2, max_bounces=2, mode=m))
    host_b = acc.cpu().numpy().copy()
    pt2.render([og.make_view(vb, accum=acc, history=2)],
               og.make_settings(spp=1, max_bounces=2, sample_index_base=2, mode=m))
    for _ in range(2):   # twice: the second call's upload follows the first call's download of the same buffer
        h = host_b.copy()
        pt2.render_host([og.make_view(vb, history=2)],
                        og.make_settings(spp=1, max_bounces=2, sample_index_base=2, mode=m), [h])
        assert np.array_equal(h, acc.cpu().numpy())


def test_aov_first_hit(gpu_lib, oracle):
    sd = scenes.cornell(20, 20, 1)
    pt = gpu_tracer(gpu_lib, sd)
    _, _, aov = render_paths_gpu(gpu_lib, pt, sd.views[0], 1, dict(max_bounces=1), aov=True)
    a = aov.cpu().numpy().reshape(20, 20, 12)
    centre = a[5:15, 5:15].reshape(-1, 12)
    assert np.all(centre[:, 7] == 1.0)      # the centre of the frame sees the box interior
    flat = a.reshape(-1, 12)
    hit = flat[flat[:, 7] == 1.0]
    assert np.all((hit[:, 0:3] >= 0) & (hit[:, 0:3] <= 1))
    n = hit[:, 3:6] * 2.0 - 1.0
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    assert np.all(hit[:, 6] > 0)
    # roughness and metallic of the hit material (the Cornell box: rough dielectrics)
    mats = sd.materials
    assert np.all((hit[:, 8] >= 0) & (hit[:, 8] <= 1)) and np.all(np.isin(hit[:, 9], mats[:, 5]))
    assert np.all(np.isin(hit[:, 8], mats[:, 4]))
    miss = flat[flat[:, 7] == 0.0]
    assert np.all(miss[:, 8:12] == 0.0) and np.all(hit[:, 10:12] == 0.0)


def test_errors_are_status_codes(gpu_lib):
    import torch
    og = gpu_lib
    pt = og.PathTracer()
    sd = scenes.cornell(8, 8, 1)
    pt.set_geometry(sd.pos, sd.normals, sd.uvs, sd.indices, sd.mat_ids)
    with pytest.raises(og.OhaoError) as e:
        pt.render([og.make_view(sd.views[0])], og.make_settings())
    assert e.value.status in (-1, -5)
    with pytest.raises(og.OhaoError):
        pt.create_blas(0, 10 ** 6)
    bad = sd.materials.copy()
    bad[0, 6:7] = np.array([70000], np.uint32).view(np.float32)   # beyond the 65536 texture slots
    with pytest.raises(og.OhaoError) as e:
        pt.set_materials(bad)
    assert e.value.status == -1
    pt.set_materials(sd.materials)
    with pytest.raises(og.OhaoError) as e:
        pt.update_materials(bad[:1])
    assert e.value.status == -1
    with pytest.raises(og.OhaoError) as e:
        pt.update_materials(sd.materials[:1], first=sd.materials.shape[0])
    assert e.value.status == -1
    # a texture index that names no texture: accepted in the table, refused by a render
    missing = sd.materials.copy()
    missing[0, 6:7] = np.array([3], np.uint32).view(np.float32)
    pt.set_materials(missing)
    for fi, ic in sd.blas:
        pt.create_blas(fi, ic)
    pt.set_instances(sd.instances)
    pt.build()
    with pytest.raises(og.OhaoError) as e:
        pt.render([og.make_view(sd.views[0], accum=torch.zeros((64, 4), device="cuda"))], og.make_settings())
    assert e.value.status == -1


def test_build_rechecks_blas_ranges(gpu_lib):
    """A BLAS created over the old geometry that a smaller new geometry no
    longer covers: the build reports it instead of reading past the index
    buffer, nothing renders from that state, and restoring the geometry
    builds again."""
    og = gpu_lib
    sd = scenes.cornell(8, 8, 1)
    idx = np.asarray(sd.indices, np.uint32)
    mids = np.asarray(sd.mat_ids, np.uint32)
    pt = og.PathTracer()
    pt.set_geometry(sd.pos, sd.normals, sd.uvs, idx, mids)
    b = pt.create_blas(54, 54)                       # the second half of the 36 triangles
    inst = scenes.identity_instance(1)
    inst["blas"] = b
    pt.set_instances(inst)
    pt.set_materials(sd.materials)
    pt.build()
    pt.set_geometry(sd.pos, sd.normals, sd.uvs, idx[:54], mids[:18])
    with pytest.raises(og.OhaoError) as e:
        pt.build()
    assert e.value.status == -1
    with pytest.raises(og.OhaoError) as e:
        pt.render([og.make_view(sd.views[0])], og.make_settings())
    assert e.value.status == -5
    pt.set_geometry(sd.pos, sd.normals, sd.uvs, idx, mids)
    pt.build()
    pt.close()


def test_full_size_sphere_properties(gpu_lib, oracle):
    """1,003,522-triangle scene: bit-exact BVH, hits on 100k rays, per-path
    radiance on a seeded pixel subset of a 1920x1080 frame."""
    sd = scenes.sphere_1m()
    pt = gpu_tracer(gpu_lib, sd)
    orc = oracle.OracleScene(sd)
    gn, gt, _ = pt.bvh()
    on, ot, _ = orc.bvh()
    assert np.array_equal(gn, on) and np.array_equal(gt, ot)
    rng = np.random.default_rng(9)
    rays = random_rays(rng, 100000, -1.6, 1.6)
    assert np.array_equal(trace_gpu(gpu_lib, pt, rays), orc.trace(rays, 0))
    v = sd.views[0]
    g, _, _ = render_paths_gpu(gpu_lib, pt, v, 1, dict(max_bounces=4, sampler=0))
    pix = np.sort(rng.choice(v.width * v.height, 4000, replace=False)).astype(np.uint32)
    o = orc.render_paths(v, dict(max_bounces=4, sampler=0), 0, 1, pixels=pix)
    assert_paths_match(g[:, pix], o, "sphere_1m subset")


@pytest.mark.parametrize("two_level", [False, True])
def test_persistent_multiview_matches_wavefront_and_oracle(gpu_lib, oracle, two_level):
    """The persistent multi-view kernel produces the same paths and
    accumulators as the per-view wavefront, bit for bit."""
    import torch
    og = gpu_lib
    if two_level:
        sd = small_instanced(side=20)
        fl = 1
        sd.views = [scenes.look_at_view(np.array([60.0, 10.0 * k, 40.0]), (0, 0, 0), width=16 + 4 * k, height=12 + 2 * k)
                    for k in range(5)]
    else:
        sd = small_env_scene(freq=12)
        fl = 0
        sd.views = [scenes.look_at_view((0.5 * k, 0.6, 3.2), (0, -0.1, 0), width=20 + 6 * k, height=14 + 3 * k)
                    for k in range(5)]
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    spp = 3
    outs = {}
    for mode in (og.MODE_WAVEFRONT, og.MODE_PERSISTENT):
        accs, paths, views = [], [], []
        for v in sd.views:
            npix = v.width * v.height
            a = torch.full((npix, 4), 7.0, dtype=torch.float32, device="cuda")
            p = torch.zeros((spp, npix, 4), dtype=torch.float32, device="cuda")
            accs.append(a)
            paths.append(p)
            views.append(og.make_view(v, accum=a, history=0, path_radiance=p))
        pt.render(views, og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=5, mode=mode))
        torch.cuda.synchronize()
        outs[mode] = ([a.cpu().numpy() for a in accs], [p.cpu().numpy()[:, :, :3] for p in paths])
    for k, v in enumerate(sd.views):
        assert np.array_equal(outs[og.MODE_WAVEFRONT][0][k], outs[og.MODE_PERSISTENT][0][k]), f"accum view {k}"
        assert np.array_equal(outs[og.MODE_WAVEFRONT][1][k], outs[og.MODE_PERSISTENT][1][k]), f"paths view {k}"
        o = orc.render_paths(v, dict(max_bounces=4, sampler=1), 5, spp)
        assert_paths_match(outs[og.MODE_PERSISTENT][1][k], o, f"persistent view {k}")
    # autotune picks a variant and renders stay identical
    views = [og.make_view(v, accum=torch.zeros((v.width * v.height, 4), device="cuda")) for v in sd.views]
    ms = pt.autotune(views, og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=5))
    assert ms > 0 and pt.launch_config != "default"
    accs = []
    views = []
    for v in sd.views:
        a = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
        accs.append(a)
        views.append(og.make_view(v, accum=a))
    pt.render(views, og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=5, mode=og.MODE_PERSISTENT))
    torch.cuda.synchronize()
    for k in range(len(sd.views)):
        assert np.array_equal(accs[k].cpu().numpy(), outs[og.MODE_WAVEFRONT][0][k])
    # every compiled launch shape (pool size, ray reordering, persistent-warp
    # traversal) gives the same accumulators and per-path radiance
    names = pt.launch_configs()
    assert len(names) >= 5 and any("fetch" in n for n in names)
    with pytest.raises(og.OhaoError):
        pt.launch_config = "no_such_shape"
    for name in names:
        pt.launch_config = name
        assert pt.launch_config == name
        accs, paths, views = [], [], []
        for v in sd.views:
            npix = v.width * v.height
            accs.append(torch.full((npix, 4), 7.0, dtype=torch.float32, device="cuda"))
            paths.append(torch.zeros((spp, npix, 4), dtype=torch.float32, device="cuda"))
            views.append(og.make_view(v, accum=accs[-1], history=0, path_radiance=paths[-1]))
        pt.render(views, og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=5,
                                          mode=og.MODE_PERSISTENT))
        torch.cuda.synchronize()
        for k in range(len(sd.views)):
            assert np.array_equal(accs[k].cpu().numpy(), outs[og.MODE_WAVEFRONT][0][k]), f"{name} accum view {k}"
            assert np.array_equal(paths[k].cpu().numpy()[:, :, :3], outs[og.MODE_WAVEFRONT][1][k]), \
                f"{name} paths view {k}"


@pytest.mark.parametrize("two_level", [False, True])
def test_degenerate_view_sizes(gpu_lib, oracle, two_level):
    """Views of 1x1, 3x2, 7x5, 9x4 and 1x37 pixels (no whole 8x4 work tile,
    or tiles plus ragged remainders) through the per-view wavefront and the
    persistent pool in every launch shape: per-path radiance against the
    oracle, accumulators bit-identical across forms."""
    import torch
    og = gpu_lib
    sd = small_instanced(side=8) if two_level else small_env_scene(freq=8)
    fl = 1 if two_level else 0
    sizes = [(1, 1), (3, 2), (7, 5), (9, 4), (1, 37)]
    sd.views = [scenes.look_at_view((0.0, 0.6, 3.2) if not two_level else (60.0, 10.0, 40.0),
                                    (0, -0.1, 0) if not two_level else (0, 0, 0), width=w, height=h)
                for w, h in sizes]
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    spp = 3
    ref = {}
    for k, v in enumerate(sd.views):
        g, acc, _ = render_paths_gpu(og, pt, v, spp, dict(max_bounces=4, sampler=1, sample_index_base=2))
        assert_paths_match(g, orc.render_paths(v, dict(max_bounces=4, sampler=1), 2, spp), f"view {sizes[k]}")
        ref[k] = acc.cpu().numpy()
    for name in pt.launch_configs():
        pt.launch_config = name
        accs = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in sd.views]
        pt.render([og.make_view(v, accum=a) for v, a in zip(sd.views, accs)],
                  og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=2, mode=og.MODE_PERSISTENT))
        torch.cuda.synchronize()
        for k in range(len(sd.views)):
            assert np.array_equal(accs[k].cpu().numpy(), ref[k]), f"{name} view {sizes[k]}"


@pytest.mark.parametrize("two_level", [False, True])
def test_traversal_shapes_and_material_sort_same_image(gpu_lib, two_level):
    """The per-view wavefront in every traversal shape (one ray per thread;
    persistent warps refilled at 1, 4 or 16 idle lanes), with the
    material-binned shading order and the ray-binned bounce order, and the
    persistent pool with the material binning: accumulators bit-identical,
    closest-hit visit counts identical."""
    import torch
    og = gpu_lib
    sd = small_instanced(side=24) if two_level else small_env_scene(freq=16)
    fl = 1 if two_level else 0
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    v = sd.views[0]
    ref, ref_counts = None, None
    for refill in (33, 1, 4, 16):
        for flags in (0, og.FLAG_SORT_MATERIAL, og.FLAG_SORT_RAYS, og.FLAG_SORT_MATERIAL | og.FLAG_SORT_RAYS):
            acc = torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda")
            pt.render([og.make_view(v, accum=acc)],
                      og.make_settings(spp=3, max_bounces=4, sampler=1, wavefront_refill=refill,
                                       flags=flags | og.FLAG_PROFILE, mode=og.MODE_WAVEFRONT))
            torch.cuda.synchronize()
            p = pt.profile()
            counts = (p.rays_closest, p.nodes_closest, p.tris_closest, p.rays_shadow)
            if ref is None:
                ref, ref_counts = acc.clone(), counts
            assert torch.equal(acc, ref), f"refill {refill} flags {flags}"
            assert counts == ref_counts, f"refill {refill} flags {flags}: {counts} != {ref_counts}"
    for name in ("pool_2M_sorted_chunk8", "pool_4M_unsorted_fetch4_chunk8"):
        pt.launch_config = name
        accs = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for _ in range(2)]
        pt.render([og.make_view(v, accum=a) for a in accs],
                  og.make_settings(spp=3, max_bounces=4, sampler=1, flags=og.FLAG_SORT_MATERIAL,
                                   mode=og.MODE_PERSISTENT))
        torch.cuda.synchronize()
        assert torch.equal(accs[0], ref) and torch.equal(accs[1], ref), name
