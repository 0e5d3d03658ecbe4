"""Emitter MIS (OHAO_PT_FLAG_EMITTER_MIS) on the GPU against the oracle:
emissive triangles as a light-NEE choice, sphere and area lights found by
BSDF rays, balance-heuristic weights on both sides. Per path within 1e-4
relative (FP32 oracle), accumulation bit-exact; flat and two-level, the
per-view wavefront and the persistent pool, plain and textured emission
(with the alpha test), and the emissive table rebuilt after a material
update."""
import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pt_harness import emitter_scene, gpu_tracer, rel_err, render_paths_gpu

pytestmark = pytest.mark.gpu

RTOL = 1e-4
EMITTER_MIS = 1 << 13
ALPHA = 1 << 10


def assert_paths_match(gpu, ref, what):
    assert gpu.shape == ref.shape
    assert np.isfinite(gpu).all(), what
    err = rel_err(gpu, ref, floor=1e-3)
    bad = np.argwhere(err > RTOL)
    assert bad.size == 0, f"{what}: {len(bad)} components beyond {RTOL} (first {bad[:5].tolist()})"


def _compare(og, oracle, sd, fl, flags, sampler=0, mode=0, spp=4, base=2):
    pt = gpu_tracer(og, sd, flatten_limit=fl)
    assert pt.two_level == (fl == 1)
    orc = oracle.OracleScene(sd, flatten_limit=fl if fl else 1 << 25)
    v = sd.views[0]
    g, acc, _ = render_paths_gpu(og, pt, v, spp, dict(max_bounces=4, sampler=sampler, flags=flags,
                                                      sample_index_base=base, mode=mode))
    o = orc.render_paths(v, dict(max_bounces=4, sampler=sampler, flags=flags), base, spp)
    assert_paths_match(g, o, f"{sd.name} fl={fl} flags={flags:#x} mode={mode}")
    assert np.array_equal(acc.cpu().numpy(), oracle.accumulate(o))
    return g, o


@pytest.mark.parametrize("two_level", [False, True])
@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("sampler", [0, 1])
def test_emitter_scene_paths(gpu_lib, oracle, two_level, mode, sampler):
    """Emissive quads and an instanced emissive triangle (masked and
    non-opaque copies left out of the table), an area and a sphere light,
    an environment; wavefront (mode 1) and pool (mode 2)."""
    sd = emitter_scene(env=True)
    g, o = _compare(gpu_lib, oracle, sd, 1 if two_level else 0, EMITTER_MIS, sampler=sampler, mode=mode)
    plain = oracle.OracleScene(sd, flatten_limit=1 if two_level else 1 << 25).render_paths(
        sd.views[0], dict(max_bounces=4, sampler=sampler), 2, 4)
    assert not np.array_equal(o, plain), "the flag changes the estimator on this scene"


def test_emitters_without_lights(gpu_lib, oracle):
    """No GPULights at all: the light NEE runs for the emissive triangles
    alone (the reference would skip it)."""
    _compare(gpu_lib, oracle, emitter_scene(lights=()), 0, EMITTER_MIS, sampler=1)


@pytest.mark.parametrize("alpha", [False, True])
def test_textured_emission(gpu_lib, oracle, alpha):
    """Emissive texture panel (sRGB-decoded at the sampled point), sphere
    light, environment, alpha-tested leaves."""
    flags = EMITTER_MIS | (ALPHA if alpha else 0)
    _compare(gpu_lib, oracle, scenes.textured(), 0, flags, sampler=1)


def test_cornell_area_light_and_quad(gpu_lib, oracle):
    """Area light under the emissive ceiling quad: both reached by NEE and by
    BSDF rays."""
    _compare(gpu_lib, oracle, scenes.cornell(24, 24, 1), 0, EMITTER_MIS)


def test_table_follows_material_updates(gpu_lib, oracle):
    """Emission changed with update_materials after a render: the next
    render samples by the new power (and a material without emission
    leaves the table)."""
    og = gpu_lib
    sd = emitter_scene()
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    kw = dict(max_bounces=3, sampler=1, flags=EMITTER_MIS, sample_index_base=0)
    render_paths_gpu(og, pt, v, 1, kw)
    mats = sd.materials.copy()
    mats[2, 9:12] = (2.0, 60.0, 1.0)
    mats[3, 9:12] = 0.0
    pt.update_materials(mats)
    g, _, _ = render_paths_gpu(og, pt, v, 2, kw)
    sd.materials = mats
    o = oracle.OracleScene(sd).render_paths(v, dict(max_bounces=3, sampler=1, flags=EMITTER_MIS), 0, 2)
    assert_paths_match(g, o, "after update_materials")


def test_adjoint_rejects_the_flag(gpu_lib):
    import torch
    og = gpu_lib
    sd = emitter_scene(width=8, height=8)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    acc = torch.zeros((64, 4), device="cuda")
    tgt = torch.zeros((64, 4), device="cuda")
    s = og.make_settings(spp=1, max_bounces=2, flags=EMITTER_MIS)
    with pytest.raises(Exception, match="EMITTER_MIS"):
        pt.adjoint([og.make_view(v, accum=acc)], s, [tgt])
