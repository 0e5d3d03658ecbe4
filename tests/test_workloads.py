"""The synthetic workloads the benchmark and the GPU tests run on: seeded,
reproducible, of the stated sizes, and valid input for the C ABI (indices,
material ids, instance ranges and texture slots that ohao_pt_set_* and
ohao_pt_build accept). Host only."""
import math

import numpy as np
import pytest

from ohao_engine_gb300 import scenes


def _mat(a):
    """Column-major float[16] -> 4x4."""
    return np.asarray(a, np.float64).reshape(4, 4).T


def center_ray(view):
    """Direction of the ray through the centre of the image (NDC 0, 0)."""
    p = _mat(view.inv_proj) @ np.array([0.0, 0.0, 1.0, 1.0])
    d = p[:3] / np.linalg.norm(p[:3])
    w = _mat(view.inv_view) @ np.array([d[0], d[1], d[2], 0.0])
    return _mat(view.inv_view)[:3, 3], w[:3] / np.linalg.norm(w[:3])


def check_abi_valid(sd):
    nverts = sd.pos.shape[0]
    assert sd.indices.dtype == np.uint32 and sd.indices.size % 3 == 0
    assert int(sd.indices.max()) < nverts
    assert sd.mat_ids.size == sd.ntris and int(sd.mat_ids.max()) < sd.materials.shape[0]
    assert sd.normals.shape == (nverts, 4) and sd.uvs.shape == (nverts, 2)
    assert np.isfinite(sd.pos).all() and np.isfinite(sd.normals).all()
    for fi, ic in sd.blas:
        assert ic % 3 == 0 and fi + ic <= sd.indices.size
    for inst in sd.instances:
        fi, ic = sd.blas[inst["blas"]]
        assert inst["custom_index"] + ic // 3 <= sd.ntris
        x = inst["xform"].reshape(3, 4).astype(np.float64)
        assert abs(np.linalg.det(x[:, :3])) > 1e-3
    tex = sd.materials.view(np.uint32)
    assert np.all(tex[:, 6:9] == scenes.NO_TEX)
    assert np.all((tex[:, 3] == scenes.NO_TEX) | (tex[:, 3] == 0))


def fingerprint(sd):
    h = [sd.pos.tobytes(), sd.indices.tobytes(), sd.mat_ids.tobytes(), sd.materials.tobytes(),
         sd.instances.tobytes()]
    h += [v.inv_view.tobytes() + v.inv_proj.tobytes() for v in sd.views]
    if sd.env is not None:
        h.append(sd.env.tobytes())
    return hash(b"".join(h))


def test_sphere_1m_workload():
    sd = scenes.sphere_1m()
    assert sd.ntris == 20 * 224 ** 2 + 2 == 1_003_522
    v = sd.views[0]
    assert (v.width, v.height) == (1920, 1080) and len(sd.views) == 1
    assert sd.env.shape == (512, 1024, 4) and (sd.spp, sd.max_bounces) == (1, 4)
    check_abi_valid(sd)
    # per-triangle GGX materials as stated: albedo U[0.1, 0.9], roughness U[0.05, 1]
    m = sd.materials[:-1]
    assert m[:, 0:3].min() >= 0.1 and m[:, 0:3].max() <= 0.9
    eye, d = center_ray(v)
    want = np.array([0.0, -0.1, 0.0]) - eye
    assert np.allclose(eye, [0.0, 0.6, 3.2], atol=1e-6)
    assert np.dot(d, want / np.linalg.norm(want)) > 1 - 1e-9
    assert fingerprint(sd) == fingerprint(scenes.sphere_1m())


def test_instanced_workload():
    sd = scenes.instanced()
    assert len(sd.blas) == 5 and sd.instances.size == 10_000
    assert sd.ntris == 20 * sum(f * f for f in (10, 22, 50, 71, 100)) == 362_500
    assert len(sd.views) == 64 and sd.spp == 4
    sides = [v.width for v in sd.views]
    assert all(v.width == v.height for v in sd.views) and 256 <= min(sides) and max(sides) <= 1024
    assert sum(v.width * v.height for v in sd.views) == 22_080_035
    check_abi_valid(sd)
    # scales U[0.5, 2] of a rotation: |det| in [1/8, 8]
    dets = [abs(np.linalg.det(i["xform"].reshape(3, 4)[:, :3].astype(np.float64))) for i in sd.instances]
    assert 0.125 - 1e-4 <= min(dets) and max(dets) <= 8 + 1e-3
    assert fingerprint(sd) == fingerprint(scenes.instanced())


def test_studio_workload():
    sd = scenes.studio()
    assert sd.ntris == 20 * 100 ** 2 + 2
    assert len(sd.views) == 10 and all((v.width, v.height) == (512, 512) for v in sd.views)
    assert sd.albedo_map.shape == (64, 64, 3) and sd.materials.shape == (5, 12)
    check_abi_valid(sd)
    tex = sd.materials.view(np.uint32)[:, 3]
    assert list(tex[:4]) == [0, 0, 0, 0] and tex[4] == scenes.NO_TEX   # map on the sphere regions only
    rough = [sd.materials[k, 4] for k in range(4)]
    assert np.allclose(rough, (0.3, 0.5, 0.7, 0.9))
    for v in sd.views:
        eye, d = center_ray(v)
        want = np.array([0.0, -0.1, 0.0]) - eye
        assert np.dot(d, want / np.linalg.norm(want)) > 1 - 1e-9


def test_cornell_workload():
    sd = scenes.cornell(64, 48, 2)
    assert sd.ntris == 36 and (sd.views[0].width, sd.views[0].height) == (64, 48)
    check_abi_valid(sd)


@pytest.mark.parametrize("size", [(1024, 512), (256, 128)])
def test_sky_env_cdf_valid(oracle, size):
    env = scenes.sky_env(size[0], size[1], seed=1)
    assert env.shape == (size[1], size[0], 4) and np.isfinite(env).all() and env.min() >= 0
    m, c, integral = oracle.env_cdf(env)
    assert integral > 0 and math.isfinite(integral)
    assert np.all(np.diff(m) >= 0) and m[-1] == pytest.approx(1.0, abs=1e-6)
    c = c.reshape(size[1], size[0])
    assert np.all(np.diff(c, axis=1) >= 0) and np.allclose(c[:, -1], 1.0, atol=1e-5)
