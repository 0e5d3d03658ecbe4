"""The detached-sampling FP64 estimator of the oracle (the reference for the
path-replay gradient): at theta_e == theta_s it is the forward estimator, and
it is smooth in theta_e so that central differences are a valid gradient."""
import numpy as np
import pytest

import pt_harness as H
from ohao_engine_gb300 import scenes

CASES = [
    ("studio", lambda: scenes.studio(freq=20, side=40), dict(max_bounces=3, sampler=0)),
    ("studio_sobol_aniso", lambda: scenes.studio(freq=20, side=40), dict(max_bounces=3, sampler=1, aniso=0.6,
                                                                        aniso_rot=0.4)),
    ("small_env", lambda: H.small_env_scene(), dict(max_bounces=4, sampler=0)),
    ("cornell", lambda: scenes.cornell(32, 32), dict(max_bounces=4, sampler=1)),
]


@pytest.mark.parametrize("name,make,st", CASES, ids=[c[0] for c in CASES])
def test_detached_equals_forward(oracle, name, make, st):
    sd = make()
    o = oracle.OracleScene(sd)
    fwd = o.render_paths(sd.views[0], st, 0, 2, None, fp64=False).astype(np.float64)
    det = o.detached_paths(sd.views[0], st, 0, 2)
    assert det.shape == fwd.shape
    err = np.abs(det - fwd) / np.maximum(np.abs(det), 1e-2)
    assert err.max() < 2e-5, (name, err.max())
    assert det.mean() > 0.01


def _fd(o, sd, st, spp, mats=None, amap=None, which="rough", k=0, h=1e-3):
    """Central difference of the summed image in one parameter (float32 steps)."""
    mats = sd.materials.copy() if mats is None else mats
    amap = None if sd.albedo_map is None else (sd.albedo_map.copy() if amap is None else amap)
    if which == "rough":
        mp, mm = mats.copy(), mats.copy()
        mp[k, 4] += np.float32(h)
        mm[k, 4] -= np.float32(h)
        step = float(mp[k, 4]) - float(mm[k, 4])
        fp = o.detached_paths(sd.views[0], st, 0, spp, materials=mp, albedo_map=amap).sum()
        fm = o.detached_paths(sd.views[0], st, 0, spp, materials=mm, albedo_map=amap).sum()
    else:
        ap, am = amap.copy(), amap.copy()
        ap.reshape(-1)[k] += np.float32(h)
        am.reshape(-1)[k] -= np.float32(h)
        step = float(ap.reshape(-1)[k]) - float(am.reshape(-1)[k])
        fp = o.detached_paths(sd.views[0], st, 0, spp, materials=mats, albedo_map=ap).sum()
        fm = o.detached_paths(sd.views[0], st, 0, spp, materials=mats, albedo_map=am).sum()
    return (fp - fm) / step


def test_detached_is_smooth(oracle):
    """Halving the step changes the central difference by O(h^2) only."""
    sd = scenes.studio(freq=20, side=40)
    st = dict(max_bounces=3, sampler=0)
    o = oracle.OracleScene(sd)
    for which, k in [("rough", 0), ("rough", 2), ("map", 3 * (20 * 64 + 30)), ("map", 3 * (40 * 64 + 10) + 1)]:
        g1 = _fd(o, sd, st, 2, which=which, k=k, h=2e-3)
        g2 = _fd(o, sd, st, 2, which=which, k=k, h=1e-3)
        assert abs(g1 - g2) <= 2e-3 * max(abs(g2), 1e-3), (which, k, g1, g2)
