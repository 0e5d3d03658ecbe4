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


def test_dual_gradient_matches_fd(oracle):
    """The oracle's analytic FP64 gradient (duals) equals central differences
    of its detached estimator, for roughness and map entries."""
    for sd, st in [(scenes.studio(freq=20, side=32), dict(max_bounces=3, sampler=0)),
                   (scenes.studio(freq=20, side=32), dict(max_bounces=3, sampler=1, aniso=0.6, aniso_rot=0.4)),
                   (scenes.cornell(24, 24), dict(max_bounces=4, sampler=0))]:
        o = oracle.OracleScene(sd)
        v = sd.views[0]
        rng = np.random.default_rng(3)
        dLdI = rng.normal(size=(v.width * v.height, 3))
        rough_ids = [k for k in range(sd.materials.shape[0]) if sd.materials[k, 4] > 0.04][:4]
        map_ids = [] if sd.albedo_map is None else list(rng.choice(sd.albedo_map.size, 12, replace=False))
        g = o.detached_grad(v, st, 0, 2, dLdI, rough_ids, map_ids, with_score=False)
        for j, (which, k) in enumerate([("rough", k) for k in rough_ids] + [("map", k) for k in map_ids]):
            mats = sd.materials.copy()
            amap = None if sd.albedo_map is None else sd.albedo_map.copy()
            hp = np.float32(1e-3)
            if which == "rough":
                mp, mm = mats.copy(), mats.copy()
                mp[k, 4] += hp
                mm[k, 4] -= hp
                step = float(mp[k, 4]) - float(mm[k, 4])
                Ip = o.detached_paths(v, st, 0, 2, materials=mp, albedo_map=amap).mean(axis=0)
                Im = o.detached_paths(v, st, 0, 2, materials=mm, albedo_map=amap).mean(axis=0)
            else:
                ap, am = amap.copy(), amap.copy()
                ap.reshape(-1)[k] += hp
                am.reshape(-1)[k] -= hp
                step = float(ap.reshape(-1)[k]) - float(am.reshape(-1)[k])
                Ip = o.detached_paths(v, st, 0, 2, materials=mats, albedo_map=ap).mean(axis=0)
                Im = o.detached_paths(v, st, 0, 2, materials=mats, albedo_map=am).mean(axis=0)
            fd = float((dLdI * (Ip - Im)).sum() / step)
            # the analytic gradient is exact; the difference is the O(h^2) error of the central difference
            assert abs(g[j] - fd) <= 1e-3 * max(abs(fd), 1e-3 * np.abs(g).max()), (sd.name, which, k, g[j], fd)


def _jitter_score(t, r):
    """d log q(w | r) / d r of the specular jitter, as the oracle and the
    device adjoint evaluate it (t = h.R of the cosine-distributed h)."""
    return (1 - t * t) / (t * (t + r) ** 2) + 2 / (t + r) - 2 / r


def test_jitter_score_is_a_score():
    """The jitter density q(w|r) = (s c - 1) s^2 / (pi r^2 sqrt(c^2 - 1 + r^2))
    integrates to the solid angle of its support, and its r-score has zero
    mean under it (both necessary for the score-function term)."""
    from scipy.integrate import quad
    for r in (0.04, 0.3, 0.9, 1.0, 2.5):
        val, _ = quad(lambda t: 2 * t * _jitter_score(t, r), 0, 1, limit=400)
        assert abs(val) < 1e-9, (r, val)
    rng = np.random.default_rng(0)
    R = np.array([0.3, 0.8, 0.2])
    R /= np.linalg.norm(R)
    up = np.array([0.0, 1.0, 0.0]) if abs(R[1]) < 0.999 else np.array([1.0, 0.0, 0.0])
    T = np.cross(up, R)
    T /= np.linalg.norm(T)
    B = np.cross(R, T)
    n = 400_000
    u0, u1 = rng.random(n), rng.random(n)
    rr = np.sqrt(u0)
    h = (T[:, None] * rr * np.cos(2 * np.pi * u1) + B[:, None] * rr * np.sin(2 * np.pi * u1)
         + R[:, None] * np.sqrt(1 - rr * rr))
    for r in (0.3, 0.7):
        w = R[:, None] + r * h
        w /= np.linalg.norm(w, axis=0)
        c = R @ w
        sq = np.sqrt(c * c - 1 + r * r)
        s = c + sq
        q = (s * c - 1) * s ** 2 / (np.pi * r ** 2 * sq)
        support = 2 * np.pi * (1 - 1 / np.sqrt(1 + r * r))
        assert abs(np.mean(1 / q) / support - 1) < 0.01, r
        # the closed form in t equals d log q / d r at fixed w (central difference)
        t = R @ h
        e = 1e-6
        def logq(rv):
            sqv = np.sqrt(c * c - 1 + rv * rv)
            sv = c + sqv
            return np.log((sv * c - 1) * sv ** 2 / (np.pi * rv ** 2 * sqv))
        fd = (logq(r + e) - logq(r - e)) / (2 * e)
        ok = t > 0.05
        assert np.allclose(fd[ok], _jitter_score(t, r)[ok], rtol=1e-4, atol=1e-4)
