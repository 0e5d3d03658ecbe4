"""The oracle's helper layer pinned against the reference's own code and tests.

* golden vectors in tests/golden/reference_kats.json were produced by the
  reference's compiled ohao/render/rt/{sobol_generator,owen_scramble,env_cdf}.cpp
  (tests/golden/make_golden.py);
* the known-answer tests of tests/renderer/sobol_test.cpp:10-111 and
  tests/renderer/env_cdf_test.cpp:9-61 restated as asserts;
* when the reference checkout is present, the compiled reference helpers are
  called directly as a third check.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))


def f32bits(x):
    return int(np.float32(x).view(np.uint32))


def test_sobol_matches_reference_golden(oracle):
    L = oracle.lib()
    for d in range(4):
        got = [f32bits(L.orc_sobol_sample1d(i, d)) for i in KATS["sobol_index"]]
        assert got == KATS["sobol_sample1d_bits"][str(d)], f"dim {d}"


def test_sobol_known_answers(oracle):
    """tests/renderer/sobol_test.cpp:10-66"""
    L = oracle.lib()
    dim2 = [0.0, 0.5, 0.25, 0.75, 0.875, 0.375, 0.625, 0.125]
    dim3 = [0.0, 0.5, 0.75, 0.25, 0.125, 0.625, 0.875, 0.375]
    jk = [(0.0, 0.0), (0.5, 0.5), (0.25, 0.75), (0.75, 0.25), (0.125, 0.625), (0.625, 0.125), (0.375, 0.375),
          (0.875, 0.875)]
    for i in range(8):
        assert abs(L.orc_sobol_sample1d(i, 2) - dim2[i]) < 1e-5
        assert abs(L.orc_sobol_sample1d(i, 3) - dim3[i]) < 1e-5
        assert abs(L.orc_sobol_sample1d(i, 0) - jk[i][0]) < 1e-5
        assert abs(L.orc_sobol_sample1d(i, 1) - jk[i][1]) < 1e-5
    for d in range(4):
        for i in range(128):
            v = L.orc_sobol_sample1d(i, d)
            assert 0.0 <= v < 1.0
    v = L.orc_sobol_sample1d(2**31, 1)
    assert 0.0 <= v < 1.0


def test_owen_matches_reference_golden(oracle):
    L = oracle.lib()
    got = [L.orc_owen_scramble(v, s) for v, s in zip(KATS["owen_v"], KATS["owen_seed"])]
    assert got == KATS["owen_out"]


def test_owen_properties(oracle):
    """tests/renderer/sobol_test.cpp:75-111"""
    L = oracle.lib()
    assert L.orc_owen_scramble(0xABCD1234, 0xDEADBEEF) == L.orc_owen_scramble(0xABCD1234, 0xDEADBEEF)
    assert L.orc_owen_scramble(0x01234567, 1) != L.orc_owen_scramble(0x01234567, 2)
    assert 0 <= L.orc_owen_scramble(0, 0xCAFEBABE) <= 0xFFFFFFFF
    total = 0
    for i in range(1, 1001):
        v = (i * 0x9E3779B9) & 0xFFFFFFFF
        total += bin(L.orc_owen_scramble(v, 1) ^ L.orc_owen_scramble(v, 2)).count("1")
    assert 12000 < total < 20000


@pytest.mark.parametrize("name", sorted(KATS["env_cdf"].keys()))
def test_env_cdf_matches_reference_golden(oracle, name):
    g = KATS["env_cdf"][name]
    w, h = g["w"], g["h"]
    px = np.array(g["pixels_bits"], np.uint32).view(np.float32).reshape(h, w, 4)
    marg, cond, integ = oracle.env_cdf(px)
    assert marg.view(np.uint32).tolist() == g["marg_bits"]
    assert cond.view(np.uint32).tolist() == g["cond_bits"]
    assert f32bits(integ) == g["integral_bits"]


def test_env_cdf_known_answers(oracle):
    """tests/renderer/env_cdf_test.cpp:9-61"""
    marg, cond, integ = oracle.env_cdf(np.ones((16, 32, 4), np.float32))
    assert integ > 0
    assert abs(marg[-1] - 1.0) < 1e-4 and np.all(np.diff(marg) >= 0)
    c = cond.reshape(16, 32)
    assert np.all(np.abs(c[:, -1] - 1.0) < 1e-4) and np.all(np.diff(c, axis=1) >= 0)
    px = np.full((8, 16, 4), 0.01, np.float32)
    px[4, 10, :3] = 100.0
    marg, cond, _ = oracle.env_cdf(px)
    c = cond.reshape(8, 16)
    assert c[4, 10] - c[4, 9] > 0.5
    assert marg[4] - marg[3] > 0.5


def test_reference_helpers_live(oracle):
    """Direct comparison with the compiled reference helpers (reference checkout only)."""
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("reference helpers not built here (no reference checkout)")
    L = oracle.lib()
    rng = np.random.default_rng(3)
    for _ in range(2000):
        i = int(rng.integers(0, 2**32))
        d = int(rng.integers(0, 4))
        assert f32bits(L.orc_sobol_sample1d(i, d)) == f32bits(R.ref_sobol_sample1d(i, d))
    env = rng.uniform(0, 3, (32, 64, 4)).astype(np.float32)
    m1, c1, i1 = oracle.env_cdf(env)
    m2 = np.zeros(32, np.float32)
    c2 = np.zeros(64 * 32, np.float32)
    i2 = np.zeros(1, np.float32)
    R.ref_env_cdf_build(env.ctypes.data, 64, 32, m2.ctypes.data, c2.ctypes.data, i2.ctypes.data)
    assert np.array_equal(m1.view(np.uint32), m2.view(np.uint32))
    assert np.array_equal(c1.view(np.uint32), c2.view(np.uint32))
    assert f32bits(i1) == f32bits(i2[0])


def test_sobol_table_matches_reference_golden():
    """The library's direction-number table equals the reference's table."""
    import re
    src = open(os.path.join(os.path.dirname(HERE), "ohao_engine_gb300", "csrc", "pt_path.cuh")).read()
    body = src[src.index("c_sobol_dirs[128] = {"):]
    body = body[:body.index("};")]
    vals = [int(x, 16) for x in re.findall(r"0x([0-9A-Fa-f]{8})u", body)]
    assert vals == KATS["sobol_dirs"]


# ---- the reference's GLSL helper includes, compiled as C++ (oracle/glsl_pin.py) ----
GLSL_KATS = json.load(open(os.path.join(HERE, "golden", "glsl_kats.json")))


def _u32(a):
    return np.asarray(a, np.uint32)


def test_glsl_helpers_match_reference_golden(oracle):
    """The oracle's PCG stream, balance heuristic, GGX D (isotropic and
    anisotropic), Smith terms, VNDF sampling and metal-rough unpack, and its
    environment-CDF search, sampling and pdf reproduce the reference shader
    includes bit for bit on the recorded inputs."""
    import glsl_pin
    L = oracle.lib()
    for name, rec in GLSL_KATS["helpers"].items():
        nin, nout = glsl_pin.HELPER_IO[rec["fn"]]
        x = _u32(rec["in_bits"]).view(np.float32).reshape(-1, nin)
        got = oracle.glsl_eval(L, "orc_glsl_", rec["fn"], x, nout)
        assert np.array_equal(got.view(np.uint32).reshape(-1), _u32(rec["out_bits"])), name
    e = GLSL_KATS["env_cdf"]
    env = (_u32(e["marg_bits"]).view(np.float32), _u32(e["cond_bits"]).view(np.float32), e["w"], e["h"])
    for name, rec in GLSL_KATS["env"].items():
        nin, nout = glsl_pin.ENV_IO[rec["fn"]]
        x = _u32(rec["in_bits"]).view(np.float32).reshape(-1, nin)
        got = oracle.glsl_eval(L, "orc_glsl_", rec["fn"], x, nout, env=env)
        assert np.array_equal(got.view(np.uint32).reshape(-1), _u32(rec["out_bits"])), name


def test_glsl_golden_exercises_every_branch():
    """The recorded inputs reach both GGX D branches and both unpack
    branches, and the outputs are not degenerate."""
    h = GLSL_KATS["helpers"]
    x = _u32(h["ggx_d_aniso_or_iso"]["in_bits"]).view(np.float32).reshape(-1, 10)
    assert (x[:, 8] < 0.001).any() and (x[:, 8] >= 0.001).any()
    x = _u32(h["unpack_hit_pbr"]["in_bits"]).view(np.float32).reshape(-1, 3)
    assert ((x[:, 0] < 0) & (x[:, 1] < 1e-4)).any() and (x[:, 0] >= 0).any()
    for rec in list(h.values()) + list(GLSL_KATS["env"].values()):
        y = _u32(rec["out_bits"]).view(np.float32)
        assert np.isfinite(y).all() and len(np.unique(y)) > 8


def test_glsl_helpers_live(oracle):
    """20,000 seeded records per function against the shader includes
    compiled from the reference tree (reference checkout only)."""
    import glsl_pin
    G = oracle.glsl_lib()
    if G is None and glsl_pin.available():
        glsl_pin.build()
        G = oracle.glsl_lib()
    if G is None:
        pytest.skip("reference shader includes not available here")
    L = oracle.lib()
    rng = np.random.default_rng(99)
    n = 20000
    for fn, (nin, nout) in glsl_pin.HELPER_IO.items():
        x = glsl_pin.helper_records(fn, n, rng)
        a = oracle.glsl_eval(L, "orc_glsl_", fn, x, nout)
        b = oracle.glsl_eval(G, "gref_", fn, x, nout)
        bad = (a.view(np.uint32) != b.view(np.uint32)).any(1)
        assert not bad.any(), f"{glsl_pin.HELPER_NAMES[fn]}: {bad.sum()} records differ, first {x[bad][0]}"
    envmap = rng.uniform(0, 4, (64, 128, 4)).astype(np.float32)
    envmap[10:12] = 0.0
    m, c, _ = oracle.env_cdf(envmap)
    for fn, (nin, nout) in glsl_pin.ENV_IO.items():
        x = glsl_pin.env_records(fn, n, rng, 128, 64)
        a = oracle.glsl_eval(L, "orc_glsl_", fn, x, nout, env=(m, c, 128, 64))
        b = oracle.glsl_eval(G, "gref_", fn, x, nout, env=(m, c, 128, 64))
        bad = (a.view(np.uint32) != b.view(np.uint32)).any(1)
        assert not bad.any(), f"{glsl_pin.ENV_NAMES[fn]}: {bad.sum()} records differ"


# ---- the integrator against the reference's raygen / closest-hit / miss shaders ----
def test_integrator_matches_reference_shaders_golden(oracle):
    """Per-path radiance of the oracle's integrator equals, bit for bit, the
    recorded output of the reference's own path-tracing shaders compiled as
    C++ and traced through the oracle's BVH, on every pin scene: env-lit with
    PCG and Sobol, anisotropic GGX, the firefly clamp, depth 0 and 2, all four
    analytic light types, two-level instancing with rotated, scaled
    instances, and the default benchmark frame (1M triangles, 1080p)."""
    import pin_cases
    assert set(GLSL_KATS["paths"]) == set(pin_cases.CASES)
    for name, (make, settings, flatten_limit) in pin_cases.CASES.items():
        rec = GLSL_KATS["paths"][name]
        sd = make()
        scene = oracle.OracleScene(sd, flatten_limit=flatten_limit)
        got = scene.render_paths(sd.views[0], settings, pin_cases.SAMPLE_BASE, pin_cases.SPP, pixels=rec["pixels"])
        want = _u32(rec["out_bits"]).view(np.float32).reshape(got.shape)
        assert np.isfinite(want).all() and np.abs(want).max() > 0, name
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
            f"{name}: {(got != want).any(-1).sum()} paths differ from the reference shaders"


def test_integrator_matches_reference_shaders_live(oracle):
    """Whole views of every pin scene against the shaders compiled from the
    reference tree (reference checkout only)."""
    import glsl_pin
    import pin_cases
    P = oracle.glsl_pt_lib()
    if P is None and glsl_pin.pt_available():
        glsl_pin.build_pt()
        P = oracle.glsl_pt_lib()
    if P is None:
        pytest.skip("reference shaders not available here")
    for name, (make, settings, flatten_limit) in pin_cases.CASES.items():
        sd = make()
        scene = oracle.OracleScene(sd, flatten_limit=flatten_limit)
        for v in sd.views[:2]:
            pix = _live_pixels(v)
            a = scene.render_paths(v, settings, 0, 2, pixels=pix)
            b = oracle.shader_paths(P, scene, v, settings, 0, 2, pix)
            bad = (a.view(np.uint32) != b.view(np.uint32)).any(-1)
            assert not bad.any(), f"{name}: {bad.sum()} of {bad.size} paths differ from the reference shaders"


def test_alpha_test_matches_reference_anyhit_golden(oracle):
    """The oracle's alpha test (and so the kernels', which equal it on the
    GPU) against the recorded decisions of the reference's any-hit shader
    (pt_anyhit.rahit compiled as C++) on candidate hits of the textured pin
    scene; some hits are ignored, some accepted."""
    import pin_cases
    rec = GLSL_KATS["anyhit"]
    inst, prim = _u32(rec["inst"]), _u32(rec["prim"])
    uv = _u32(rec["uv_bits"]).view(np.float32).reshape(-1, 2)
    scene = oracle.OracleScene(pin_cases.CASES["textured_pcg"][0]())
    got = scene.alpha_accept(inst, prim, uv)
    want = np.asarray(rec["accept"], np.uint32)
    assert np.array_equal(got, want)
    leaves = inst == 1
    assert 0.1 < want[leaves].mean() < 0.9 and want[~leaves].all()


def test_alpha_test_matches_reference_anyhit_live(oracle):
    import glsl_pin
    import pin_cases
    P = oracle.glsl_pt_lib()
    if P is None and glsl_pin.pt_available():
        glsl_pin.build_pt()
        P = oracle.glsl_pt_lib()
    if P is None:
        pytest.skip("reference shaders not available here")
    scene = oracle.OracleScene(pin_cases.CASES["textured_pcg"][0]())
    rng = np.random.default_rng(5)
    n = 50000
    inst = np.ones(n, np.uint32)
    prim = rng.integers(0, 10, n).astype(np.uint32)
    uv = rng.random((n, 2))
    flip = uv.sum(1) > 1.0
    uv[flip] = 1.0 - uv[flip]
    uv = uv.astype(np.float32)
    assert np.array_equal(scene.alpha_accept(inst, prim, uv), oracle.shader_anyhit(P, scene, inst, prim, uv))


def _live_pixels(v):
    import pin_cases
    n = v.width * v.height
    if n <= pin_cases.LIVE_PIXELS:
        return None
    return np.sort(np.random.default_rng(n).choice(n, pin_cases.LIVE_PIXELS, replace=False)).astype(np.uint32)


OFFLINE_RTOL = 1e-6   # the offline raygen regroups the analytic-light NEE products


def _offline_check(name, sd, got, want):
    if sd.lights.shape[0] == 0:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{name}: offline raygen, no lights"
    else:
        rel = np.abs(got - want) / np.maximum(np.maximum(np.abs(got), np.abs(want)), 1e-3)
        assert rel.max() <= OFFLINE_RTOL, f"{name}: offline raygen differs by {rel.max():.3g} relative"


def test_integrator_within_offline_raygen_golden(oracle):
    """Against the offline profile's raygen (pt_raygen_offline.rgen, the
    subsurface terms off): bit-identical without analytic lights, within
    1e-6 relative with them (its light NEE multiplies the same factors in
    another grouping)."""
    import pin_cases
    for name, (make, settings, flatten_limit) in pin_cases.CASES.items():
        rec = GLSL_KATS["paths_offline"][name]
        sd = make()
        scene = oracle.OracleScene(sd, flatten_limit=flatten_limit)
        got = scene.render_paths(sd.views[0], settings, pin_cases.SAMPLE_BASE, pin_cases.SPP, pixels=rec["pixels"])
        _offline_check(name, sd, got, _u32(rec["out_bits"]).view(np.float32).reshape(got.shape))


def test_integrator_within_offline_raygen_live(oracle):
    import glsl_pin
    import pin_cases
    P = oracle.glsl_pt_lib("offline")
    if P is None and glsl_pin.pt_available():
        glsl_pin.build_pt()
        P = oracle.glsl_pt_lib("offline")
    if P is None:
        pytest.skip("reference shaders not available here")
    for name, (make, settings, flatten_limit) in pin_cases.CASES.items():
        sd = make()
        scene = oracle.OracleScene(sd, flatten_limit=flatten_limit)
        v = sd.views[0]
        pix = _live_pixels(v)
        _offline_check(name, sd, scene.render_paths(v, settings, 0, 2, pixels=pix),
                       oracle.shader_paths(P, scene, v, settings, 0, 2, pix))
