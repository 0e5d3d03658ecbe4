"""The host oracle against the reference's own golden image.

``tests/golden/cornell_box.png`` in the reference is its offline path tracer's
output on the GPU (Vulkan ray tracing, driver traversal) for
``examples/cornell_box.cpp``: 1920x1080, 16 spp, Sobol sampler, depth 4,
denoiser off, samples 0..15 (19 frames with three in flight), tonemapped as
``pt_raygen_offline.rgen:1338-1354`` (ACES of half the radiance, gamma 1/2.2,
RGBA8) and downscaled to 640x360 with PIL's bilinear filter
(``tests/golden/render_golden.py:37-44``). ``scenes.cornell_example`` rebuilds
that scene as the engine uploads it; a band of output rows 100..139 of the
golden is stored in ``tests/golden/cornell_example_band.npz``
(``tests/golden/make_golden_image.py``).

What agrees: the oracle's image carries the golden's noise. Its high-pass
residual (image minus a 5x5 box blur) correlates at 0.88 with the golden's,
and at under 0.1 with the PCG sampler in place of Sobol or with the light
records in declaration order instead of the engine's upload order. So camera
rays, geometry, the Sobol streams and light selection follow the reference's
GPU render. What does not agree: radiance. The golden's 8-bit values are
about 0.7 times the oracle's (about 0.6 times in radiance), with a slight
colour shift, and no single scale of the light intensity brings the pixels
together (the closest leaves a mean difference of 3 LSB). The reference's
own shaders, compiled as C++ over the same scene, give the oracle's
radiance, not the golden's (within 3.2e-7 relative on 4,096 pixels x 4
samples; the last test here checks 1,024 pixels). The checkout has no
history to show which engine revision wrote the golden. Parity at this level
is therefore partial; the tolerance of ``tests/golden/manifest.json``
(max 4 LSB, at most 1% of pixels differing) is not met.
"""
import math
import os

import numpy as np
import pytest

from ohao_engine_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
BAND = np.load(os.path.join(HERE, "golden", "cornell_example_band.npz"))
OUT_W, OUT_H = 640, 360
TRIM = 3   # output rows at each band edge whose filter reaches outside the rendered rows


def tonemap_rgba8(acc):
    """pow(ACES(acc * 0.5), 1/2.2) stored to an RGBA8 UNORM image."""
    x = (acc * np.float32(0.5)).astype(np.float32)
    num = x * (np.float32(2.51) * x + np.float32(0.03))
    den = x * (np.float32(2.43) * x + np.float32(0.59)) + np.float32(0.14)
    a = np.clip(num / den, 0.0, 1.0).astype(np.float32)
    return np.clip(np.rint(np.power(a.astype(np.float64), 1.0 / 2.2) * 255.0), 0, 255).astype(np.uint8)


def _coeffs(in_size, out_size):
    """Pillow's resampling weights for the bilinear (triangle) filter: support
    scaled by the reduction factor, weights normalised, then fixed point with
    22 fraction bits (Pillow's libImaging/Resample.c, 8-bit path)."""
    scale = in_size / out_size
    fs = max(scale, 1.0)
    support = fs
    out = []
    for xx in range(out_size):
        center = (xx + 0.5) * scale
        xmin = max(int(center - support + 0.5), 0)
        n = min(int(center + support + 0.5), in_size) - xmin
        w = [max(0.0, 1.0 - abs((x + xmin - center + 0.5) / fs)) for x in range(n)]
        tot = sum(w)
        k = [int(0.5 + (v / tot) * (1 << 22)) for v in w]
        out.append((xmin, np.array(k, np.int64)))
    return out


def downscale(img, out_w, out_h):
    """Horizontal pass then vertical pass, each rounded and clipped to 8 bits."""
    h = img.shape[0]
    tmp = np.zeros((h, out_w, 3), np.int64)
    for xx, (xmin, k) in enumerate(_coeffs(img.shape[1], out_w)):
        s = (1 << 21) + np.tensordot(k, img[:, xmin:xmin + k.size].astype(np.int64).transpose(1, 0, 2), axes=1)
        tmp[:, xx] = np.clip(s >> 22, 0, 255)
    out = np.zeros((out_h, out_w, 3), np.int64)
    for yy, (ymin, k) in enumerate(_coeffs(h, out_h)):
        out[yy] = np.clip(((1 << 21) + np.tensordot(k, tmp[ymin:ymin + k.size], axes=1)) >> 22, 0, 255)
    return out.astype(np.uint8)


def render_band(oracle, sd, sampler, sample_base=0, spp=16):
    """The oracle's accumulated image over the full-resolution rows behind
    the stored band, tonemapped and downscaled like the golden."""
    v = sd.views[0]
    r0, r1 = (int(r) * v.height // OUT_H for r in BAND["rows"])
    pix = (np.arange(r0, r1)[:, None] * v.width + np.arange(v.width)[None, :]).reshape(-1).astype(np.uint32)
    scene = oracle.OracleScene(sd)
    paths = scene.render_paths(v, dict(max_bounces=4, sampler=sampler), sample_base, spp, pixels=pix)
    acc = oracle.accumulate(paths)[:, :3].reshape(r1 - r0, v.width, 3)
    return downscale(tonemap_rgba8(acc), OUT_W, (r1 - r0) * OUT_H // v.height)


def _highpass(img):
    a = img.astype(np.float64)
    k = np.ones(5) / 5.0
    b = np.apply_along_axis(lambda r: np.convolve(r, k, "same"), 1, a)
    b = np.apply_along_axis(lambda r: np.convolve(r, k, "same"), 0, b)
    return (a - b)[TRIM:-TRIM, TRIM:-TRIM]


def noise_correlation(ours, golden):
    return float(np.corrcoef(_highpass(ours[TRIM:-TRIM]).ravel(), _highpass(golden[TRIM:-TRIM]).ravel())[0, 1])


def test_cornell_example_scene_shape():
    sd = scenes.cornell_example()
    v = sd.views[0]
    assert (v.width, v.height) == (1920, 1080)
    assert sd.ntris == 5 * 2 + 2 * 32 * 16 * 2
    assert len(sd.blas) == 7 and sd.instances["custom_index"].tolist() == [0, 2, 4, 6, 8, 10, 1034]
    assert sd.lights.shape == (12, 20) and np.all(sd.lights[:, 3] == 0.0)
    # camera at (0, 0, 13) looking down -z, tan(19 degrees) vertically
    assert np.allclose(sd.views[0].inv_view[12:15], (0, 0, 13), atol=1e-6)
    assert math.isclose(float(sd.views[0].inv_proj[5]), math.tan(math.radians(19.0)), rel_tol=1e-6)


@pytest.fixture(scope="module")
def band_sobol(oracle):
    return render_band(oracle, scenes.cornell_example(), sampler=1)


def test_noise_matches_reference_golden(band_sobol):
    """Same sample streams, camera, geometry and light order as the
    reference's GPU render: the high-frequency noise lines up."""
    corr = noise_correlation(band_sobol, BAND["band"])
    assert corr >= 0.8, f"noise correlation with the golden {corr:.3f}"


def test_noise_correlation_discriminates(oracle, band_sobol):
    """Controls: the light records in declaration order, or the PCG sampler,
    give uncorrelated noise; the golden's radiance stays below the oracle's
    (the open difference the module docstring describes)."""
    declared = scenes.cornell_example(light_order=tuple(range(12)))
    assert noise_correlation(render_band(oracle, declared, sampler=1), BAND["band"]) < 0.3
    assert noise_correlation(render_band(oracle, scenes.cornell_example(), sampler=0), BAND["band"]) < 0.3
    ratio = BAND["band"].reshape(-1, 3).mean(axis=0) / band_sobol.reshape(-1, 3).mean(axis=0)
    assert np.all(ratio < 0.8), f"golden / oracle mean 8-bit value {ratio}"


def test_example_scene_radiance_equals_reference_shaders(oracle):
    """Where the reference tree exists: on this scene the reference's offline
    raygen, closest-hit and miss shaders compiled as C++ give the oracle's
    per-path radiance (within the 1e-6 relative that the offline raygen's
    regrouped light-sampling products allow), so the radiance gap to the
    golden image is not in the restatement of those shaders."""
    import glsl_pin
    lib = oracle.glsl_pt_lib("offline")
    if lib is None and glsl_pin.pt_available():
        glsl_pin.build_pt()
        lib = oracle.glsl_pt_lib("offline")
    if lib is None:
        pytest.skip("reference shaders not available here")
    sd = scenes.cornell_example()
    v = sd.views[0]
    scene = oracle.OracleScene(sd)
    pix = np.sort(np.random.default_rng(7).choice(v.width * v.height, 1024, replace=False)).astype(np.uint32)
    settings = dict(max_bounces=4, sampler=1)
    got = scene.render_paths(v, settings, 0, 2, pixels=pix)
    want = oracle.shader_paths(lib, scene, v, settings, 0, 2, pix)
    rel = np.abs(got - want) / np.maximum(np.maximum(np.abs(got), np.abs(want)), 1e-3)
    assert rel.max() <= 1e-6, f"oracle vs the reference's offline shaders: {rel.max():.3g} relative"
