"""Seeded scenes and settings on which the oracle's integrator is compared
with the reference's own path-tracing shaders (raygen, closest hit, miss)
compiled as C++ (oracle/glsl_pin.py). The reference shades emission only
from emissive textures, so these scenes carry no slot-2 emission; light
comes from the environment, from analytic lights of all four GPULight types
and, in the textured scene, from an emissive texture. Its bindless diffuse,
normal, roughness-metal and emissive textures go through the reference's
closest-hit shader; the reference traces every ray opaque, so the alpha
test is pinned on its own (pt_anyhit.rahit, tests/test_oracle_pins.py)."""
from __future__ import annotations

import numpy as np

from ohao_engine_gb300 import scenes
from pt_harness import small_env_scene, small_instanced


def gpu_light(kind, pos, color, intensity, direction=(0.0, -1.0, 0.0), param=0.1, outer_deg=0.0):
    """One 80-byte GPULight record (gpu_light.hpp:10-16): sphere (0),
    directional (1) or spot (2)."""
    L = np.zeros(20, np.float32)
    L[0:3] = pos
    L[3] = kind
    L[4:7] = color
    L[7] = intensity
    L[8:11] = direction
    L[11] = param
    L[15] = outer_deg
    return L


def _cornell_lit(n_types: int):
    sd = scenes.cornell(24, 24, 1)
    sd.materials = sd.materials.copy()
    sd.materials[:, 9:12] = 0.0
    lights = [scenes.area_light((-0.12, 0.998, -0.1), (0.24, 0, 0), (0, 0, 0.2), 15.0)]
    if n_types > 1:
        lights += [gpu_light(0, (0.1, 0.8, 0.1), (1.0, 0.9, 0.8), 3.0, param=0.05),
                   gpu_light(1, (0, 0, 0), (0.9, 0.9, 1.0), 2.0, direction=(0.3, -1.0, 0.2)),
                   gpu_light(2, (-0.2, 0.95, 0.0), (1, 1, 1), 5.0, param=20.0, outer_deg=35.0)]
    sd.lights = np.stack(lights)
    return sd


def _env_lit(with_lights: bool):
    sd = small_env_scene(freq=16)
    if with_lights:
        sd.lights = _cornell_lit(4).lights
    return sd


def _instanced():
    sd = small_instanced()
    sd.materials = sd.materials.copy()
    sd.materials[:, 9:12] = 0.0
    return sd


def _bench_sphere():
    return scenes.sphere_1m()   # the default benchmark frame: 1,003,522 triangles, 1920x1080, sky + sun


# name -> (scene maker, oracle settings, flatten limit)
CASES = {
    "env_pcg": (lambda: _env_lit(False), dict(max_bounces=4, sampler=0), 1 << 25),
    "env_sobol_aniso": (lambda: _env_lit(False), dict(max_bounces=4, sampler=1, aniso=0.7, aniso_rot=0.5), 1 << 25),
    "env_firefly_depth2": (lambda: _env_lit(False), dict(max_bounces=2, sampler=0, flags=4, clamp_lum=2.0), 1 << 25),
    "env_depth0": (lambda: _env_lit(False), dict(max_bounces=0, sampler=1), 1 << 25),
    "env_lights_sobol": (lambda: _env_lit(True), dict(max_bounces=4, sampler=1), 1 << 25),
    "cornell_area_pcg": (lambda: _cornell_lit(1), dict(max_bounces=4, sampler=0), 1 << 25),
    "cornell_4_types_sobol": (lambda: _cornell_lit(4), dict(max_bounces=3, sampler=1), 1 << 25),
    "instanced_two_level": (_instanced, dict(max_bounces=4, sampler=0), 1000),
    "sphere_1m_1080p": (_bench_sphere, dict(max_bounces=4, sampler=0), 1 << 25),
    "textured_pcg": (lambda: scenes.textured(), dict(max_bounces=4, sampler=0), 1 << 25),
    "textured_sobol_two_level": (lambda: scenes.textured(), dict(max_bounces=3, sampler=1), 1),
}
LIVE_PIXELS = 4096   # live comparisons sample at most this many pixels of a view
SAMPLE_BASE, SPP = 3, 2
