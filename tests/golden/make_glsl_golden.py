"""Regenerate tests/golden/glsl_kats.json from the reference's own shader text.

Compiles the reference's GLSL helper includes as C++ where they lie in the
reference tree (oracle/glsl_pin.py) and records their outputs on seeded
inputs: 64 records per helper, the environment-CDF functions over the CDFs
of a seeded 32x16 map, and the per-path radiance of the raygen, closest-hit
and miss shaders (traced through the oracle's BVH) on the seeded scenes of
tests/pin_cases.py, 96 pixels of the first view each, and the any-hit
shader's accept / ignore decision on 2,048 seeded candidate hits of the
textured scene. Run in a container
that has the reference checkout:

    python tests/golden/make_glsl_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import glsl_pin  # noqa: E402
import pyoracle  # noqa: E402

N = 64
ENV_W, ENV_H = 32, 16


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32).reshape(-1).tolist()


def anyhit_candidates(n=2048, seed=77):
    """Seeded candidate hits (instance, primitive, barycentrics) of the
    textured pin scene: three quarters on the alpha-tested leaves (instance
    1, 10 triangles), the rest on the opaque geometry (instance 0)."""
    rng = np.random.default_rng(seed)
    inst = (rng.random(n) < 0.75).astype(np.uint32)
    prim = np.where(inst == 1, rng.integers(0, 10, n), rng.integers(0, 2884, n)).astype(np.uint32)
    uv = rng.random((n, 2))
    flip = uv.sum(1) > 1.0
    uv[flip] = 1.0 - uv[flip]
    return inst, prim, np.ascontiguousarray(uv, np.float32)


def main():
    pyoracle.build(ref=True)
    G = pyoracle.glsl_lib()
    assert G is not None, "GLSL helpers not built (needs the reference checkout)"
    rng = np.random.default_rng(2024)
    out = {"generator": "tests/golden/make_glsl_golden.py",
           "source": "reference shader includes " + ", ".join(glsl_pin.GLSL_FILES) + ", compiled as C++",
           "helpers": {}, "env": {}}
    for fn, (nin, nout) in glsl_pin.HELPER_IO.items():
        x = glsl_pin.helper_records(fn, N, rng)
        y = pyoracle.glsl_eval(G, "gref_", fn, x, nout)
        out["helpers"][glsl_pin.HELPER_NAMES[fn]] = {"fn": fn, "in_bits": bits(x), "out_bits": bits(y)}
    env = rng.uniform(0, 4, (ENV_H, ENV_W, 4)).astype(np.float32)
    env[3] = 0.0
    env[9, 20, :3] = 200.0
    marg, cond, _ = pyoracle.env_cdf(env)
    out["env_cdf"] = {"w": ENV_W, "h": ENV_H, "marg_bits": bits(marg), "cond_bits": bits(cond)}
    for fn, (nin, nout) in glsl_pin.ENV_IO.items():
        x = glsl_pin.env_records(fn, N, rng, ENV_W, ENV_H)
        y = pyoracle.glsl_eval(G, "gref_", fn, x, nout, env=(marg, cond, ENV_W, ENV_H))
        out["env"][glsl_pin.ENV_NAMES[fn]] = {"fn": fn, "in_bits": bits(x), "out_bits": bits(y)}
    import pin_cases
    for key, variant in (("paths", "base"), ("paths_offline", "offline")):
        P = pyoracle.glsl_pt_lib(variant)
        assert P is not None, "path-tracing shaders not built (needs the reference checkout)"
        out[key] = {}
        for name, (make, settings, flatten_limit) in pin_cases.CASES.items():
            sd = make()
            scene = pyoracle.OracleScene(sd, flatten_limit=flatten_limit)
            v = sd.views[0]
            pix = np.sort(np.random.default_rng(len(name)).choice(v.width * v.height, 96, replace=False))
            pix = pix.astype(np.uint32)
            y = pyoracle.shader_paths(P, scene, v, settings, pin_cases.SAMPLE_BASE, pin_cases.SPP, pix)
            out[key][name] = {"pixels": pix.tolist(), "out_bits": bits(y)}
    # the any-hit shader (alpha test) on candidate hits of the textured scene's
    # non-opaque leaves and its opaque geometry
    import pin_cases
    P = pyoracle.glsl_pt_lib("base")
    inst, prim, uv = anyhit_candidates()
    scene = pyoracle.OracleScene(pin_cases.CASES["textured_pcg"][0]())
    out["anyhit"] = {"inst": inst.tolist(), "prim": prim.tolist(), "uv_bits": bits(uv),
                     "accept": pyoracle.shader_anyhit(P, scene, inst, prim, uv).tolist()}
    path = os.path.join(HERE, "glsl_kats.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print("wrote", path)


if __name__ == "__main__":
    main()
