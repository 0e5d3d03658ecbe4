"""Regenerate tests/golden/reference_kats.json from the reference's own code.

Compiles ohao/render/rt/{env_cdf,sobol_generator,owen_scramble}.cpp where they
lie in the reference tree (``make -C oracle ref``) and records their outputs
on fixed inputs. Run in a container that has the reference checkout:

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402


def env_maps():
    rng = np.random.default_rng(7)
    maps = {}
    maps["uniform_32x16"] = np.ones((16, 32, 4), np.float32)
    hot = np.full((8, 16, 4), 0.01, np.float32)
    hot[4, 10, :3] = 100.0
    maps["hotspot_16x8"] = hot
    maps["random_24x12"] = rng.uniform(0, 5, (12, 24, 4)).astype(np.float32)
    black = np.zeros((6, 10, 4), np.float32)
    black[2] = 3.0
    maps["blackrows_10x6"] = black
    return maps


def main():
    pyoracle.build(ref=True)
    R = pyoracle.ref_lib()
    assert R is not None, "reference helpers not built (needs the reference checkout)"
    out = {"generator": "tests/golden/make_golden.py", "source": "reference ohao/render/rt helpers, compiled in place"}
    idx = list(range(256)) + [1000, 4095, 65535, 2**31, 2**32 - 1]
    out["sobol_index"] = idx
    out["sobol_sample1d_bits"] = {str(d): [int(np.float32(R.ref_sobol_sample1d(i, d)).view(np.uint32)) for i in idx]
                                 for d in range(4)}
    dirs = R.ref_sobol_dirs()
    out["sobol_dirs"] = [int(dirs[i]) for i in range(128)]
    rng = np.random.default_rng(11)
    vs = [int(x) for x in rng.integers(0, 2**32, 512, dtype=np.uint64)]
    ss = [int(x) for x in rng.integers(0, 2**32, 512, dtype=np.uint64)]
    out["owen_v"], out["owen_seed"] = vs, ss
    out["owen_out"] = [int(R.ref_owen_scramble(v, s)) for v, s in zip(vs, ss)]
    cdfs = {}
    for name, m in env_maps().items():
        h, w = m.shape[:2]
        marg = np.zeros(h, np.float32)
        cond = np.zeros(w * h, np.float32)
        integ = np.zeros(1, np.float32)
        R.ref_env_cdf_build(m.ctypes.data, w, h, marg.ctypes.data, cond.ctypes.data, integ.ctypes.data)
        cdfs[name] = {"w": w, "h": h, "pixels_bits": m.reshape(-1).view(np.uint32).tolist(),
                      "marg_bits": marg.view(np.uint32).tolist(), "cond_bits": cond.view(np.uint32).tolist(),
                      "integral_bits": int(integ.view(np.uint32)[0])}
    out["env_cdf"] = cdfs
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(out, f)
    print("wrote", os.path.join(HERE, "reference_kats.json"))


if __name__ == "__main__":
    main()
