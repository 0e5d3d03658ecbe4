"""Compiles the reference's path-tracing shaders as C++ -- TEST INFRASTRUCTURE ONLY.

The path's shaders run only through Vulkan ray tracing, which neither this
machine nor the GPU host can bring up. Their arithmetic is ordinary scalar
GLSL, so it is compiled here, from the reference tree where it lies, as C++
against the GLSL subset of ``glsl_shim.hpp`` (and the ray-tracing built-ins
of ``glsl_rt.hpp``) with ``-fsingle-precision-constant`` (GLSL float
literals are single precision). Two libraries come out of it:

* ``oracle/_ref/libohao_glsl.so``: the helper includes (PCG sampler, balance
  heuristic, GGX D / Smith / VNDF sampling, metal-rough unpack, environment
  CDF search and pdf) behind ``glsl_ref_api.inc``;
* ``oracle/_ref/libohao_glslpt[_offline].so``: a raygen (the default one or
  the offline profile's) with the closest-hit, miss and any-hit (alpha test)
  shaders and every file they include, behind ``glsl_pt_api.inc``;
  ``traceRayEXT`` runs the oracle's traversal (``glsl_pt_host.cpp``); the
  any-hit shader is driven on its own for candidate hits.

The text changes are mechanical and listed in ``shader_text``: GLSL's
``out`` / ``inout T name`` parameters written as C++ references ``T& name``
(the same copy-out result when arguments do not alias), comments and
``#version`` / ``#extension`` lines dropped, includes inlined, the
specialization constant made a settable global, unsized buffer arrays as
pointers, array constructors as brace lists. The source text goes to the
compiler on standard input; only the libraries are written. The pin tests
compare them with the oracle bit for bit, and
``tests/golden/make_glsl_golden.py`` records their outputs as fixtures for
machines without the reference tree.
"""
from __future__ import annotations

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("OHAO_REFERENCE_ROOT", "/root/reference")   # the reference checkout, where present
LIB_PATH = os.path.join(HERE, "_ref", "libohao_glsl.so")

GLSL_FILES = [
    "shaders/includes/rt/sampler_pcg.glsl",
    "shaders/includes/rt/mis.glsl",
    "shaders/includes/material/ggx_aniso.glsl",
    "shaders/rt/includes/pbr_unpack.glsl",
    "shaders/includes/rt/env_sampling.glsl",
]

_OUT_PARAM = re.compile(r"\bout\s+(\w+)\s+(\w+)")


def translation_unit(ref_root: str = REF_ROOT) -> str:
    parts = ['#include "glsl_shim.hpp"', "namespace glsl {",
             "inline FloatBuffer envMarg{nullptr}, envCond{nullptr};   // env_sampling.glsl's CDF buffers"]
    for rel in GLSL_FILES:
        with open(os.path.join(ref_root, rel)) as f:
            text = f.read()
        parts.append(f'#line 1 "{rel}"')
        parts.append(_OUT_PARAM.sub(r"\1& \2", text))
    parts.append("}  // namespace glsl")
    parts.append('#include "glsl_ref_api.inc"')
    return "\n".join(parts) + "\n"


def available(ref_root: str = REF_ROOT) -> bool:
    return all(os.path.exists(os.path.join(ref_root, rel)) for rel in GLSL_FILES)


def build(ref_root: str = REF_ROOT) -> str:
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fsingle-precision-constant",
           "-fno-strict-aliasing",
           "-Wall", "-Wno-unused-variable", "-Wno-unused-but-set-variable", "-I", HERE, "-x", "c++", "-",
           "-o", LIB_PATH]
    subprocess.run(cmd, input=translation_unit(ref_root), text=True, check=True)
    return LIB_PATH


# ---- record layouts and input generators shared by the fixtures and tests ----
# (inputs, outputs) floats per record; function ids as in glsl_ref_api.inc
HELPER_IO = {0: (3, 10), 1: (2, 1), 2: (10, 1), 3: (2, 1), 4: (2, 1), 5: (2, 1), 6: (3, 1), 7: (7, 3), 8: (3, 2)}
HELPER_NAMES = {0: "pcg_stream", 1: "mis_balance", 2: "ggx_d_aniso_or_iso", 3: "ggx_d_iso", 4: "smith_lambda",
                5: "smith_g1", 6: "smith_g2_over_g1", 7: "sample_ggx_vndf", 8: "unpack_hit_pbr"}
ENV_IO = {0: (1, 1), 1: (2, 1), 2: (2, 4), 3: (3, 1)}
ENV_NAMES = {0: "search_marginal", 1: "search_conditional", 2: "sample_env_map", 3: "pdf_env_map"}


def _unit(rng, n):
    import numpy as np
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def helper_records(fn: int, n: int, rng):
    """n input records of helper ``fn``, float32 [n, inputs]: the ranges the
    integrator feeds them plus the branch edges (anisotropy at and around its
    0.001 switch, signed-roughness payloads, zero pdfs)."""
    import numpy as np
    if fn == 0:
        x = np.stack([rng.integers(0, 4096, n), rng.integers(0, 4096, n), rng.integers(0, 1 << 20, n)], 1)
    elif fn == 1:
        x = rng.exponential(1.0, (n, 2)) * (rng.random((n, 2)) < 0.9)
    elif fn == 2:
        N, H = _unit(rng, n), _unit(rng, n)
        ndh = np.abs((N * H).sum(1, keepdims=True))
        x = np.concatenate([N, H, ndh, rng.uniform(0, 1, (n, 1)),
                            rng.choice([0.0, 0.0005, 0.001, 0.3, 0.9, 1.0], (n, 1)), rng.uniform(-3, 3, (n, 1))], 1)
    elif fn in (3, 4, 5):
        x = np.stack([rng.uniform(-1, 1, n), rng.uniform(0, 1, n)], 1)
    elif fn == 6:
        x = rng.uniform(0, 1, (n, 3))
    elif fn == 7:
        ve = _unit(rng, n)
        ve[:, 2] = np.abs(ve[:, 2]) + 1e-3
        ve /= np.linalg.norm(ve, axis=1, keepdims=True)
        x = np.concatenate([ve, rng.uniform(0.001, 1, (n, 2)), rng.random((n, 2))], 1)
    else:
        x = np.concatenate([rng.uniform(-12, 12, (n, 1)), rng.choice([0.0, 5e-5, 0.5, 1.0, 1.5, -0.2], (n, 1)),
                            rng.random((n, 1))], 1)
    return np.ascontiguousarray(x, np.float32)


def env_records(fn: int, n: int, rng, w: int, h: int):
    import numpy as np
    if fn == 0:
        x = rng.random((n, 1))
    elif fn == 1:
        x = np.stack([rng.integers(0, h, n), rng.random(n)], 1)
    elif fn == 2:
        x = rng.random((n, 2))
    else:
        x = _unit(rng, n)
    return np.ascontiguousarray(x, np.float32)


# ---- the path-tracing shaders themselves (raygen, closest hit, miss) ----
# raygen variants: the path tracer's default raygen, and the offline
# profile's (the same estimator with its analytic-light products regrouped
# and optional subsurface terms, off unless push constant tuning.w > 0)
PT_RAYGENS = {"base": "shaders/rt/pt_raygen.rgen", "offline": "shaders/rt/pt_raygen_offline.rgen"}
PT_HIT_MISS = [("rchit", "shaders/rt/pt_closesthit.rchit"), ("rmiss", "shaders/rt/pt_miss.rmiss"),
               ("rahit", "shaders/rt/pt_anyhit.rahit")]


def pt_lib_path(variant: str = "base") -> str:
    return os.path.join(HERE, "_ref", "libohao_glslpt.so" if variant == "base" else f"libohao_glslpt_{variant}.so")

_COMMENTS = re.compile(r"//[^\n]*|/\*.*?\*/", re.S)
_INOUT_PARAM = re.compile(r"\b(?:out|inout)\s+(\w+)\s+(\w+)")
_SPEC_CONST = re.compile(r"layout\s*\(\s*constant_id\s*=\s*\d+\s*\)\s*const\s+")
_UNSIZED = re.compile(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;")
_ARRAY_CTOR = re.compile(r"=\s*\w+\s*\[\s*\d*\s*\]\s*\(")
_DEFINE = re.compile(r"^\s*#\s*define\s+(\w+)", re.M)


def _expand(path: str, ref_root: str) -> str:
    """The shader with its #include files inlined (resolved against the
    including file's folder, then shaders/), #version / #extension dropped."""
    out = []
    with open(path) as f:
        for line in f.read().splitlines():
            m = re.match(r'\s*#\s*include\s+"([^"]+)"', line)
            if m:
                cands = [os.path.join(os.path.dirname(path), m.group(1)), os.path.join(ref_root, "shaders", m.group(1))]
                out.append(_expand(next(c for c in cands if os.path.exists(c)), ref_root))
            elif not re.match(r"\s*#\s*(version|extension)\b", line):
                out.append(line)
    return "\n".join(out)


def _array_ctors(text: str) -> str:
    """`= T[N](a, b, ...)` array constructors -> `= {a, b, ...}`."""
    while True:
        m = _ARRAY_CTOR.search(text)
        if not m:
            return text
        depth, i = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        text = text[:m.start()] + "= {" + text[m.end():i - 1] + "}" + text[i:]


def shader_text(rel: str, ref_root: str = REF_ROOT) -> str:
    """GLSL -> C++ for one shader: comments removed, `out`/`inout T x` ->
    `T& x`, specialization constants as plain globals, unsized buffer arrays
    as pointers, array constructors as brace lists. Nothing else changes."""
    text = _COMMENTS.sub(lambda m: "\n" * m.group(0).count("\n"), _expand(os.path.join(ref_root, rel), ref_root))
    text = _INOUT_PARAM.sub(r"\1& \2", text)
    text = _SPEC_CONST.sub("", text)
    text = _UNSIZED.sub(r"\1* \2;", text)
    return _array_ctors(text)


def pt_translation_unit(ref_root: str = REF_ROOT, variant: str = "base") -> str:
    parts = ['#include "glsl_rt.hpp"']
    for ns, rel in [("rgen", PT_RAYGENS[variant])] + PT_HIT_MISS:
        text = shader_text(rel, ref_root)
        parts += [f"namespace {ns} {{", "using namespace glsl;", f'#line 1 "{rel}"', text, f"}}  // namespace {ns}"]
        parts += [f"#undef {name}" for name in sorted(set(_DEFINE.findall(text)))]
    parts.append('#include "glsl_pt_api.inc"')
    return "\n".join(parts) + "\n"


def pt_available(ref_root: str = REF_ROOT) -> bool:
    rels = list(PT_RAYGENS.values()) + [rel for _, rel in PT_HIT_MISS]
    return all(os.path.exists(os.path.join(ref_root, rel)) for rel in rels)


def build_pt(ref_root: str = REF_ROOT) -> list:
    """libohao_glslpt[_offline].so: a raygen variant with the closest-hit and
    miss shaders (GLSL float semantics) + the host side over the oracle's
    scene (glsl_pt_host.cpp, ordinary flags)."""
    paths = []
    for variant in PT_RAYGENS:
        out = pt_lib_path(variant)
        os.makedirs(os.path.dirname(out), exist_ok=True)
        obj = out[:-3] + ".o"
        subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-c", "-ffp-contract=off",
                        "-fsingle-precision-constant", "-fno-strict-aliasing", "-w", "-I", HERE, "-x", "c++", "-",
                        "-o", obj], input=pt_translation_unit(ref_root, variant), text=True, check=True)
        subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", HERE,
                        os.path.join(HERE, "glsl_pt_host.cpp"), obj, "-o", out], check=True)
        os.remove(obj)
        paths.append(out)
    return paths


if __name__ == "__main__":
    print(build())
    print(build_pt())
