"""In-tree build of libohao_pt.so (sm_103a) with nvcc and g++.

``build()`` compiles every translation unit under ``csrc/`` in parallel and
links ``_lib/libohao_pt.so`` (CUDA runtime linked statically, no torch).
Device code is compiled with ``-fmad=false`` so that floating-point results
follow the operation order written in the source (fused multiply-adds only
where ``fmaf`` is explicit).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libohao_pt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++20", "-fmad=false", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wall"]

CU_SOURCES = ["bvh_build.cu", "scene_kernels.cu", "wavefront.cu", "adjoint.cu", "dn_kernels.cu", "display.cu", "aov.cu"]
CPP_SOURCES = ["abi.cpp", "dn_net.cpp"]


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home:
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _nvcc() -> str:
    return shutil.which("nvcc") or os.path.join(_cuda_home(), "bin", "nvcc")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))] + [
        os.path.join(PKG, "..", "include", "ohao_pt.h"), os.path.join(PKG, "..", "include", "ohao_dn.h")]


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if _newer(obj, deps):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, f"-I{os.path.join(_cuda_home(), 'include')}", "-c", src,
               "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _newer(LIB, objs):
        return LIB
    cmd = [_nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", LIB, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
