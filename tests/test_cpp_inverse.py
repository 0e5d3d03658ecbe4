"""The C++ caller of the ABI (tests/cpp/inverse_formation.cpp, through
include/ohao_pt_inverse.hpp): compiled and linked with g++ against
libohao_pt.so here, run on the GPU (forward RGBA8 renders, then a tile
albedo map fitted with the analytic display-space gradient)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "inverse_formation.cpp")
LIBDIR = os.path.join(ROOT, "ohao_engine_gb300", "_lib")
EXE = os.path.join(ROOT, "ohao_engine_gb300", "_build", "inverse_formation")


def build_exe():
    from ohao_engine_gb300 import _build
    _build.build()
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    assert shutil.which(cxx), "g++ is needed for the C++ caller"
    cmd = [cxx, "-std=c++20", "-O2", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", SRC, f"-L{LIBDIR}",
           "-lohao_pt", f"-Wl,-rpath,{LIBDIR}", "-o", EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_cpp_caller_compiles_and_links():
    assert os.path.exists(build_exe())


@pytest.mark.gpu
def test_cpp_caller_runs_forward_and_fit(gpu_lib):
    exe = build_exe()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
