"""The guide tables of the environment map's inverse-CDF sampling
(ohao_engine_gb300/csrc/env_guide.hpp, used by the device's sample_env):
tests/cpp/env_guide_check.cpp, compiled with g++ here, runs the guided
search against the reference sampler's whole-row binary search
(shaders/includes/rt/env_sampling.glsl:15-37) on awkward CDF rows and
boundary draws, and requires the same index every time."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "env_guide_check.cpp")
EXE = os.path.join(ROOT, "ohao_engine_gb300", "_build", "env_guide_check")


def test_guided_search_equals_full_search():
    cxx = os.environ.get("CXX", "g++")
    assert shutil.which(cxx), "g++ is needed for the check"
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-ffp-contract=off",
           f"-I{os.path.join(ROOT, 'ohao_engine_gb300', 'csrc')}", SRC, "-o", EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([EXE], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
