"""C-ABI library checks that need no GPU: it loads, exports every function
include/ohao_pt.h declares, its host EnvCDF helper is bit-identical to the
reference's EnvCDF::build, and device entry points fail with a status code
(not a crash) when no CUDA device is usable."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def og():
    from ohao_engine_gb300 import _build
    _build.build()
    import ohao_engine_gb300 as og
    og.load_library()
    return og


def header_functions():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ohao_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(og):
    import subprocess
    names = header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", og.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    from ohao_engine_gb300 import denoise
    assert sorted(og.EXPORTED_SYMBOLS + denoise.EXPORTED_SYMBOLS) == names


def test_struct_sizes_match_header(og):
    import ctypes as C
    assert C.sizeof(og.View) == 16 * 4 * 2 + 16 + 4 * 8
    assert C.sizeof(og.Settings) == 64
    from ohao_engine_gb300 import scenes
    assert scenes.INSTANCE_DTYPE.itemsize == 64


def test_env_cdf_helper_bit_identical(og, oracle):
    rng = np.random.default_rng(5)
    for shape in ((16, 32), (7, 13), (64, 128)):
        env = rng.uniform(0, 4, shape + (4,)).astype(np.float32)
        env[1] = 0.0   # a black row exercises the uniform fallback
        a = og.EnvCDF().build(env)
        m, c, i = oracle.env_cdf(env)
        assert np.array_equal(a.marginal.view(np.uint32), m.view(np.uint32))
        assert np.array_equal(a.conditional.view(np.uint32), c.view(np.uint32))
        assert np.float32(a.integral).view(np.uint32) == np.float32(i).view(np.uint32)


def test_version_string(og):
    assert "sm_103a" in og.version()


def test_no_device_reports_status(og):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(og.OhaoError):
        og.PathTracer()


def test_no_device_reports_status_denoiser(og):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from ohao_engine_gb300.denoise import Denoiser
    with pytest.raises(og.OhaoError):
        Denoiser(max_pixels=1024, seed=1)


def test_launch_shapes_listed_without_device(og):
    """The persistent launch shapes are a host table: listed without a GPU,
    each name unique, the persistent-warp traversal among them."""
    L = og.load_library()
    names, i = [], 0
    while True:
        n = L.ohao_pt_launch_config_at(i)
        if n is None:
            break
        names.append(n.decode())
        i += 1
    assert len(names) == len(set(names)) >= 5
    assert any("fetch" in n for n in names) and any("sorted" in n for n in names)


def test_buffer_checks_before_any_device_call(og):
    """Buffers the kernels write unchecked are checked in the Python layer:
    host arrays, wrong dtypes, short or strided tensors and host tensors
    where a device buffer is needed raise ValueError; raw pointers pass."""
    import torch
    from ohao_engine_gb300 import scenes
    v = scenes.look_at_view((0, 0, 3), (0, 0, 0), width=8, height=4)
    npix = 32
    bad = [np.zeros((npix, 4), np.float32),                       # host array
           torch.zeros((npix, 4), dtype=torch.float64),             # dtype
           torch.zeros((npix - 1, 4), dtype=torch.float32),         # too short
           torch.zeros((npix, 8), dtype=torch.float32)[:, :4],      # strided
           torch.zeros((npix, 4), dtype=torch.float32)]             # on the host
    for b in bad:
        with pytest.raises(ValueError):
            og.make_view(v, accum=b)
    with pytest.raises(ValueError):
        og.make_view(v, aov=torch.zeros((npix, og.AOV_FLOATS - 1)))
    assert og.make_view(v, accum=0x7f0000000000).accum == 0x7f0000000000
    # host buffers (render_host): writable C-contiguous float32 arrays
    ok = np.zeros((npix, 4), np.float32)
    assert og._buffer(ok, npix * 4, "host_accum", host=True) == ok.ctypes.data
    ro = np.zeros((npix, 4), np.float32)
    ro.flags.writeable = False
    for b in (np.zeros((npix, 4)), ro, np.zeros((npix, 3), np.float32)):
        with pytest.raises(ValueError):
            og._buffer(b, npix * 4, "host_accum", host=True)
    # 4-byte integer buffers (trace hits) where floats are not required
    with pytest.raises(ValueError):
        og._buffer(torch.zeros(10, dtype=torch.int32), 10, "hits")
    with pytest.raises(ValueError, match="CUDA device"):
        og._buffer(torch.zeros(10, dtype=torch.int32), 10, "hits", floats=False)


def test_path_radiance_must_hold_the_call_samples(og):
    from ohao_engine_gb300 import scenes
    v = og.make_view(scenes.look_at_view((0, 0, 3), (0, 0, 0), width=8, height=4))
    v._path_samples = 2
    assert len(og._view_array([v], og.make_settings(spp=2))) == 1
    with pytest.raises(ValueError):
        og._view_array([v], og.make_settings(spp=3))


def test_denoiser_frame_checks(og):
    import torch
    from ohao_engine_gb300 import denoise
    with pytest.raises(ValueError, match="2 buffers expected"):
        denoise._frames([torch.zeros(8)], 2, 8, "aov")
    with pytest.raises(ValueError):
        denoise._frames([torch.zeros(7)], 1, 8, "aov")
    assert list(denoise._frames([0x1000, 0x2000], 2, 8, "out")) == [0x1000, 0x2000]
