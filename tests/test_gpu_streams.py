"""The per-view wavefront's concurrent schedule against its serial one: the
shadow rays of each step run on a second stream beside the next step's
closest-hit rays, and with one ray per thread in traversal the view renders
as four pixel lanes on their own streams. A profiled render
(OHAO_PT_FLAG_PROFILE) runs everything in one lane on the caller's stream,
so it is the serial reference: the accumulators must be bit-identical,
including views whose lanes take several waves (more paths than a lane's
share of the scratch) and the host-buffer path."""
import numpy as np
import pytest

from pt_harness import gpu_tracer, small_env_scene, small_instanced

pytestmark = pytest.mark.gpu


def _render(og, pt, v, spp, profile, history=0, acc=None):
    import torch
    npix = v.width * v.height
    if acc is None:
        acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    flags = og.FLAG_SORT_MATERIAL | (og.FLAG_PROFILE if profile else 0)
    pt.render([og.make_view(v, accum=acc, history=history)],
              og.make_settings(spp=spp, max_bounces=4, sampler=1, sample_index_base=5, flags=flags,
                               mode=og.MODE_WAVEFRONT))
    torch.cuda.synchronize()
    return acc, (pt.profile().lanes if profile else None)


@pytest.mark.parametrize("kind", ["flat_small", "flat_multiwave", "two_level"])
def test_concurrent_schedule_equals_serial(gpu_lib, kind):
    og = gpu_lib
    if kind == "two_level":
        sd = small_instanced(side=48)
        pt = gpu_tracer(og, sd, flatten_limit=1)
        v, spp, want_lanes = sd.views[0], 3, 1   # persistent-warp traversal keeps one lane
    else:
        w, h = (64, 48) if kind == "flat_small" else (1024, 1024)
        sd = small_env_scene(freq=16, width=w, height=h)
        pt = gpu_tracer(og, sd)
        v, spp, want_lanes = sd.views[0], 3, 4
    serial, lanes = _render(og, pt, v, spp, profile=True)
    assert lanes == want_lanes
    concurrent, _ = _render(og, pt, v, spp, profile=False)
    assert np.array_equal(concurrent.cpu().numpy(), serial.cpu().numpy()), kind
    # a second call accumulating onto the first (history), both ways
    serial2, _ = _render(og, pt, v, 2, profile=True, history=spp, acc=serial.clone())
    concurrent2, _ = _render(og, pt, v, 2, profile=False, history=spp, acc=concurrent.clone())
    assert np.array_equal(concurrent2.cpu().numpy(), serial2.cpu().numpy()), kind


def test_host_buffer_path_equals_serial(gpu_lib):
    """ohao_pt_render_host (history uploaded on its own stream, the lanes
    waiting for it before they fold) against a serial device render."""
    import torch
    og = gpu_lib
    sd = small_env_scene(freq=16, width=96, height=64)
    pt = gpu_tracer(og, sd)
    v = sd.views[0]
    npix = v.width * v.height
    rng = np.random.default_rng(3)
    hist = np.zeros((npix, 4), np.float32)
    hist[:, :3] = rng.uniform(0.0, 2.0, (npix, 3))
    hist[:, 3] = 2.0
    dev = torch.from_numpy(hist.copy()).cuda()
    serial, _ = _render(og, pt, v, 3, profile=True, history=2, acc=dev)
    host = hist.copy()
    pt.render_host([og.make_view(v, history=2)], og.make_settings(
        spp=3, max_bounces=4, sampler=1, sample_index_base=5, flags=og.FLAG_SORT_MATERIAL,
        mode=og.MODE_WAVEFRONT), [host])
    assert np.array_equal(host, serial.cpu().numpy())
