"""ohao_bvh_build_noalloc: the BVH build for callers that cannot allocate
device memory (a host that owns the GPU's memory budget, or a per-frame
rebuild of a small animated mesh where cudaMalloc would synchronise the
device). It must produce exactly what the regular build (ohao_pt_build)
produces, call after call, although every call reuses one fixed device
array for its scratch. Collected last so that a failure here stops a -x run
only after every other test has run."""
import ctypes as C

import numpy as np
import pytest

from ohao_engine_gb300 import scenes
from pt_harness import small_env_scene

pytestmark = pytest.mark.gpu

TOO_LARGE = -8


def scene_boxes(sd):
    v = sd.pos[sd.indices.reshape(-1, 3)].astype(np.float32)
    lo = np.minimum(np.minimum(v[:, 0], v[:, 1]), v[:, 2])
    hi = np.maximum(np.maximum(v[:, 0], v[:, 1]), v[:, 2])
    return np.ascontiguousarray(np.concatenate([lo, hi], axis=1), np.float32)


def regular_build(og, sd):
    pt = og.PathTracer()
    pt.load_scene(sd)
    nodes, tris, height = pt.bvh()
    order = tris.view(np.uint32).reshape(-1, 12)[:, 11].copy()   # the record's build index
    pt.close()
    return nodes, order, height


def noalloc_build(og, boxes):
    import torch
    fn = og.load_library().ohao_bvh_build_noalloc
    n = boxes.shape[0]
    d_boxes = torch.from_numpy(boxes).cuda()
    d_nodes = torch.zeros(max(n, 1) * 80, dtype=torch.uint8, device="cuda")
    d_order = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    d_root = torch.zeros(8, dtype=torch.float32, device="cuda")
    nn, hh = C.c_uint32(), C.c_uint32()
    st = fn(C.c_void_p(d_boxes.data_ptr()), n, C.c_void_p(d_nodes.data_ptr()), C.c_void_p(d_order.data_ptr()),
            C.c_void_p(d_root.data_ptr()), C.byref(nn), C.byref(hh), None)
    assert st == 0, f"ohao_bvh_build_noalloc status {st}"
    torch.cuda.synchronize()
    nodes = d_nodes.cpu().numpy()[: nn.value * 80]
    order = d_order.cpu().numpy().view(np.uint32)
    root = d_root.cpu().numpy()[:6]
    return nodes, order, hh.value, root


def test_noalloc_matches_regular_build_call_after_call(gpu_lib):
    og = gpu_lib
    cases = [scenes.cornell(8, 8, 1), small_env_scene(freq=24), scenes.cornell(8, 8, 1)]
    for sd in cases:   # consecutive calls share the static scratch
        boxes = scene_boxes(sd)
        ref_nodes, ref_order, ref_h = regular_build(og, sd)
        nodes, order, h, root = noalloc_build(og, boxes)
        assert h == ref_h
        assert np.array_equal(nodes, ref_nodes), "node bytes differ from ohao_pt_build"
        assert np.array_equal(order, ref_order), "leaf order differs from ohao_pt_build"
        assert np.array_equal(root, np.concatenate([boxes[:, :3].min(0), boxes[:, 3:].max(0)]))


def triangle_soup(n, seed):
    """n seeded random small triangles in a unit cube: a scene with exactly n
    primitives, for builds at the fixed capacity of the scratch array."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.0, 1.0, (n, 1, 3))
    pos = (c + rng.normal(scale=0.01, size=(n, 3, 3))).reshape(-1, 3).astype(np.float32)
    nrm = np.zeros((pos.shape[0], 4), np.float32)
    nrm[:, 1] = 1.0
    uv = np.zeros((pos.shape[0], 2), np.float32)
    idx = np.arange(3 * n, dtype=np.uint32)
    mats = np.stack([scenes.material((0.5, 0.5, 0.5))])
    return scenes.SceneData("soup", pos, nrm, uv, idx, np.zeros(n, np.uint32), mats, np.zeros((0, 20), np.float32),
                            None, 1.0, [(0, idx.size)], scenes.identity_instance(1))


@pytest.mark.parametrize("n", [65536, 65535])
def test_noalloc_at_capacity(gpu_lib, n):
    """Builds at and one below OHAO_BVH_NOALLOC_MAX_PRIMS, where the scratch
    layout uses all of its per-primitive share, twice in a row."""
    og = gpu_lib
    sd = triangle_soup(n, seed=n)
    boxes = scene_boxes(sd)
    ref_nodes, ref_order, ref_h = regular_build(og, sd)
    for _ in range(2):
        nodes, order, h, _ = noalloc_build(og, boxes)
        assert h == ref_h
        assert np.array_equal(nodes, ref_nodes), "node bytes differ from ohao_pt_build at capacity"
        assert np.array_equal(order, ref_order), "leaf order differs from ohao_pt_build at capacity"


def test_noalloc_rejects_oversize(gpu_lib):
    fn = gpu_lib.load_library().ohao_bvh_build_noalloc
    nn, hh = C.c_uint32(), C.c_uint32()
    dummy = C.c_void_p(1)   # never dereferenced: the size check comes first
    st = fn(dummy, 65537, dummy, dummy, dummy, C.byref(nn), C.byref(hh), None)
    assert st == TOO_LARGE
