"""Emitter MIS (OHAO_PT_FLAG_EMITTER_MIS) in the host oracle: the emissive-
triangle table, the light-NEE sampler's pdf (its estimates of the solid
angle and of the cosine-weighted solid angle of the emitters match a closed
form and a quadrature), and the agreement of the pdf the NEE side uses with the one
the BSDF side finds for the same direction, for emissive triangles, area and
sphere lights. The device follows the same code path for path; its parity
is checked in test_gpu_emitter_mis.py."""
import math

import numpy as np
import pytest

from pt_harness import emitter_scene

EMITTER_MIS = 1 << 13


def _world_tris(sd):
    """(instance, prim, world corners float32) of every triangle of every
    instance, the transform applied as the oracle applies it."""
    out = []
    for ii, inst in enumerate(sd.instances):
        fi, ic = sd.blas[int(inst["blas"])]
        x = inst["xform"].astype(np.float32).reshape(3, 4)
        for p in range(ic // 3):
            v = sd.pos[sd.indices[fi + 3 * p: fi + 3 * p + 3]].astype(np.float32)
            w = np.zeros((3, 3), np.float32)
            for k in range(3):
                for r in range(3):
                    w[k, r] = np.float32(np.float32(np.float32(x[r, 0] * v[k, 0]) + np.float32(x[r, 1] * v[k, 1]))
                                         + np.float32(x[r, 2] * v[k, 2])) + x[r, 3]
            out.append((ii, p, w))
    return out


def _emission_weight(m):
    l = 0.2126 * max(m[9], 0) + 0.7152 * max(m[10], 0) + 0.0722 * max(m[11], 0)
    return l + (1.0 if m[7:8].view(np.uint32)[0] != 0xFFFFFFFF else 0.0)


def test_table_entries_and_pdfs(oracle):
    """Entries: the emissive triangles of visible, opaque instances in
    instance and triangle order (the masked and the non-opaque instance of
    the emissive triangle left out); pdf per area x area is the CDF step,
    and the steps are proportional to area x emission weight."""
    sd = emitter_scene()
    o = oracle.OracleScene(sd)
    tri, cdf = o.emitter_table()
    blas_flags = sd.blas_flags
    want = []
    for ii, p, w in _world_tris(sd):
        inst = sd.instances[ii]
        gtri = int(inst["custom_index"]) + p
        m = sd.materials[sd.mat_ids[gtri]]
        if inst["mask"] & 0xFF and not blas_flags[int(inst["blas"])] and _emission_weight(m) > 0:
            want.append((ii, p, w, _emission_weight(m)))
    assert [(a, b) for a, b, _, _ in want] == list(zip(tri[:, 7].view(np.uint32), tri[:, 11].view(np.uint32)))
    assert [a for a, _, _, _ in want] == [0, 0, 0, 0, 1]
    for k, (_, _, w, _) in enumerate(want):
        assert np.array_equal(tri[k, 0:3], w[0])
        assert np.array_equal(tri[k, 4:7], w[1] - w[0])
        assert np.array_equal(tri[k, 8:11], w[2] - w[0])
    area = np.array([0.5 * np.linalg.norm(np.cross(tri[k, 4:7].astype(np.float64), tri[k, 8:11].astype(np.float64)))
                     for k in range(len(want))])
    power = area * np.array([wt for _, _, _, wt in want])
    assert np.all(np.diff(cdf) >= 0) and cdf[-1] == 1.0
    step = np.diff(np.concatenate([[0.0], cdf.astype(np.float64)]))
    assert np.allclose(step, power / power.sum(), rtol=1e-5)
    assert np.allclose(tri[:, 3] * area, step, rtol=1e-5)


def _solid_angle(P, tris):
    """Solid angle of triangles seen from P (Van Oosterom and Strackee)."""
    sa = 0.0
    for w in tris:
        a, b, c = w.astype(np.float64) - P
        la, lb, lc = np.linalg.norm(a), np.linalg.norm(b), np.linalg.norm(c)
        num = abs(np.dot(a, np.cross(b, c)))
        den = la * lb * lc + np.dot(a, b) * lc + np.dot(a, c) * lb + np.dot(b, c) * la
        sa += 2.0 * math.atan2(num, den)
    return sa


def _cosine_solid_angle(P, N, tris, m=256):
    """Integral of max(N.L, 0) over the directions to the triangles from P:
    midpoint rule over m^2 sub-triangles of each (float64)."""
    i, j = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    up = (i + j) < m
    dn = (i + j) < m - 1
    bary = np.concatenate([np.stack([(i[up] + 1 / 3) / m, (j[up] + 1 / 3) / m], -1),
                           np.stack([(i[dn] + 2 / 3) / m, (j[dn] + 2 / 3) / m], -1)])
    total = 0.0
    for w in tris:
        w = w.astype(np.float64)
        e1, e2 = w[1] - w[0], w[2] - w[0]
        ng = np.cross(e1, e2)
        area = 0.5 * np.linalg.norm(ng)
        ng /= np.linalg.norm(ng)
        pts = w[0] + bary[:, :1] * e1 + bary[:, 1:] * e2
        d = pts - P
        ld = np.linalg.norm(d, axis=1)
        L = d / ld[:, None]
        f = np.maximum(L @ N, 0.0) * np.abs(L @ ng) / ld ** 2
        total += f.sum() * area / m ** 2
    return total


@pytest.mark.parametrize("P", [(0.0, -0.5, 0.0), (-1.0, 0.2, 0.5)])
def test_sampler_estimates_closed_forms(oracle, P):
    """No GPULights: every draw picks an emissive triangle. The estimates
    E[1 / pdf] (weight x choices) and E[max(N.L, 0) / pdf] equal the
    emitters' solid angle (closed form) and cosine-weighted solid angle
    (quadrature) within 5 standard errors."""
    sd = emitter_scene(lights=())
    o = oracle.OracleScene(sd)
    tri, _ = o.emitter_table()
    P = np.array(P, np.float64)
    N = np.array([0.3, 1.0, -0.2])
    N /= np.linalg.norm(N)
    n = 200_000
    s = o.light_samples(EMITTER_MIS, P, N, n, seed=3).astype(np.float64)
    assert np.all(s[:, 7] == 1.0)
    inv_pdf = s[:, 6] * s[:, 7]
    cosw = inv_pdf * np.maximum(s[:, :3] @ N, 0.0)
    corners = [np.stack([t[0:3], t[0:3] + t[4:7], t[0:3] + t[8:11]]) for t in tri]
    for est, ref, tol in ((inv_pdf, _solid_angle(P, corners), 1e-6), (cosw, _cosine_solid_angle(P, N, corners), 1e-3)):
        se = est.std() / math.sqrt(n)
        assert abs(est.mean() - ref) < 5 * se + tol * ref, (est.mean(), ref, se)


def test_triangle_pdf_agrees_with_hit_side(oracle):
    """An emissive-triangle draw and a BSDF ray along the same direction find
    the same pdf (the hit point is the sampled point)."""
    sd = emitter_scene(lights=())
    o = oracle.OracleScene(sd)
    s = o.light_samples(EMITTER_MIS, (0.2, -0.6, 0.3), (0.0, 1.0, 0.0), 4000, seed=5)
    ok = (s[:, 9] == 1.0) & (s[:, 10] > 0)
    assert ok.sum() > 1000
    assert np.allclose(s[ok, 10], s[ok, 8], rtol=2e-4)


@pytest.mark.parametrize("kind", ["area", "sphere"])
def test_light_pdf_agrees_with_hit_side(oracle, kind):
    """A GPULight draw weighted for MIS (emitter-MIS pdf p) and a BSDF ray
    of pdf 1 along the same direction, which finds the light with weight
    1 / (1 + p): Le / found - 1 = p away from the silhouette, and the BSDF
    weights agree everywhere (at grazing draws the entry point of the ray is
    ill-conditioned, but both weights are near 0 there)."""
    sd = emitter_scene(lights=(kind,))
    sd.materials[:, 9:12] = 0.0      # no emissive triangles: the light is the only choice
    o = oracle.OracleScene(sd)
    s = o.light_samples(EMITTER_MIS, (0.1, -0.9, 0.4), (0.0, 1.0, 0.0), 4000, seed=7)
    assert np.all(s[:, 7] == 1.0)
    ok = (s[:, 9] == 1.0) & (s[:, 11] > 0)
    assert ok.sum() > 1000
    p_hit = s[ok, 3] / s[ok, 11] - 1.0
    away = s[ok, 8] < 50.0
    assert away.sum() > 1000
    assert np.allclose(p_hit[away], s[ok, 8][away], rtol=2e-3)
    assert np.allclose(1.0 / (1.0 + p_hit), 1.0 / (1.0 + s[ok, 8]), atol=2e-3)


def test_flag_off_is_the_reference_choice(oracle):
    """Without the flag the NEE chooses among the GPULights alone, with no
    MIS pdf."""
    sd = emitter_scene()
    o = oracle.OracleScene(sd)
    s = o.light_samples(0, (0.0, -0.5, 0.0), (0.0, 1.0, 0.0), 256, seed=1)
    assert np.all(s[:, 7] == len(sd.lights)) and np.all(s[:, 8] == 0.0)
    s = o.light_samples(EMITTER_MIS, (0.0, -0.5, 0.0), (0.0, 1.0, 0.0), 256, seed=1)
    assert np.all(s[:, 7] == len(sd.lights) + 1) and np.all(s[s[:, 9] == 1, 8] > 0)


def test_degenerate_and_negative_emitters(oracle):
    """A zero-area emissive triangle keeps its table slot with pdf 0 (the
    search never lands on a zero CDF step, and a BSDF hit on it takes weight
    1); negative emission channels count as 0 in the power; a material whose
    emission is all non-positive is not an emitter."""
    from ohao_engine_gb300 import scenes
    sd = emitter_scene(lights=())
    n0 = sd.blas[0][1] // 3                      # BLAS 0's triangles; the instanced triangle follows
    idx = sd.indices.reshape(-1, 3)
    deg, nonpos = len(sd.materials), len(sd.materials) + 1
    sd.materials = np.concatenate([sd.materials,
                                   scenes.material((0.5, 0.5, 0.5), emissive=(8.0, -3.0, 2.0))[None],
                                   scenes.material((0.5, 0.5, 0.5), emissive=(-1.0, 0.0, -2.0))[None]])
    # two new triangles appended to BLAS 0: collinear corners, and a plain one
    nv = sd.pos.shape[0]
    new_pos = np.array([(0.0, 0.5, 0.0), (0.5, 0.5, 0.0), (1.0, 0.5, 0.0),
                        (0.0, 0.9, 0.0), (0.5, 0.9, 0.0), (0.0, 0.9, 0.5)], np.float32)
    sd.pos = np.concatenate([sd.pos, new_pos])
    sd.normals = np.concatenate([sd.normals, np.tile(np.array([0.0, 1.0, 0.0, 0.0], np.float32), (6, 1))])
    sd.uvs = np.concatenate([sd.uvs, np.zeros((6, 2), np.float32)])
    new_idx = np.array([[nv, nv + 1, nv + 2], [nv + 3, nv + 4, nv + 5]], np.uint32)
    sd.indices = np.ascontiguousarray(np.concatenate([idx[:n0], new_idx, idx[n0:]]).reshape(-1))
    sd.mat_ids = np.ascontiguousarray(np.concatenate([sd.mat_ids[:n0], [deg, nonpos], sd.mat_ids[n0:]]).astype(np.uint32))
    sd.blas = [(0, 3 * (n0 + 2)), (3 * (n0 + 2), 3), (3 * (n0 + 2), 3)]
    inst = sd.instances.copy()
    for k in (1, 2, 3):
        inst[k]["custom_index"] = n0 + 2
    sd.instances = inst
    o = oracle.OracleScene(sd)
    tri, cdf = o.emitter_table()
    pairs = list(zip(tri[:, 7].view(np.uint32).tolist(), tri[:, 11].view(np.uint32).tolist()))
    assert (0, n0) in pairs, "the degenerate emitter keeps its slot"
    assert (0, n0 + 1) not in pairs, "non-positive emission is no emitter"
    k = pairs.index((0, n0))
    assert tri[k, 3] == 0.0
    step = np.diff(np.concatenate([[0.0], cdf.astype(np.float64)]))
    assert step[k] == 0.0
    s = o.light_samples(EMITTER_MIS, (0.2, -0.6, 0.3), (0.0, 1.0, 0.0), 20000, seed=9)
    assert np.all(np.isfinite(s[s[:, 9] == 1]))
