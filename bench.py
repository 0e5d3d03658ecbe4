#!/usr/bin/env python3
"""Benchmark: Msamples/s of the 4-bounce path tracer on one GB300.

Default workload (the reference's metric on its single-object config):
geodesic sphere of frequency 224 (1,003,520 triangles) displaced by 5% value
noise plus a 2-triangle plane, per-triangle GGX materials, 1024x512 sky+sun
environment with importance sampling and balance-heuristic MIS, 1920x1080,
1 sample per pixel per step, max depth 4, PCG sampler, progressive
accumulation. A step is one render call (one sample per pixel) of that frame.

Prints one JSON line (rank 0). `value` is device-timed with inputs resident
in HBM; `e2e` repeats the measurement through ohao_pt_render_host with host
buffers (accumulator uploaded and downloaded every step); `roofline` covers
the dominant kernel (closest-hit traversal, k_extend); `cpu_baseline` times
the host oracle on a bounded pixel subset on this machine's cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "Msamples/s 4-bounce PT; batched+adjoint vs plain at equal RMSE, 1 GB300"
UNIT = "Msamples/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sphere_1m", choices=["sphere_1m", "cornell", "instanced", "studio", "denoise"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shade-order", default="material", choices=["material", "queue"],
                    help="shade each ray queue in material order (binned on the device) or in queue order; "
                         "the image is the same")
    ap.add_argument("--no-gates", action="store_true",
                    help="skip the gates (configs 3-5 and the FP64 comparisons) after the headline")
    ap.add_argument("--case", default=None, choices=sorted(CASES),
                    help="run one small profiling case instead of the benchmark (one process, a few GB at most)")
    ap.add_argument("--case-arg", default=None, help="launch shape name for --case instanced_pool")
    return ap.parse_args()


def workload(name):
    from ohao_engine_gb300 import scenes
    if name == "cornell":
        sd = scenes.cornell(256, 256, 16)
        desc = ("cornell: 36 tris, 1 area light, 256x256, 16 spp per step, depth 4, PCG")
        return sd, 16, desc
    sd = scenes.sphere_1m()
    desc = ("sphere_1m: geodesic sphere f=224 displaced 5% (1,003,520 tris) + 2-tri plane, per-triangle GGX, "
            "env 1024x512 sky+sun with IS + balance MIS, 1920x1080, 1 spp per step, depth 4, PCG")
    return sd, 1, desc


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.dev), "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


TRAVERSAL_SOURCES = ["pt_device.cuh", "pt_traverse.cuh", "pt_fetch.cuh", "wavefront.cu", "pt_types.hpp"]


def traversal_source_sha():
    """sha256 of the sources k_extend is compiled from: a committed DRAM
    traffic figure is used only while it was captured from these sources."""
    import hashlib
    h = hashlib.sha256()
    for f in TRAVERSAL_SOURCES:
        with open(os.path.join(ROOT, "ohao_engine_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def traffic_from_profiles(kernel, workload_name):
    """DRAM bytes per launch of the kernel from the committed ncu capture
    (profiles/<kernel>_<workload>.json), or None with the reason when the
    capture does not match the current traversal sources."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload_name}.json")
    if not os.path.exists(p):
        return None, "no ncu capture committed for this kernel and workload"
    d = json.load(open(p))
    if d.get("source_sha256") != traversal_source_sha():
        return None, (f"the committed capture ({os.path.basename(p)}) was taken from other traversal sources than "
                      "these; re-capture with the command in profiles/ to fill traffic")
    return d.get("dram_bytes_per_launch"), d.get("note")


def cpu_baseline(sd, spp_step, target_s, full_step_samples):
    import pyoracle
    t0 = time.time()
    orc = pyoracle.OracleScene(sd)
    build_s = time.time() - t0
    v = sd.views[0]
    npix = v.width * v.height
    rng = np.random.default_rng(123)
    st = dict(max_bounces=sd.max_bounces, sampler=0)
    # calibrate on a small subset, then time a subset sized for ~target_s
    n0 = min(npix, 4096)
    pix = np.sort(rng.choice(npix, n0, replace=False)).astype(np.uint32)
    t0 = time.time()
    orc.render_paths(v, st, 0, spp_step, pixels=pix)
    dt0 = max(time.time() - t0, 1e-3)
    want = n0 * target_s / dt0                      # paths (at spp_step per pixel) for ~target_s
    n1 = int(min(npix, max(n0, want)))
    spp = spp_step * max(1, int(round(want / n1)))  # whole frame not enough: more samples per pixel
    pix = np.sort(rng.choice(npix, n1, replace=False)).astype(np.uint32)
    t0 = time.time()
    orc.render_paths(v, st, 0, spp, pixels=pix)
    dt = time.time() - t0
    samples = n1 * spp
    return {"value": samples / dt / 1e6, "unit": UNIT, "cores": int(pyoracle.lib().orc_num_threads()),
            "kind": "port",
            "sample": f"{n1} seeded random pixels x {spp} spp of the same frame ({samples} paths, "
                      f"{dt:.1f} s; host BVH build {build_s:.1f} s excluded); full step = {full_step_samples} paths"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sd, spp_step, desc = workload(args.workload)
    import pyoracle
    pyoracle.build(ref=False)
    orc = pyoracle.OracleScene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    st = dict(max_bounces=sd.max_bounces, sampler=0)
    rng = np.random.default_rng(7)
    n0 = min(npix, 2048)
    pix = np.sort(rng.choice(npix, n0, replace=False)).astype(np.uint32)
    t0 = time.time()
    orc.render_paths(v, st, 0, spp_step, pixels=pix)
    dt0 = max(time.time() - t0, 1e-3)
    per_step_s = min(3.0, 60.0 / (args.steps + args.warmup))   # the whole run stays near a minute
    n = int(min(npix, max(256, n0 * per_step_s / dt0)))
    times = []
    for k in range(args.warmup + args.steps):
        pix = np.sort(rng.choice(npix, n, replace=False)).astype(np.uint32)
        t0 = time.time()
        orc.render_paths(v, st, k, spp_step, pixels=pix)
        dt = time.time() - t0
        if k >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = n * spp_step * len(times) / total / 1e6
    cores = int(pyoracle.lib().orc_num_threads())
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": desc, "step_sample": f"{n} random pixels x {spp_step} spp per step"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n} pixels x {spp_step} spp per step on {cores} host threads (OpenMP); "
                                       "the reference's GLSL integrator runs only through Vulkan RT, "
                                       "unavailable on this box, so its host restatement is timed"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Gates: the rest of the metric, measured in the default run after the
# headline (configs 3-5 and the FP64 comparison of every config). Each gate
# is CUDA-event timed on the render stream with its own clock record; all of
# them together stay within a few minutes on one GB300.
# ---------------------------------------------------------------------------
def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_steps(fn, warmup, steps, flush):
    """CUDA-event milliseconds of each of `steps` calls of fn(k) after
    `warmup` untimed calls; L2 flushed before every timed call."""
    import torch
    for k in range(warmup):
        fn(k)
    torch.cuda.synchronize()
    times = []
    for k in range(steps):
        flush.zero_()
        e0, e1 = _events()
        e0.record()
        fn(warmup + k)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times


def gate_batched(flush, warmup=3, steps=3):
    """Config 3: the 64-view instanced set through the per-view wavefront
    (plain) and the persistent multi-view pool (batched, launch shape chosen
    by the autotuner on the same views); equal RMSE is shown by equal
    images (bit identity of the two forms' accumulators)."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    t0 = time.time()
    sd = scenes.instanced()
    gen_s = time.time() - t0
    pt = og.PathTracer()
    t0 = time.time()
    pt.load_scene(sd)
    torch.cuda.synchronize()
    build_s = time.time() - t0
    spp = sd.spp
    accs = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in sd.views]
    total_px = sum(v.width * v.height for v in sd.views)

    def views_for(k):
        return [og.make_view(v, accum=a, history=k * spp) for v, a in zip(sd.views, accs)]

    def settings(k, mode):
        return og.make_settings(spp=spp, max_bounces=sd.max_bounces, sample_index_base=k * spp, mode=mode)

    t0 = time.time()
    tune_ms = pt.autotune(views_for(0), settings(0, og.MODE_PERSISTENT))
    tune_s = time.time() - t0
    out = {"workload": "instanced: 10,000 instances of 5 displaced geodesic spheres (362,500 base tris, two-level), "
                       f"64 views log-uniform 256..1024 ({total_px} pixels), {spp} spp, depth 4, PCG",
           "scene_gen_s": gen_s, "upload_and_build_s": build_s, "autotune_s": tune_s,
           "launch_config": pt.launch_config, "autotune_best_ms": tune_ms, "warmup": warmup, "steps": steps}
    for name, mode in (("plain", og.MODE_WAVEFRONT), ("batched", og.MODE_PERSISTENT)):
        clk = ClockSampler(0)
        clk.start()
        times = _time_steps(lambda k: pt.render(views_for(k), settings(k, mode)), warmup, steps, flush)
        out[name] = {"msamples_per_s": total_px * spp * steps / (sum(times) / 1e3) / 1e6,
                     "ms_per_step": sum(times) / steps, "clocks": clk.stop()}
    out["batched_over_plain"] = out["batched"]["msamples_per_s"] / out["plain"]["msamples_per_s"]
    pt.render(views_for(0), settings(0, og.MODE_WAVEFRONT))
    a_plain = [a.clone() for a in accs]
    pt.render(views_for(0), settings(0, og.MODE_PERSISTENT))
    out["bit_identical"] = bool(all(torch.equal(x, y) for x, y in zip(a_plain, accs)))
    pt.close()
    return out, sd


def gate_adjoint(flush, warmup=3, steps=3):
    """Config 4: one full gradient of the multi-view L2 loss (64x64x3 tile
    albedo map + 4 roughness regions, 8 views of 512^2, 16 spp, depth 3)
    through ohao_pt_adjoint, against coordinate finite differences (two
    renders of the 8 views per parameter, the reference fitter's method)
    timed with the same renderer."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    from ohao_engine_gb300.fit import AdjointFit
    sd = scenes.studio()
    train = sd.views[:8]
    pt = og.PathTracer()
    pt.load_scene(sd)
    tgt = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in train]
    pt.render([og.make_view(v, accum=a) for v, a in zip(train, tgt)],
              og.make_settings(spp=256, max_bounces=3, sample_index_base=1 << 20))
    rng = np.random.default_rng(2)
    init_map = np.clip(sd.albedo_map + rng.uniform(-0.4, 0.4, sd.albedo_map.shape), 0, 1).astype(np.float32)
    rough_ids = np.arange(4)
    mats0 = sd.materials.copy()
    mats0[rough_ids, 4] = np.clip(mats0[rough_ids, 4] + rng.uniform(-0.2, 0.2, 4), 0.05, 1.0).astype(np.float32)
    fit = AdjointFit(pt, mats0, init_map, train, tgt, spp=16, max_bounces=3, rough_ids=rough_ids, lr=0.03)
    n_params = int(fit.theta.size)
    npix = sum(v.width * v.height for v in train)
    acc = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in train]
    st16 = og.make_settings(spp=16, max_bounces=3, sample_index_base=0)
    clk = ClockSampler(0)
    clk.start()
    g_times = _time_steps(lambda k: pt.adjoint([og.make_view(v, accum=a) for v, a in zip(train, fit.accums)],
                                               fit.settings(k * 16), fit.targets, fit.gmap, fit.grough),
                          warmup, steps, flush)
    r_times = _time_steps(lambda k: pt.render([og.make_view(v, accum=a) for v, a in zip(train, acc)], st16),
                          warmup, steps, flush)
    clocks = clk.stop()
    t_grad = sum(g_times) / steps / 1e3
    t_render = sum(r_times) / steps / 1e3
    adj_rate = n_params / t_grad
    fd_rate = 1.0 / (2.0 * t_render)
    pt.close()
    return {"workload": f"studio: displaced sphere + plane ({sd.ntris} tris), 64x64x3 tile albedo map + 4 roughness "
                        "regions, 8 views 512x512, 16 spp, depth 3, PCG; targets 256 spp",
            "params": n_params, "paths_per_gradient": npix * 16, "warmup": warmup, "steps": steps,
            "adjoint_ms_per_gradient": t_grad * 1e3, "adjoint_param_gradients_per_s": adj_rate,
            "render_ms_8_views": t_render * 1e3, "coordinate_fd_param_gradients_per_s": fd_rate,
            "coordinate_fd_ms_per_gradient": 2 * n_params * t_render * 1e3,
            "adjoint_over_coordinate_fd": adj_rate / fd_rate, "clocks": clocks}, sd


# camera samples whose first-hit features the denoiser takes beside its
# 1-spp radiance
AOV_SPP = 8


def gate_denoiser(flush, n_scenes=20, iters=3000, crop=128, batch=8, variants=6, ref_spp=4096, aov_spp=AOV_SPP):
    """Config 5: the U-Net trained here by the library's own tcgen05
    kernels (bounded: n_scenes scenes x variants 1-spp renders against a
    1024-spp target, `iters` Adam steps), then judged on the 1920x1080
    headline frame against a ref_spp render: RMSE after the reference's
    display transform of the denoised 1-spp image and of plain accumulation,
    with CUDA-event wall time of each. The denoiser's first-hit inputs are
    the mean over aov_spp camera samples (ohao_pt_aov; 1: the 1-spp render's
    own record), their time counted in the denoised image's."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    from ohao_engine_gb300.denoise import Denoiser, render_pair, tonemap, training_scene
    t0 = time.time()
    side = 256
    data = []
    for seed in range(1, n_scenes + 1):
        sd = training_scene(seed, side=side, freq=64)
        pt = og.PathTracer()
        pt.load_scene(sd)
        pairs = [render_pair(pt, sd.views[0], side, side, 1, 1024 if k == 0 else 1, seed_base=4096 * k,
                             aov_spp=aov_spp)
                 for k in range(variants)]
        data.append(([p[0] for p in pairs], [p[1] for p in pairs], pairs[0][2]))
        pt.close()
    torch.cuda.synchronize()
    data_s = time.time() - t0
    dn = Denoiser(max_pixels=max(batch * crop * crop, 1920 * 1088), seed=1)
    rng = np.random.default_rng(0)

    def crop_of(t, ch, y0, x0):
        return t.view(side, side, ch)[y0:y0 + crop, x0:x0 + crop].contiguous().view(-1, ch)

    losses = []
    t0 = time.time()
    for it in range(iters):
        xs, aovs, ts = [], [], []
        for _ in range(batch):
            s = int(rng.integers(n_scenes))
            k = int(rng.integers(variants))
            y0, x0 = (int(v) for v in rng.integers(0, side - crop + 1, 2) // 16 * 16)
            xs.append(crop_of(data[s][0][k], 4, y0, x0))
            aovs.append(crop_of(data[s][1][k], og.AOV_FLOATS, y0, x0))
            ts.append(crop_of(data[s][2], 4, y0, x0))
        lr = 2e-3 * min(1.0, (it + 1) / 200.0) * (0.1 ** (it / iters))
        losses.append(dn.train_step(xs, aovs, ts, crop, crop, lr))
    torch.cuda.synchronize()
    train_s = time.time() - t0
    del data
    sd = scenes.sphere_1m()
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    ref = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    t0 = time.time()
    for k in range(ref_spp // 256):
        pt.render([og.make_view(v, accum=ref, history=k * 256)],
                  og.make_settings(spp=256, max_bounces=4, sample_index_base=(1 << 24) + k * 256))
    torch.cuda.synchronize()
    ref_s = time.time() - t0
    ref_ldr = tonemap(ref.cpu().numpy()[:, :3])

    def rmse(t):
        return float(np.sqrt(((tonemap(t.cpu().numpy()[:, :3]) - ref_ldr) ** 2).mean()))

    clk = ClockSampler(0)
    clk.start()
    plain = {}
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    for spp in (1, 4, 16, 64):
        ms = min(_time_steps(lambda k: pt.render([og.make_view(v, accum=acc)],
                                                 og.make_settings(spp=spp, max_bounces=4, sample_index_base=0)),
                             1, 3, flush))
        plain[str(spp)] = {"rmse": rmse(acc), "ms": ms}
    noisy = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    aov = torch.zeros((npix, og.AOV_FLOATS), dtype=torch.float32, device="cuda")
    out = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    def render_1spp(k):
        pt.render([og.make_view(v, accum=noisy, aov=aov if aov_spp <= 1 else None)],
                  og.make_settings(spp=1, max_bounces=4, sample_index_base=0))
        if aov_spp > 1:
            pt.aov(og.make_view(v), og.make_settings(spp=aov_spp, max_bounces=4, sample_index_base=1 << 19), aov)

    render_ms = min(_time_steps(render_1spp, 1, 3, flush))
    infer_ms = min(_time_steps(lambda k: dn.infer([noisy], [aov], [out], v.width, v.height), 2, 5, flush))
    clocks = clk.stop()
    den = rmse(out)
    matched = max([int(s) for s, r in plain.items() if r["rmse"] >= den], default=0)
    flops = 2.0 * 9 * sum(ci * co * (1920 * 1088) / 4 ** lv for ci, co, lv in (
        (12, 32, 0), (32, 32, 0), (32, 48, 1), (48, 48, 1), (48, 64, 2), (64, 64, 2), (64, 96, 3), (96, 96, 3),
        (96, 128, 4), (128, 128, 4), (224, 96, 3), (96, 96, 3), (160, 64, 2), (64, 64, 2), (112, 48, 1), (48, 48, 1),
        (80, 32, 0), (32, 32, 0), (32, 3, 0)))
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = float(json.load(open(pk)).get("bf16_tflops", 0)) if os.path.exists(pk) else 1900.0
    dn.close()
    res = {"workload": "U-Net 32/48/64/96/128 (BF16 tcgen05, FP32 accumulation) trained here: "
                       f"{n_scenes} scenes x 256^2 ({variants} x 1 spp vs 1024 spp), {iters} Adam steps of "
                       f"{batch}x{crop}^2 crops; judged on sphere_1m 1920x1080 against {ref_spp} spp; "
                       f"first-hit inputs averaged over {aov_spp} camera samples",
           "aov_spp": aov_spp,
           "training": {"data_s": data_s, "train_s": train_s, "iters": iters,
                        "loss_first100": float(np.mean(losses[:100])), "loss_last100": float(np.mean(losses[-100:]))},
           "reference_render_s": ref_s,
           "denoised": {"rmse": den, "render_1spp_ms": render_ms, "infer_ms": infer_ms,
                        "total_ms": render_ms + infer_ms},
           "plain": plain, "plain_spp_matched": matched,
           "meets_64spp": bool(den <= plain["64"]["rmse"] and render_ms + infer_ms < plain["64"]["ms"]),
           "infer_tflops": flops / (infer_ms / 1e3) / 1e12, "infer_frac_of_bf16_peak": flops / (infer_ms / 1e3) / 1e12 / peak,
           "clocks": clocks}
    return res, pt, sd, ref


def fp64_compare(og, pt, orc, view, spp, sample_base, pixels, settings):
    """GPU FP32 image (spp samples per pixel, progressive mean) against the
    FP64 host render of the same samples on `pixels`: relative RMSE of the
    per-pixel means, and the relative Monte-Carlo standard error of those
    means (the noise level the difference is to be read against)."""
    import torch
    npix = view.width * view.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    pt.render([og.make_view(view, accum=acc)], og.make_settings(spp=spp, sample_index_base=sample_base, **settings))
    g = acc.cpu().numpy()[pixels, :3].astype(np.float64)
    t0 = time.time()
    p64 = orc.render_paths(view, dict(settings, sampler=settings.get("sampler", 0)), sample_base, spp, pixels=pixels,
                           fp64=True)
    host_s = time.time() - t0
    m64 = p64.mean(axis=0)
    scale = float(np.sqrt((m64 ** 2).mean())) or 1.0
    rel = float(np.sqrt(((g - m64) ** 2).mean())) / scale
    se = float(np.sqrt((p64.var(axis=0, ddof=1) / spp).mean())) / scale if spp > 1 else None
    return {"pixels": int(pixels.size), "spp": spp, "rel_rmse_vs_fp64": rel, "rel_mc_stderr": se,
            "max_abs_diff": float(np.abs(g - m64).max()), "host_fp64_s": host_s}


def gate_fp64(headline_sd, instanced_sd, studio_sd, dn_pt, dn_sd, dn_ref):
    """Converged-image comparison against an FP64 host render for every
    config: the GPU's FP32 image and the host oracle instantiated in double,
    on the same samples (same PCG streams), over seeded pixel subsets."""
    import pyoracle
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    pyoracle.build(ref=False)
    out = {}
    rng = np.random.default_rng(99)

    def subset(v, n):
        npx = v.width * v.height
        return np.sort(rng.choice(npx, min(n, npx), replace=False)).astype(np.uint32)

    sd = scenes.cornell(256, 256, 16)
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    out["config1_cornell"] = fp64_compare(og, pt, pyoracle.OracleScene(sd), v, 16, 0,
                                          np.arange(v.width * v.height, dtype=np.uint32), dict(max_bounces=4))
    pt.close()
    sd = headline_sd
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    out["config2_sphere_1m"] = fp64_compare(og, pt, pyoracle.OracleScene(sd), v, 64, 0, subset(v, 8192),
                                            dict(max_bounces=4))
    pt.close()
    sd = instanced_sd
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = max(sd.views, key=lambda x: x.width * x.height)
    out["config3_instanced"] = fp64_compare(og, pt, pyoracle.OracleScene(sd), v, 16, 0, subset(v, 4096),
                                            dict(max_bounces=4))
    pt.close()
    sd = studio_sd
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    out["config4_studio"] = fp64_compare(og, pt, pyoracle.OracleScene(sd), v, 16, 0, subset(v, 8192),
                                         dict(max_bounces=3))
    pt.close()
    # the denoiser's 4096-spp reference frame (sphere_1m) against FP64 on the same samples
    v = dn_sd.views[0]
    pix = subset(v, 512)
    orc = pyoracle.OracleScene(dn_sd)
    t0 = time.time()
    p64 = np.zeros((len(pix), 3))
    for k in range(16):
        p64 += orc.render_paths(v, dict(max_bounces=4), (1 << 24) + k * 256, 256, pixels=pix, fp64=True).sum(axis=0)
    m64 = p64 / 4096.0
    g = dn_ref.cpu().numpy()[pix, :3].astype(np.float64)
    scale = float(np.sqrt((m64 ** 2).mean())) or 1.0
    out["config5_reference_frame"] = {"pixels": int(pix.size), "spp": 4096,
                                      "rel_rmse_vs_fp64": float(np.sqrt(((g - m64) ** 2).mean())) / scale,
                                      "max_abs_diff": float(np.abs(g - m64).max()), "host_fp64_s": time.time() - t0}
    dn_pt.close()
    return out


def run_gates(headline_sd, flush):
    res = {}
    t0 = time.time()
    res["config3_batched"], inst_sd = gate_batched(flush)
    res["config4_adjoint"], studio_sd = gate_adjoint(flush)
    res["config5_denoiser"], dn_pt, dn_sd, dn_ref = gate_denoiser(flush)
    res["fp64_rmse"] = gate_fp64(headline_sd, inst_sd, studio_sd, dn_pt, dn_sd, dn_ref)
    res["wall_s"] = time.time() - t0
    return res


def run_ours(args):
    import torch
    from ohao_engine_gb300 import replicas
    ranks = replicas.init("nccl")
    world, rank, local = ranks.world, ranks.rank, ranks.local
    torch.cuda.set_device(local)
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import _build
    if not os.path.exists(og.LIB_PATH):
        _build.build()
    og.load_library()
    sd, spp_step, desc = workload(args.workload)
    v = sd.views[0]
    npix = v.width * v.height
    pt = og.PathTracer(device=local)
    t0 = time.time()
    pt.load_scene(sd, build=False)
    torch.cuda.synchronize()
    t1 = time.time()
    pt.build()
    build_s = time.time() - t1
    upload_s = t1 - t0
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB > L2

    order = og.FLAG_SORT_MATERIAL if args.shade_order == "material" else 0

    def step(k, flags=0):
        s = og.make_settings(spp=spp_step, max_bounces=sd.max_bounces, sample_index_base=k * spp_step,
                             sampler=og.SAMPLER_PCG, flags=flags | order)
        pt.render([og.make_view(v, accum=acc, history=k * spp_step)], s)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    times = []
    replicas.barrier(ranks)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        step(args.warmup + k)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    replicas.barrier(ranks)
    clocks = clk.stop()
    total_ms = replicas.max_over_ranks(ranks, float(sum(times)))
    value = replicas.whole_job_rate(npix * spp_step * args.steps, ranks, total_ms / 1e3) / 1e6

    # profiled pass: per-kernel CUDA events + traversal visit counters
    prof_ms = []
    lanes = 1
    for k in range(args.steps):
        flush.zero_()
        step(args.warmup + args.steps + k, flags=og.FLAG_PROFILE)
        p = pt.profile()
        lanes = max(lanes, int(p.lanes))
        prof_ms.append((p.extend_ms, p.extend_launches, p.nodes_closest, p.tris_closest, p.shadow_ms,
                        p.shadow_launches, p.nodes_shadow, p.tris_shadow, p.shade_ms, p.other_ms, p.total_ms,
                        p.shade_launches, p.other_launches, p.rays_closest, p.rays_shadow))
    torch.cuda.synchronize()
    ext_ms = sum(x[0] for x in prof_ms)
    ext_launches = sum(x[1] for x in prof_ms)
    ext_bytes = sum(80 * x[2] + 48 * x[3] for x in prof_ms)
    sh_ms = sum(x[4] for x in prof_ms)
    sh_bytes = sum(80 * x[6] + 48 * x[7] for x in prof_ms)
    # the timed steps run `lanes` pixel lanes, each with the profiled pass's kernel sequence
    launches_per_step = lanes * (sum(x[1] + x[5] + x[11] + x[12] for x in prof_ms)) / len(prof_ms)
    rays_c = sum(x[13] for x in prof_ms)
    rays_s = sum(x[14] for x in prof_ms)
    peak, peak_kind = peaks()
    achieved = ext_bytes / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else 0.0
    traffic, tnote = traffic_from_profiles("k_extend", args.workload)
    roofline = {"bound": "hbm", "kernel": "k_extend (closest-hit traversal)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic,
                "algorithmic_bytes_per_launch": ext_bytes / max(ext_launches, 1),
                "avg_launch_ms": ext_ms / max(ext_launches, 1),
                "bytes_model": "80 B per 8-wide node visited + 48 B per triangle tested, counted on the device",
                "shadow_kernel_GBps": sh_bytes / (sh_ms / 1e3) / 1e9 if sh_ms > 0 else 0.0,
                "closest_rays_per_s": rays_c / (ext_ms / 1e3) if ext_ms > 0 else 0.0,
                "shadow_rays_per_s": rays_s / (sh_ms / 1e3) if sh_ms > 0 else 0.0,
                "kernel_share": {"extend": ext_ms, "shadow": sh_ms, "shade": sum(x[8] for x in prof_ms),
                                 "other": sum(x[9] for x in prof_ms), "total_ms": sum(x[10] for x in prof_ms)}}
    if tnote:
        roofline["traffic_note"] = tnote

    # end to end through the host-buffer C-ABI call
    host = torch.zeros((npix, 4), dtype=torch.float32).pin_memory()
    hnp = host.numpy()
    e2e_times = []
    base = 2 * args.steps + args.warmup
    s0 = og.make_settings(spp=spp_step, max_bounces=sd.max_bounces, sample_index_base=0, sampler=og.SAMPLER_PCG,
                          flags=order)
    pt.render_host([og.make_view(v, history=0)], s0, [hnp])
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s = og.make_settings(spp=spp_step, max_bounces=sd.max_bounces, sample_index_base=(base + k) * spp_step,
                             sampler=og.SAMPLER_PCG, flags=order)
        t0 = time.perf_counter()
        pt.render_host([og.make_view(v, history=1 + k * spp_step)], s, [hnp])
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = replicas.whole_job_rate(npix * spp_step * args.steps, ranks, sum(e2e_times)) / 1e6
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": npix * 16, "d2h_bytes_per_step": npix * 16,
           "call": "ohao_pt_render_host (pinned host accumulator in and out)"}

    gates = None
    if rank == 0 and world == 1 and not args.no_gates and args.workload == "sphere_1m":
        gates = run_gates(sd, flush)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sd, spp_step, args.cpu_seconds, npix * spp_step)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": desc, "l2": "flushed between timed steps (256 MB write)",
                           "path": "plain wavefront", "parallelism": f"replicas x{world}",
                           "shade_order": args.shade_order,
                           "pixel_lanes": lanes, "shadow_rays": "beside the next step's closest-hit rays (second stream)",
                           "bvh_build_s": build_s, "scene_upload_s": upload_s,
                           "rays_per_step": {"closest": rays_c / len(prof_ms), "shadow": rays_s / len(prof_ms)}},
                "clocks": clocks, "e2e": e2e, "gpu_launches": int(round(launches_per_step * args.steps)),
                "roofline": roofline, "cpu_baseline": cpu}
        if gates is not None:
            line["gates"] = gates
        print(json.dumps(line), flush=True)
    pt.close()
    replicas.finish(ranks)


def run_instanced(args):
    """Batched multi-view workload: 10,000 instances of 5 displaced geodesic
    spheres (362,500 base triangles, two-level TLAS/BLAS), 64 views with
    log-uniform sides in [256, 1024], 4 spp, depth 4. The same steps are
    timed for the plain per-view wavefront and the persistent multi-view
    kernel (after its autotuner picked a launch shape); both produce
    bit-identical images, so RMSE is equal by construction."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import _build, scenes
    torch.cuda.set_device(0)
    if not os.path.exists(og.LIB_PATH):
        _build.build()
    og.load_library()
    t0 = time.time()
    sd = scenes.instanced()
    gen_s = time.time() - t0
    pt = og.PathTracer(device=0)
    t0 = time.time()
    pt.load_scene(sd)
    torch.cuda.synchronize()
    build_s = time.time() - t0
    spp = sd.spp
    accs = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in sd.views]
    total_px = sum(v.width * v.height for v in sd.views)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def views_for(k):
        return [og.make_view(v, accum=a, history=k * spp) for v, a in zip(sd.views, accs)]

    def settings(k, mode, flags=0):
        return og.make_settings(spp=spp, max_bounces=sd.max_bounces, sample_index_base=k * spp,
                                sampler=og.SAMPLER_PCG, flags=flags, mode=mode)

    tune_ms = pt.autotune(views_for(0), settings(0, og.MODE_PERSISTENT))
    results = {}
    for name, mode in (("plain", og.MODE_WAVEFRONT), ("batched", og.MODE_PERSISTENT)):
        for k in range(args.warmup):
            pt.render(views_for(k), settings(k, mode))
        torch.cuda.synchronize()
        clk = ClockSampler(0)
        clk.start()
        times = []
        for k in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            pt.render(views_for(args.warmup + k), settings(args.warmup + k, mode))
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        clocks = clk.stop()
        tot = sum(times)
        results[name] = {"value": total_px * spp * args.steps / (tot / 1e3) / 1e6, "ms_per_step": tot / args.steps,
                         "clocks": clocks}
    # bit-identity of the two forms on one step
    ref = [a.clone() for a in accs]
    pt.render(views_for(0), settings(0, og.MODE_WAVEFRONT))
    a_plain = [a.clone() for a in accs]
    pt.render(views_for(0), settings(0, og.MODE_PERSISTENT))
    identical = all(torch.equal(x, y) for x, y in zip(a_plain, accs))
    del ref
    # end to end with host buffers (batched form)
    hosts = [torch.zeros((v.width * v.height, 4), dtype=torch.float32).pin_memory().numpy() for v in sd.views]
    e2e_t = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pt.render_host([og.make_view(v, history=0) for v in sd.views], settings(k, og.MODE_PERSISTENT), hosts)
        e2e_t.append(time.perf_counter() - t0)
    e2e = {"value": total_px * spp * args.steps / sum(e2e_t) / 1e6, "unit": UNIT, "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": total_px * 16, "call": "ohao_pt_render_host, 64 views (host accumulators out)"}
    line = {"metric": METRIC, "value": results["batched"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": results["batched"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "instanced: 10,000 instances of 5 displaced geodesic spheres (362,500 base tris, "
                                   "two-level), 64 views log-uniform 256..1024, 4 spp, depth 4, PCG",
                       "pixels": total_px, "l2": "flushed between timed steps (256 MB write)",
                       "scene_gen_s": gen_s, "upload_and_build_s": build_s,
                       "launch_config": pt.launch_config, "autotune_best_ms": tune_ms},
            "plain": results["plain"], "batched": results["batched"],
            "batched_over_plain": results["batched"]["value"] / results["plain"]["value"],
            "bit_identical": bool(identical), "clocks": results["batched"]["clocks"], "e2e": e2e}
    print(json.dumps(line), flush=True)
    pt.close()


def run_studio(args, fit_iters=80):
    """Differentiable inverse fit: 200k-tri displaced sphere on a plane, 64x64
    tile albedo map + 4 roughness regions, 8 train + 2 holdout views at
    512x512, targets at 256 spp, gradient at 16 spp depth 3. A step is one
    full gradient (12,288 map entries + 5 roughness values) of the multi-view
    L2 loss through ohao_pt_adjoint. The coordinate-FD rate that it replaces
    is 2 renders of the 8 train views per parameter, timed on the same GPU
    with the same renderer."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import _build, scenes
    from ohao_engine_gb300.fit import AdjointFit
    torch.cuda.set_device(0)
    if not os.path.exists(og.LIB_PATH):
        _build.build()
    og.load_library()
    sd = scenes.studio()
    train, hold = sd.views[:8], sd.views[8:]
    pt = og.PathTracer(device=0)
    pt.load_scene(sd)
    ntris = sd.ntris
    # ground-truth targets at 256 spp
    tgt = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in sd.views]
    st_t = og.make_settings(spp=256, max_bounces=3, sample_index_base=1 << 20, sampler=og.SAMPLER_PCG)
    pt.render([og.make_view(v, accum=a) for v, a in zip(sd.views, tgt)], st_t)
    torch.cuda.synchronize()
    rng = np.random.default_rng(2)
    gt_map = sd.albedo_map.copy()
    init_map = np.clip(gt_map + rng.uniform(-0.4, 0.4, gt_map.shape), 0.0, 1.0).astype(np.float32)
    rough_ids = np.arange(4)
    gt_rough = sd.materials[rough_ids, 4].copy()
    mats0 = sd.materials.copy()
    mats0[rough_ids, 4] = np.clip(gt_rough + rng.uniform(-0.2, 0.2, 4), 0.05, 1.0).astype(np.float32)
    fit = AdjointFit(pt, mats0, init_map, train, tgt[:8], spp=16, max_bounces=3, rough_ids=rough_ids, lr=0.03)
    n_params = fit.theta.size
    npix = sum(v.width * v.height for v in train)
    st16 = og.make_settings(spp=16, max_bounces=3, sample_index_base=0, sampler=og.SAMPLER_PCG)
    acc = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in train]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    # timed: full gradients (render + loss + backward)
    for k in range(args.warmup):
        fit.gradient(sample_base=k * 16)
    torch.cuda.synchronize()
    clk = ClockSampler(0)
    clk.start()
    g_times = []
    for k in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        vs = [og.make_view(v, accum=a) for v, a in zip(train, fit.accums)]
        pt.adjoint(vs, fit.settings((args.warmup + k) * 16), fit.targets, fit.gmap, fit.grough)
        e1.record()
        e1.synchronize()
        g_times.append(e0.elapsed_time(e1))
    clocks = clk.stop()
    # the forward render alone (what coordinate FD repeats twice per parameter)
    r_times = []
    for k in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        pt.render([og.make_view(v, accum=a) for v, a in zip(train, acc)], st16)
        e1.record()
        e1.synchronize()
        r_times.append(e0.elapsed_time(e1))
    t_grad = sum(g_times) / len(g_times) / 1e3
    t_render = sum(r_times) / len(r_times) / 1e3
    adj_rate = n_params / t_grad
    fd_rate = 1.0 / (2.0 * t_render)
    # end to end: targets uploaded from pinned host memory, gradients read back, every step
    host_t = [t.cpu().pin_memory() for t in tgt[:8]]
    host_g = torch.zeros(fit.gmap.numel() + fit.grough.numel(), dtype=torch.float32).pin_memory()
    e2e_t = []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for d, h in zip(fit.targets, host_t):
            d.copy_(h, non_blocking=True)
        vs = [og.make_view(v, accum=a) for v, a in zip(train, fit.accums)]
        pt.adjoint(vs, fit.settings(k * 16), fit.targets, fit.gmap, fit.grough)
        host_g[:fit.gmap.numel()].copy_(fit.gmap, non_blocking=True)
        host_g[fit.gmap.numel():].copy_(fit.grough, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    t_e2e = sum(e2e_t) / len(e2e_t)
    # the fit itself
    def holdout_loss():
        hacc = [torch.zeros((v.width * v.height, 4), dtype=torch.float32, device="cuda") for v in hold]
        pt.render([og.make_view(v, accum=a) for v, a in zip(hold, hacc)],
                  og.make_settings(spp=64, max_bounces=3, sample_index_base=1 << 24, sampler=og.SAMPLER_PCG))
        return float(np.mean([((a[:, :3] - t[:, :3]) ** 2).mean().item() for a, t in zip(hacc, tgt[8:])]))
    map_rmse0 = float(np.sqrt(((fit.albedo_map - gt_map) ** 2).mean()))
    hold0 = holdout_loss()
    losses = []
    t0 = time.time()
    for _ in range(fit_iters):
        losses.append(fit.step())
    fit_s = time.time() - t0
    map_rmse1 = float(np.sqrt(((fit.albedo_map - gt_map) ** 2).mean()))
    hold1 = holdout_loss()
    line = {"metric": "gradients/s of the multi-view L2 loss (path-replay adjoint) vs coordinate-FD gradients/s",
            "value": adj_rate, "unit": "parameter-gradients/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_grad * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"studio: displaced sphere + plane ({ntris} tris), 64x64 tile albedo map, "
                                   "4 roughness regions, 8 train views 512x512, gradient at 16 spp depth 3, PCG; "
                                   "targets 256 spp", "params": int(n_params),
                       "l2": "flushed between timed steps (256 MB write)"},
            "adjoint": {"ms_per_gradient": t_grad * 1e3, "param_gradients_per_s": adj_rate,
                        "paths_per_gradient": npix * 16},
            "coordinate_fd": {"render_ms_8_views": t_render * 1e3, "param_gradients_per_s": fd_rate,
                              "renders_per_gradient": 2 * int(n_params),
                              "ms_per_gradient": 2 * n_params * t_render * 1e3},
            "adjoint_over_fd": adj_rate / fd_rate,
            "fit": {"iterations": fit_iters, "seconds": fit_s, "optimizer": "Adam lr 0.03, decorrelated replay",
                    "roughness_init": [float(x) for x in mats0[rough_ids, 4]], "loss_first": losses[0], "loss_last": losses[-1],
                    "map_rmse_init": map_rmse0, "map_rmse_final": map_rmse1, "holdout_mse_init": hold0,
                    "holdout_mse_final": hold1, "roughness_gt": [float(x) for x in gt_rough],
                    "roughness_final": [float(x) for x in fit.roughness]},
            "clocks": clocks,
            "e2e": {"value": n_params / t_e2e, "unit": "parameter-gradients/s",
                    "h2d_bytes_per_step": int(sum(t.numel() * 4 for t in host_t)),
                    "d2h_bytes_per_step": int(host_g.numel() * 4),
                    "call": "ohao_pt_adjoint (targets from pinned host memory, gradients back to host)"}}
    print(json.dumps(line), flush=True)
    pt.close()


def run_denoise(args, n_scenes=50, iters=10000, crop=128, batch=8, variants=6):
    """Learned denoiser: the U-Net (tcgen05 BF16 convolutions, FP32
    accumulation) is trained on this GPU by the library's own kernels on
    1-spp / 1024-spp pairs of 256x256 renders of n_scenes seeded scenes of
    the single-object family (random crops of crop^2), then judged on the
    1920x1080 headline scene against a 4096-spp render: RMSE after the
    reference's display transform for the denoised 1-spp image and for plain
    accumulation at 1..256 spp, with the wall time of each."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import _build, scenes
    from ohao_engine_gb300.denoise import Denoiser, render_pair, tonemap, training_scene
    torch.cuda.set_device(0)
    if not os.path.exists(og.LIB_PATH):
        _build.build()
    og.load_library()
    t0 = time.time()
    side = 256
    data = []
    for seed in range(1, n_scenes + 1):
        sd = training_scene(seed, side=side, freq=64)
        pt = og.PathTracer()
        pt.load_scene(sd)
        pairs = [render_pair(pt, sd.views[0], side, side, 1, 1024 if k == 0 else 1, seed_base=4096 * k)
                 for k in range(variants)]
        ref = pairs[0][2]
        data.append(([p[0] for p in pairs], [p[1] for p in pairs], ref))
        pt.close()
    torch.cuda.synchronize()
    data_s = time.time() - t0
    dn = Denoiser(max_pixels=max(batch * crop * crop, 1920 * 1088), seed=1)
    rng = np.random.default_rng(0)

    def crop_of(t, ch, y0, x0):
        return t.view(side, side, ch)[y0:y0 + crop, x0:x0 + crop].contiguous().view(-1, ch)

    losses = []
    t0 = time.time()
    for it in range(iters):
        xs, aovs, ts = [], [], []
        for _ in range(batch):
            s = int(rng.integers(n_scenes))
            k = int(rng.integers(variants))
            y0, x0 = (int(v) for v in rng.integers(0, side - crop + 1, 2) // 16 * 16)
            xs.append(crop_of(data[s][0][k], 4, y0, x0))
            aovs.append(crop_of(data[s][1][k], og.AOV_FLOATS, y0, x0))
            ts.append(crop_of(data[s][2], 4, y0, x0))
        lr = 2e-3 * min(1.0, (it + 1) / 200.0) * (0.1 ** (it / iters))   # 200-step warm-up, then decay
        losses.append(dn.train_step(xs, aovs, ts, crop, crop, lr))
    torch.cuda.synchronize()
    train_s = time.time() - t0
    del data
    # evaluate on the headline scene
    sd = scenes.sphere_1m()
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    ref = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    for k in range(16):   # 4096 spp in 16 progressive calls
        pt.render([og.make_view(v, accum=ref, history=k * 256)],
                  og.make_settings(spp=256, max_bounces=4, sample_index_base=(1 << 24) + k * 256))
    ref_ldr = tonemap(ref.cpu().numpy()[:, :3])

    def rmse(t):
        return float(np.sqrt(((tonemap(t.cpu().numpy()[:, :3]) - ref_ldr) ** 2).mean()))

    def timed(fn, reps=3):
        best = 1e30
        for _ in range(reps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    plain = {}
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    for spp in (1, 4, 16, 64, 256):
        ms = timed(lambda: pt.render([og.make_view(v, accum=acc)],
                                     og.make_settings(spp=spp, max_bounces=4, sample_index_base=0)))
        plain[str(spp)] = {"rmse": rmse(acc), "ms": ms}
    noisy = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    aov = torch.zeros((npix, og.AOV_FLOATS), dtype=torch.float32, device="cuda")
    out = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    render_ms = timed(lambda: pt.render([og.make_view(v, accum=noisy, aov=aov)],
                                        og.make_settings(spp=1, max_bounces=4, sample_index_base=0)))
    infer_ms = timed(lambda: dn.infer([noisy], [aov], [out], v.width, v.height), reps=5)
    den_rmse = rmse(out)
    matched = max([int(s) for s, r in plain.items() if r["rmse"] >= den_rmse], default=0)
    flops = 2.0 * 9 * sum(ci * co * (1920 * 1088) / 4 ** lv for ci, co, lv in (
        (12, 32, 0), (32, 32, 0), (32, 48, 1), (48, 48, 1), (48, 64, 2), (64, 64, 2), (64, 96, 3), (96, 96, 3),
        (96, 128, 4), (128, 128, 4), (224, 96, 3), (96, 96, 3), (160, 64, 2), (64, 64, 2), (112, 48, 1), (48, 48, 1),
        (80, 32, 0), (32, 32, 0), (32, 3, 0)))
    peak = None
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peak = float(json.load(open(pk)).get("bf16_tflops", 0)) or None
    achieved = flops / (infer_ms / 1e3) / 1e12
    line = {"metric": "denoised 1-spp RMSE and wall time vs plain accumulation (1920x1080, vs 4096 spp)",
            "value": den_rmse, "unit": "RMSE (display-transformed)", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": render_ms + infer_ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 (FP32 accumulation)", "data": "synthetic (seeded)",
            "config": {"workload": "U-Net 32/48/64/96/128, 12-ch input (albedo-demodulated radiance, albedo, normal, "
                                   "inverse depth, roughness, metallic); trained on "
                                   f"{n_scenes} scenes x 256^2 (1 spp x{variants} vs 1024 spp), {iters} Adam steps "
                                   f"of {batch}x{crop}^2 crops, L1 on log demodulated radiance + L1 after the display "
                                   "transform; judged on sphere_1m 1920x1080"},
            "denoised": {"rmse": den_rmse, "render_1spp_ms": render_ms, "infer_ms": infer_ms,
                         "total_ms": render_ms + infer_ms},
            "plain": plain, "plain_spp_matched": matched,
            "beats_64spp": bool(den_rmse <= plain["64"]["rmse"] and render_ms + infer_ms < plain["64"]["ms"]),
            "training": {"data_s": data_s, "train_s": train_s, "iters": iters, "loss_first100": float(np.mean(losses[:100])),
                         "loss_last100": float(np.mean(losses[-100:])), "ms_per_iter": train_s / iters * 1e3},
            "roofline": {"bound": "tensor", "kernel": "k_conv (forward, whole U-Net inference)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if peak else None, "flops_per_frame": flops}}
    print(json.dumps(line), flush=True)
    pt.close()


# ---------------------------------------------------------------------------
# Small profiling cases (bench.py --case NAME): self-contained runs of one
# GPU path for ncu captures, each printing its CUDA-event time per call.
# ---------------------------------------------------------------------------
def _timed_calls(fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def case_denoise_infer(arg):
    """U-Net inference at 1920x1080 on seeded inputs (3 + 10 calls)."""
    import torch
    from ohao_engine_gb300.denoise import Denoiser
    w, h = 1920, 1080
    rng = np.random.default_rng(0)
    rad = torch.from_numpy(rng.exponential(0.5, (w * h, 4)).astype(np.float32)).cuda()
    aov = torch.from_numpy(rng.random((w * h, 12)).astype(np.float32)).cuda()
    out = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    dn = Denoiser(max_pixels=1920 * 1088, seed=1)
    for _ in range(3):
        dn.infer([rad], [aov], [out], w, h)
    ms = _timed_calls(lambda: dn.infer([rad], [aov], [out], w, h), 10)
    print(f"denoise_infer 1920x1080: {ms:.3f} ms per call")


def case_adjoint(arg):
    """ohao_pt_adjoint on the studio scene, one 256^2 view, 4 spp (2 calls)."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    sd = scenes.studio(n_train=1, n_holdout=0, side=256)
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    tgt = torch.full((npix, 4), 0.3, device="cuda")
    acc = torch.zeros((npix, 4), device="cuda")
    gm = torch.zeros(sd.albedo_map.size, device="cuda")
    gr = torch.zeros(sd.materials.shape[0], device="cuda")
    s = og.make_settings(spp=4, max_bounces=3, flags=og.FLAG_ADJOINT_DECORRELATE)
    ms = _timed_calls(lambda: pt.adjoint([og.make_view(v, accum=acc)], s, [tgt], gm, gr), 2)
    print(f"adjoint studio 256^2 x 4 spp: {ms:.3f} ms per call")


def case_instanced_view(arg):
    """One 512^2 view of the instanced scene, 4 spp, per-view wavefront (3 calls)."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    sd = scenes.instanced(n_views=1, side_range=(512, 512))
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    acc = torch.zeros((v.width * v.height, 4), device="cuda")
    s = og.make_settings(spp=4, max_bounces=4, mode=og.MODE_WAVEFRONT)
    ms = _timed_calls(lambda: pt.render([og.make_view(v, accum=acc)], s), 3)
    print(f"instanced one 512^2 view x 4 spp: {ms:.3f} ms per call")


def case_instanced_pool(arg):
    """Four 384^2 views of the instanced scene, 4 spp, persistent pool (2 calls)."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    sd = scenes.instanced(n_views=4, side_range=(384, 384))
    pt = og.PathTracer()
    pt.load_scene(sd)
    pt.launch_config = arg or "pool_4M_unsorted_fetch4_chunk8"
    accs = [torch.zeros((v.width * v.height, 4), device="cuda") for v in sd.views]
    s = og.make_settings(spp=4, max_bounces=4, mode=og.MODE_PERSISTENT)
    ms = _timed_calls(lambda: pt.render([og.make_view(v, accum=a) for v, a in zip(sd.views, accs)], s), 2)
    print(f"instanced 4 views 384^2 x 4 spp, {pt.launch_config}: {ms:.3f} ms per call")


def case_emitter_mis(arg):
    """Emitter MIS on scenes.emitters (512x320, glossy floor of roughness
    0.25, an area and a sphere light): for the reference estimator and with
    OHAO_PT_FLAG_EMITTER_MIS, CUDA-event ms per 4-spp frame and the
    per-pixel variance of one path (64 paths per pixel; mean and median
    over the pixels)."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    sd = scenes.emitters(width=512, height=320, floor_rough=0.25)
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    paths = torch.zeros((64, npix, 4), dtype=torch.float32, device="cuda")
    stats = {}
    for name, flags in (("reference", 0), ("emitter MIS", og.FLAG_EMITTER_MIS)):
        pt.render([og.make_view(v, accum=acc, path_radiance=paths)],
                  og.make_settings(spp=64, max_bounces=4, flags=flags, sample_index_base=1 << 16))
        var = paths[..., :3].var(dim=0).sum(-1)
        mean = paths[..., :3].mean(dim=0)
        ms = _timed_calls(lambda: pt.render([og.make_view(v, accum=acc)], og.make_settings(spp=4, max_bounces=4,
                                                                                          flags=flags)), 10)
        stats[name] = (float(var.mean()), float(var.median()), mean)
        print(f"{name:12s}: {ms:.3f} ms per 4-spp frame; per-pixel path variance mean {stats[name][0]:.3f} "
              f"median {stats[name][1]:.4f}")
    r, m = stats["reference"], stats["emitter MIS"]
    print(f"variance ratio (reference / MIS): mean {r[0] / m[0]:.2f}, median {r[1] / m[1]:.2f}; mean radiance "
          f"{float(r[2].mean()):.4f} / {float(m[2].mean()):.4f}")


def case_traversal_shapes(arg):
    """Per-view wavefront on sphere_1m (1920x1080, 1 spp, depth 4) in each
    traversal shape -- one ray per thread, or persistent warps refilled at
    1-32 idle lanes -- and queue order (queue order, material-binned
    shading, ray-binned bounces); CUDA-event ms per frame (3 warm-up, 20
    timed, L2 flushed), and the images' bit identity."""
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import scenes
    sd = scenes.sphere_1m() if arg != "instanced" else scenes.instanced(n_views=1, side_range=(1024, 1024))
    pt = og.PathTracer()
    pt.load_scene(sd)
    v = sd.views[0]
    npix = v.width * v.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ref = None
    m, r = og.FLAG_SORT_MATERIAL, og.FLAG_SORT_RAYS
    for refill, flags in ((33, 0), (33, m), (33, r), (1, 0), (4, 0), (8, 0), (16, 0), (24, 0), (32, 0), (16, m),
                          (24, m), (32, m)):
        st = og.make_settings(spp=1, max_bounces=4, wavefront_refill=refill, flags=flags)
        times = _time_steps(lambda k: pt.render([og.make_view(v, accum=acc)], st), 3, 20, flush)
        same = True
        if ref is None:
            ref = acc.clone()
        else:
            same = bool(torch.equal(acc, ref))
        pt.render([og.make_view(v, accum=acc)], og.make_settings(spp=1, max_bounces=4, wavefront_refill=refill,
                                                                 flags=og.FLAG_PROFILE | flags))
        p = pt.profile()
        order = ("material " if flags & m else "") + ("rays " if flags & r else "") or "queue "
        print(f"refill {refill:2d} order {order:15s}: {sum(times) / len(times):.3f} ms/frame  extend "
              f"{p.extend_ms:.3f} ms shadow {p.shadow_ms:.3f} ms shade {p.shade_ms:.3f} ms other {p.other_ms:.3f} ms  "
              f"identical={same}")


CASES = {"traversal_shapes": case_traversal_shapes, "denoise_infer": case_denoise_infer, "adjoint": case_adjoint, "instanced_view": case_instanced_view,
         "instanced_pool": case_instanced_pool, "emitter_mis": case_emitter_mis}


def run_case(args):
    import torch
    import ohao_engine_gb300 as og
    from ohao_engine_gb300 import _build
    torch.cuda.set_device(0)
    if not os.path.exists(og.LIB_PATH):
        _build.build()
    og.load_library()
    CASES[args.case](args.case_arg)


def main():
    args = parse()
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "instanced":
        run_instanced(args)
    elif args.workload == "studio":
        run_studio(args)
    elif args.workload == "denoise":
        run_denoise(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
