#!/usr/bin/env python
"""Throughput benchmark of the GB300 path tracer (forward trace).

Workload (the largest single-GPU configuration of the headline metric):
c1 -- 1920x1080, 16 spp, max depth 8, Russian roulette from depth 3, a
100k-triangle soup (centroids U[-50,50]^3, vertices + N(0, 0.5^2)), 256
materials, 16-bin SAH BVH with leaf size 4, sky 1.0, seed 1.  Synthetic data.

A step is one trace of the full frame.  `value` is Mrays/s with the scene
resident in HBM (one ray = one trace_ray call, closest-hit or shadow, counted
on the device); `e2e` is the same metric through the public C ABI with host
buffers (FrameData in, RGBA8 image out to pinned host memory) inside the timed
region.  L2 is flushed (256 MiB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: one process per GPU (torchrun); every rank traces its own frame
(independent seeds), so per-GPU work is fixed: weak scaling, no data-path
collective.  --impl reference times the CPU restatement of the reference
shader (oracle/, with the same BVH) on the host cores.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "vk-renderer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "Mrays/s on 1 GB300 (fwd, adjoint, batched) at ≤1e-3 RMSE vs plain trace"
UNIT = "Mrays/s"
L2_FLUSH_BYTES = 256 << 20

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per ray of the
# 8-wide extend kernel, from one ncu capture of every extend launch of two
# whole c1 frames (1920x1080, 16 spp, finishing kernel off so that every ray
# goes through it: 3.816 GB read + 0.26 GB written per frame of 67.6 M rays;
# profiles/wf_extend_cw8_c1_dram.md); the frame's traffic is this times its
# rays.
NCU_EXTEND_DRAM_BYTES_PER_RAY = 60.3

# DRAM bytes of one replay of the c2 batch's graph (the bench's tuned shape:
# 8-wide, 256 threads, hand-over at 1M paths), from one ncu capture of every
# kernel of four replays (profiles/batch_c2_graph_launches.md): the extend
# kernel's (21.4 GB read + 2.45 GB written) and all kernels' (42.0 + 14.5 GB;
# wf_shade 20.4 + 9.8 GB).  The 2.1M triangles' 64-byte records and nodes
# exceed L2, unlike c1's.
NCU_BATCH_EXTEND_DRAM_BYTES = 23.85e9
NCU_BATCH_ALL_DRAM_BYTES = 56.45e9


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        self.proc.wait()
        self.f.flush()
        with open(self.f.name) as fh:
            rows = [r.split(",") for r in fh.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for k, n in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(st: dict, pixels: int, out_bytes_per_pixel: int) -> int:
    """Bytes one trace must read/write by definition: 32 B per BVH node record
    fetched, 48 B per triangle and 64 B per sphere/plane tested, 48 B material
    per closest hit, plus the image written."""
    return (32 * st["node_fetches"] + 48 * st["tri_tests"] + 64 * st["sphere_tests"] + 64 * st["plane_tests"]
            + 48 * st["hits"] + out_bytes_per_pixel * pixels)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_seed(seed: float, rank: int) -> float:
    """Weak scaling: every rank traces its own frame (the reference draws a
    new seed per frame, GraphicsDevice.cpp:1262)."""
    return float(seed) + 0.125 * rank


def aggregate(world: int, rays: float, seconds: float, device: str = "cuda"):
    """Whole-job throughput: all ranks' rays over the slowest rank's time.
    Returns (Mrays/s, max seconds, total rays).  One collective each for the
    max and the sum; nothing on the data path."""
    if world == 1:
        return rays / seconds / 1e6, seconds, rays
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    r = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(r, op=dist.ReduceOp.SUM)
    return r.item() / t.item() / 1e6, t.item(), r.item()


TRAVERSAL_LABEL = {0: "auto (= compressed 8-wide for triangle-only scenes)", 2: "binary", 4: "4-wide",
                   8: "compressed 8-wide"}


def workload_config(wl, world: int) -> dict:
    """The `config` both arms print (identical dicts): the workload and its
    sizes.  Arm-specific launch details go under `impl_config`."""
    return {"workload": wl.name, "width": wl.width, "height": wl.height, "spp": wl.spp,
            "max_depth": wl.max_depth, "rr_start": wl.rr_start, "triangles": int(len(wl.scene.triangles)),
            "materials": int(len(wl.scene.materials)), "bvh": "sah16-leaf4",
            "l2": "GPU arm: flushed before each timed step (256 MiB write)",
            "parallelism": f"replicas x{world} (independent frames)"}


def parity_summary(gpu: dict, ora: dict, rows) -> dict:
    """Parity of a GPU frame against the oracle's on the oracle's rows:
    primary-hit id mismatches (those not explained by a tie within 1e-6 in
    t), the largest relative t difference of equal ids, the float image's
    RMSE without column 0 (NaN by construction), and whether column 0 is NaN
    in the same places."""
    import numpy as np
    r = np.arange(*rows)
    gid, oid = gpu["hit_id"][r], ora["hit_id"][r]
    gt, ot = gpu["hit_t"][r], ora["hit_t"][r]
    mism = gid != oid
    ties = mism & (np.abs(gt - ot) <= 1e-6)
    both = (gid == oid) & (gid != 0xFFFFFFFF)
    rel = np.abs(gt[both] - ot[both]) / np.maximum(np.abs(ot[both]), 1e-30)
    a = gpu["rgba32f"][r][:, 1:, :3].astype(np.float64)
    b = ora["rgba32f"][r][:, 1:, :3].astype(np.float64)
    return {"rows": f"{len(r)} of {gpu['hit_id'].shape[0]}", "pixels": int(gid.size),
            "id_mismatch": int((mism & ~ties).sum()), "id_ties": int(ties.sum()),
            "max_t_rel": float(rel.max()) if rel.size else 0.0,
            "rmse": float(np.sqrt(np.mean((a - b) ** 2))),
            "column0_nan_equal": bool(np.array_equal(np.isnan(gpu["rgba32f"][r][:, 0]),
                                                     np.isnan(ora["rgba32f"][r][:, 0]))),
            "bar": {"id_mismatch": 0, "max_t_rel": 1e-5, "rmse": 1e-3}}


def cpu_baseline_sample(wl, tri_bvh, seconds_target: float = 15.0):
    """Oracle (CPU port of the shader, same BVH) on a bounded row subset, all
    host threads.  Returns (Mrays/s, threads, description)."""
    import pyoracle
    pyoracle.build()
    threads = os.cpu_count() or 1
    step = 64
    rows = (0, wl.height, step)
    prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start, sky=wl.sky,
                          tie_mode=wl.tie_mode, trig_mode=0, threads=threads, rows=rows)
    t0 = time.perf_counter()
    out = pyoracle.render(wl.scene, wl.frame, prm, tri_bvh=tri_bvh)
    dt = time.perf_counter() - t0
    # grow the sample toward the target duration
    if dt < seconds_target / 4:
        step = max(1, int(step * dt / (seconds_target / 2)) or 1)
        prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                              sky=wl.sky, tie_mode=wl.tie_mode, trig_mode=0, threads=threads, rows=(0, wl.height, step))
        t0 = time.perf_counter()
        out = pyoracle.render(wl.scene, wl.frame, prm, tri_bvh=tri_bvh)
        dt = time.perf_counter() - t0
    st = out["stats"]
    rays = st["closest_rays"] + st["shadow_rays"]
    nrows = len(range(0, wl.height, step))
    return rays / dt / 1e6, threads, f"every {step}th scanline ({nrows} of {wl.height} rows, full width, " \
                                     f"{wl.spp} spp), {dt:.1f} s, {rays} rays", out, (0, wl.height, step)


def tail_summary(rounds, tail_paths: int) -> dict | None:
    """Where the profiled frame handed its last paths to the finishing
    kernel, and what the rounds before cost."""
    if rounds is None or len(rounds) == 0:
        return None
    fin = rounds["finish"] == 1
    out = {"tail_paths": "auto (twice the extend kernel's resident threads)" if tail_paths == 0 else tail_paths,
           "rounds": int((~fin).sum()), "first_round_paths": int(rounds["paths"][0])}
    if fin.any():
        out["handover_paths"] = int(rounds["paths"][-1])
        out["finish_ms"] = float(rounds["extend_ms"][-1])
    full = rounds["paths"][~fin] >= rounds["paths"][0] // 2
    out["ms_in_rounds_with_half_the_paths_or_more"] = float(
        (rounds["extend_ms"][~fin][full] + rounds["shade_ms"][~fin][full]).sum())
    return out


def batched_section(local: int, steps: int, warmup: int) -> dict:
    """c2: 64 scenes (triangles log-uniform in [1k, 200k], c1 geometry,
    resolutions from {128^2 .. 1024^2}, 4 spp, depth 6) traced (a) by the plain
    kernel launched once per scene and (b) as one wavefront over all scenes
    replayed as one CUDA graph, with the launch shape picked by the autotuner.
    Mrays/s from canonical ray counts; L2 flushed before every timed step."""
    import numpy as np
    import torch
    from vktrace import abi, configs, tune
    wls = configs.c2()
    tr = abi.Tracer(local)
    tr.upload_scenes([w.scene for w in wls])
    frames = [w.frame for w in wls]

    def prm(kernel, stats=False, aovs=(abi.AOV_RGBA8,)):
        return [abi.Tracer.params(w.width, w.height, spp=w.spp, max_depth=w.max_depth, rr_start=w.rr_start,
                                  sky=w.sky, kernel=kernel, aovs=aovs, stats=stats) for w in wls]

    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    tr.trace_batched(frames, prm(abi.KERNEL_PLAIN, stats=True), use_graph=False, stream=sptr)
    st = {k: int(v) for k, v in zip(abi.STATS_FIELDS, tr.readback_scene(0, abi.AOV_STATS))}
    rays = st["closest_rays"] + st["shadow_rays"]

    def timed(params, use_graph):
        for _ in range(warmup):
            flush.zero_()
            tr.trace_batched(frames, params, use_graph=use_graph, stream=sptr)
        tr.synchronize()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            evs[k][0].record(stream)
            tr.trace_batched(frames, params, use_graph=use_graph, stream=sptr)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        tr.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / steps

    p_plain = prm(abi.KERNEL_PLAIN, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F))
    ms_plain = timed(p_plain, False)
    plain_imgs = [tr.readback_scene(k, abi.AOV_RGBA32F) for k in range(len(wls))]
    p_wf = prm(abi.KERNEL_WAVEFRONT, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F))
    # the compressed 8-wide and the binary traversal (the uncompressed 4-wide
    # measured slower on these soups), the stack the BVHs need, the
    # finishing kernel's threshold: the library's choice or 1M live paths
    best, table = tune.autotune_batched(tr, frames, p_wf, widths=(8, 2), blocks=(128, 256), stacks=(0,),
                                        wavefronts=(0, 6), tails=(0, 1_000_000), budget_s=40.0)
    for p in p_wf:
        p.block, p.stack_depth, p.wavefront = best["block"], best["stack_depth"], best["wavefront"]
        p.bvh_width, p.tail_paths = best["bvh_width"], best["tail_paths"]
    ms_wf = timed(p_wf, True)
    rmse = 0.0
    for k in range(len(wls)):
        a = tr.readback_scene(k, abi.AOV_RGBA32F)[:, 1:, :3].astype(np.float64)
        b = plain_imgs[k][:, 1:, :3].astype(np.float64)
        rmse = max(rmse, float(np.sqrt(np.mean((a - b) ** 2))))
    tr.close()
    decomp = batch_decomposition(local, wls, p_plain)
    pixels = sum(w.pixels for w in wls)
    hbm, hbm_src = peaks()
    k_bytes = algorithmic_bytes(st, pixels, 4)
    return {"metric": "batched Mrays/s (64 scenes, one CUDA-graph wavefront)", "value": rays / (ms_wf / 1e3) / 1e6,
            "unit": UNIT, "ms_per_step": ms_wf,
            "plain_per_scene": {"value": rays / (ms_plain / 1e3) / 1e6, "ms_per_step": ms_plain,
                                "kernel": "k_plain, one launch per scene"},
            "speedup_vs_plain_per_scene": ms_plain / ms_wf,
            "max_image_rmse_vs_plain": rmse, "rays_per_step": rays, "scenes": len(wls), "pixels": pixels,
            "triangles": int(sum(len(w.scene.triangles) for w in wls)),
            "autotuned": best, "autotune_candidates": len(table),
            "decomposition": decomp,
            # canonical algorithmic bytes (the plain kernel's counts) over the
            # whole replay, against measured HBM; DRAM traffic from ncu
            "roofline": {"bound": "issue / L2 latency (extend kernel, 88.6 % of a replay); the scenes exceed L2",
                         "achieved": k_bytes / (ms_wf / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": k_bytes / (ms_wf / 1e3) / 1e9 / hbm, "peak_source": hbm_src,
                         "algorithmic_bytes_per_step": k_bytes, "traffic": NCU_BATCH_EXTEND_DRAM_BYTES,
                         "kernel": "wf_extend_cw8 (MULTI)", "traffic_all_kernels": NCU_BATCH_ALL_DRAM_BYTES,
                         "dram_gbs_all_kernels": NCU_BATCH_ALL_DRAM_BYTES / (ms_wf / 1e3) / 1e9},
            "config": {"workload": "c2-64scenes-tris-loguniform-1k-200k-res128-1024-4spp-d6-rr3-sah16",
                       "l2": "flushed before each timed step (256 MiB write)"}}


def batch_decomposition(local: int, wls, p_plain) -> dict:
    """Where the batch's speed-up over one plain launch per scene comes from:
    every scene traced on its own (its own upload, one tracer_trace) with the
    plain kernel and with the wavefront (the library's defaults: automatic
    width and hand-over), device-timed (median of 3, L2 flushed), against
    the batch.  plain -> wavefront per scene is the kernels' gain; the rest is
    the batch's (one queue filling the GPU across scenes, one tail, no
    per-scene launches).  Also split by image size."""
    import torch
    from vktrace import abi
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    tr = abi.Tracer(local)
    rows = []
    for k, w in enumerate(wls):
        tr.upload_scene(w.scene)
        pw = abi.Tracer.params(w.width, w.height, spp=w.spp, max_depth=w.max_depth, rr_start=w.rr_start, sky=w.sky,
                               kernel=abi.KERNEL_WAVEFRONT, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F))
        ms = {}
        for name, p in (("plain", p_plain[k]), ("wavefront", pw)):
            tr.trace(w.frame, p, sptr)
            times = []
            for _ in range(3):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                tr.trace(w.frame, p, sptr)
                b.record(stream)
                torch.cuda.synchronize()
                tr.synchronize()
                times.append(a.elapsed_time(b))
            ms[name] = sorted(times)[1]
        rows.append((w.width, len(w.scene.triangles), ms["plain"], ms["wavefront"]))
    tr.close()
    out = {"plain_single_ms": sum(r[2] for r in rows), "wavefront_single_ms": sum(r[3] for r in rows),
           "by_resolution": {}}
    for res in sorted({r[0] for r in rows}):
        sel = [r for r in rows if r[0] == res]
        out["by_resolution"][f"{res}^2"] = {"scenes": len(sel), "plain_ms": sum(r[2] for r in sel),
                                            "wavefront_ms": sum(r[3] for r in sel)}
    return out


def _perturbed_albedo(mats, seed, sigma=0.1):
    from vktrace import scene as S
    import numpy as np
    g = S.SplitMix64(seed)
    out = mats.copy()
    out["albedo"] = np.clip(mats["albedo"] + sigma * g.normal(3 * len(mats)).reshape(-1, 3), 0.0, 1.0)
    return out


def adjoint_section(local: int, steps: int) -> dict:
    """c3: 256^2, 4 spp, depth 4, 10k triangles in [-10,10]^3, 64 materials.
    Target rendered with albedos perturbed by N(0, 0.1^2) (clamped); L2 image
    loss.  Forward (wavefront) and adjoint (path replay) Mrays/s, device-timed
    with every buffer resident; gradient spot check against central
    differences of the forward (step 1e-3) on the largest albedo components."""
    import numpy as np
    import torch
    from vktrace import abi, configs
    wl = configs.c3()
    tr = abi.Tracer(local)
    tr.upload_scene(wl.scene)
    base = wl.scene.materials.copy()
    nm = len(base)
    p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                          sky=wl.sky, aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR), stats=True)
    tr.set_materials(_perturbed_albedo(base, 3))
    tr.trace(wl.frame, p)
    target = tr.readback(abi.AOV_RGBA32F)
    tr.set_materials(base)

    def loss_dl(img):
        d = img[:, 1:, :3].astype(np.float64) - target[:, 1:, :3]
        dl = np.zeros(img.shape, np.float32)
        dl[:, 1:, :3] = 2 * d
        return float((d * d).sum()), dl

    tr.trace(wl.frame, p)
    fwd_rays = sum(tr.stats()[k] for k in ("closest_rays", "shadow_rays"))
    img = tr.readback(abi.AOV_RGBA32F)
    lin = tr.readback(abi.AOV_LINEAR)
    L0, dl = loss_dl(img)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    dl_d = torch.from_numpy(dl).cuda()
    lin_d = torch.from_numpy(lin).cuda()
    ga = torch.zeros((nm, 3), device="cuda")
    ge = torch.zeros((nm, 3), device="cuda")
    gc = torch.zeros(3, device="cuda")
    p_run = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                              sky=wl.sky, aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR))

    def timed(fn):
        for _ in range(2):
            fn()
        tr.synchronize()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        tr.synchronize()
        return a.elapsed_time(b) / steps

    ms_fwd = timed(lambda: tr.trace(wl.frame, p_run, sptr))
    adj = lambda: tr.trace_adjoint(wl.frame, p_run, dl_d.data_ptr(), lin_d.data_ptr(),
                                   outputs=(ga.data_ptr(), ge.data_ptr(), gc.data_ptr()), stream=sptr)
    ms_adj = timed(adj)  # AUTO: the wavefront (c3 has no emissive spheres); pure path replay
    adj_rays = sum(tr.stats()[k] for k in ("closest_rays", "shadow_rays"))
    # the opt-in hit log: pass 1's hits of the current sample kept (16 B x
    # depth per pixel) so that pass 2 traces nothing; the same gradients
    tr.set_adjoint_hit_log(4 << 30)
    ms_log = timed(adj)
    log_rays = sum(tr.stats()[k] for k in ("closest_rays", "shadow_rays"))
    tr.set_adjoint_hit_log(0)
    # both adjoint forms on the same inputs, for comparison: forward rays per
    # second of each, and the rays each traced
    per_kernel = {}
    for name, k in (("per_pixel", abi.KERNEL_PLAIN), ("wavefront", abi.KERNEL_WAVEFRONT)):
        p_run.kernel = k
        ms_k = timed(adj)
        k_rays = sum(tr.stats()[q] for q in ("closest_rays", "shadow_rays"))
        per_kernel[name] = {"value": fwd_rays / (ms_k / 1e3) / 1e6, "ms_per_step": ms_k, "traced_rays": k_rays}
    p_run.kernel = abi.KERNEL_AUTO
    g_alb = ga.cpu().numpy().astype(np.float64)
    # spot check: central differences, step 1e-3, on the 6 largest components.
    # A 1e-3 step is up to 10 % of a small albedo, where the loss's curvature
    # makes that difference itself off by ~1e-3 relative; the Richardson
    # combination of steps 1e-3 and 5e-4, (4 fd(h/2) - fd(h)) / 3, cancels
    # that h^2 term.
    idx = np.argsort(-np.abs(g_alb).ravel())[:6]

    def central(m, c, h):
        mp, mm = base.copy(), base.copy()
        mp["albedo"][m, c] += h
        mm["albedo"][m, c] -= h
        tr.set_materials(mp)
        tr.trace(wl.frame, p_run)
        Lp, _ = loss_dl(tr.readback(abi.AOV_RGBA32F))
        tr.set_materials(mm)
        tr.trace(wl.frame, p_run)
        Lm, _ = loss_dl(tr.readback(abi.AOV_RGBA32F))
        return (Lp - Lm) / float(np.float32(mp["albedo"][m, c]) - np.float32(mm["albedo"][m, c]))

    rel, rel_r = [], []
    for flat in idx:
        m, c = divmod(int(flat), 3)
        f1 = central(m, c, 1e-3)
        f2 = central(m, c, 5e-4)
        fr = (4.0 * f2 - f1) / 3.0
        rel.append(abs(g_alb[m, c] - f1) / abs(f1))
        rel_r.append(abs(g_alb[m, c] - fr) / abs(fr))
    tr.set_materials(base)
    fp64 = fp64_host_check(wl, target, g_alb, idx)
    campos = campos_check(tr, wl, p_run)
    campos1 = campos_check(tr, wl, p_run, depth=1)
    tr.close()
    fwd = fwd_rays / (ms_fwd / 1e3) / 1e6
    # headline: the forward frame's rays per second of adjoint time, i.e.
    # adjoint speed against forward speed on the same frame, by pure path
    # replay (the default); beside it the rays the adjoint traced (both
    # passes) and the opt-in hit log's figures
    adjv = fwd_rays / (ms_adj / 1e3) / 1e6
    replay = adj_rays / (ms_adj / 1e3) / 1e6
    return {"metric": "adjoint Mrays/s (c3, path replay; forward rays per adjoint second)", "value": adjv,
            "unit": UNIT, "ms_per_step": ms_adj,
            "forward": {"value": fwd, "ms_per_step": ms_fwd, "rays_per_step": fwd_rays},
            "ratio_adjoint_to_forward": ms_fwd / ms_adj,
            "traced_rays": {"rays_per_step": adj_rays, "mrays_per_s": replay,
                            "ratio_to_forward_mrays_per_s": replay / fwd},
            "with_hit_log": {"value": fwd_rays / (ms_log / 1e3) / 1e6, "ms_per_step": ms_log,
                             "ratio_adjoint_to_forward": ms_fwd / ms_log, "traced_rays": log_rays,
                             "note": "opt-in (tracer_set_adjoint_hit_log): pass 1's hits of the current sample "
                                     "kept, 16 B x max_depth per pixel, so pass 2 traces nothing; off by default "
                                     "(pure path replay, no stored path vertices)"},
            "kernel": "auto (wavefront: no emissive spheres)",
            "kernels": per_kernel,
            "grad_check": {"max_rel_err_vs_central_fd": max(rel), "step": 1e-3,
                           "max_rel_err_vs_richardson_fd": max(rel_r), "steps": [1e-3, 5e-4],
                           "components": len(rel), "fp64_host": fp64, "camera_position": campos,
                           "camera_position_depth1": campos1},
            "loss": L0,
            "config": {"workload": wl.name, "triangles": len(wl.scene.triangles), "materials": nm}}


def campos_check(tr, wl, p, depth=None) -> dict:
    """The camera-position gradient at c3 (its boundary part: triangle
    outlines moving across the point-sampled pixels) against central
    differences of the GPU forward with common random numbers, for two linear
    losses (fixed weights per pixel and channel, so dL/dI is exact at every
    camera position): N(0, 1) weights, and smooth positive ones (1 + sin +
    cos over the image: outline motions add up instead of cancelling).  The
    differences are averaged over 24 x 24 sub-pixel offsets of every sample
    point (the camera's dir moved along right and up by a fraction of a
    pixel: the one-pixel box the boundary term differentiates), at steps
    h = 0.005 and 0.01 (on c3's ~2-pixel triangles a larger step lets a
    sample point cross two outlines of one triangle and biases the quotient
    towards zero); their standard error comes from 16 random groups of the
    offsets, and err_in_se is the gradient's distance from them in units of
    it.  Also the adjoint's time with the boundary part on.  depth: the path
    depth to check at (None: the workload's); at depth 1 every outline that
    moves the image is a primary one, the part the boundary term models."""
    saved_depth = p.max_depth
    if depth is not None:
        p.max_depth = depth
    try:
        return _campos_check(tr, wl, p)
    finally:
        p.max_depth = saved_depth


def _campos_check(tr, wl, p) -> dict:
    import numpy as np
    from vktrace import abi
    from vktrace import scene as S
    W, H = wl.width, wl.height
    g = np.random.default_rng(5)
    weights = {"normal": np.zeros((H, W, 4), np.float32), "smooth": np.zeros((H, W, 4), np.float32)}
    weights["normal"][:, 1:, :3] = g.normal(size=(H, W - 1, 3)).astype(np.float32)
    yy, xx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    for c in range(3):
        weights["smooth"][:, :, c] = 1.0 + 0.5 * np.sin(2 * np.pi * (xx / W + c / 3.0)) + 0.5 * np.cos(2 * np.pi * yy / H)
    weights["smooth"][:, 0] = 0.0  # column 0 is NaN by construction
    p.aov_mask = (1 << abi.AOV_RGBA32F) | (1 << abi.AOV_LINEAR)
    tr.trace(wl.frame, p)
    lin = tr.readback(abi.AOV_LINEAR)
    # the adjoint with the boundary part on (4 pieces per edge), device-timed
    # with every input resident
    import torch
    nm = len(wl.scene.materials)
    dl_d, lin_d = torch.from_numpy(weights["normal"]).cuda(), torch.from_numpy(lin).cuda()
    outs = [torch.zeros((nm, 3), device="cuda"), torch.zeros((nm, 3), device="cuda"), torch.zeros(3, device="cuda")]
    stream = torch.cuda.current_stream()
    grads = {}
    tr.set_edge_sampling(4)
    try:
        call = lambda: tr.trace_adjoint(wl.frame, p, dl_d.data_ptr(), lin_d.data_ptr(),
                                        outputs=tuple(o.data_ptr() for o in outs), stream=stream.cuda_stream)
        for _ in range(2):
            call()
        tr.synchronize()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(5):
            call()
        b.record(stream)
        torch.cuda.synchronize()
        tr.synchronize()
        ms_edges = a.elapsed_time(b) / 5
        for name, dl in weights.items():
            _, _, gc = tr.trace_adjoint(wl.frame, p, dl, lin, num_materials=nm)
            grads[name] = [float(v) for v in gc]
    finally:
        tr.set_edge_sampling(0)
    steps, ks = (0.005, 0.01), 24
    out = {"losses": {"normal": "N(0,1) weights per pixel and channel",
                      "smooth": "1 + 0.5 sin(2 pi (x/W + c/3)) + 0.5 cos(2 pi y/H) per pixel and channel"},
           "max_depth": int(p.max_depth), "steps": list(steps), "subpixel_offsets": ks * ks,
           "gradient": grads, "fd": {}, "adjoint_ms_with_boundary_part": ms_edges,
           "note": "boundary part on (tracer_set_edge_sampling 4; off by default): primary-visibility edge "
                   "sampling; outlines seen only by bounce rays are not modelled"}
    base = np.array(wl.frame, S.FRAME).reshape(())
    pos0 = np.array(base["camera"]["pos"], np.float64)
    groups = np.random.default_rng(1).permutation(ks * ks).reshape(16, -1)
    for h in steps:
        rows = {name: {"fd": [], "standard_error": [], "err_in_se": []} for name in weights}
        for axis in range(3):
            step = float(np.float32(pos0[axis] + h) - np.float32(pos0[axis] - h))
            per = {name: np.zeros(ks * ks) for name in weights}
            for i in range(ks):
                for j in range(ks):
                    ox, oy = (i + 0.5) / ks - 0.5, (j + 0.5) / ks - 0.5
                    imgs = []
                    for sgn in (1.0, -1.0):
                        f = base.copy()
                        pos = pos0.copy()
                        pos[axis] += sgn * h
                        f["camera"]["pos"] = pos.astype(np.float32)
                        cam = f["camera"]
                        cam["dir"] = (cam["dir"].astype(np.float64) + cam["right"] * (2.0 * ox / W)
                                      + cam["up"] * (2.0 * oy / H)).astype(np.float32)
                        tr.trace(f, p)
                        imgs.append(tr.readback(abi.AOV_RGBA32F)[:, 1:, :3].astype(np.float64))
                    d = (imgs[0] - imgs[1]) / step
                    for name, dl in weights.items():
                        per[name][i * ks + j] = (d * dl[:, 1:, :3]).sum()
            for name in weights:
                fd = float(per[name].mean())
                se = float(np.std([per[name][q].mean() for q in groups], ddof=1) / 4.0)
                rows[name]["fd"].append(fd)
                rows[name]["standard_error"].append(se)
                rows[name]["err_in_se"].append(abs(grads[name][axis] - fd) / se if se > 0 else None)
        out["fd"][str(h)] = rows
    return out


def fp64_host_check(wl, target, g_alb, idx) -> dict:
    """Checker: the adjoint's largest albedo components against central
    differences of the FP64 host evaluation of the same frame (the oracle in
    double precision, step 2^-12, the step measured in float), with the
    GPU's target image."""
    import numpy as np
    import pyoracle
    from vktrace import scene as S
    pyoracle.build()
    tb = pyoracle.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)[:2]
    prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                          sky=wl.sky, threads=os.cpu_count() or 1)
    tgt = target[:, 1:, :3].astype(np.float64)
    base = wl.scene.materials

    def L64(mats):
        out = pyoracle.render_f64(S.Scene(triangles=wl.scene.triangles, materials=mats, bvh=wl.scene.bvh), wl.frame,
                                  prm, tri_bvh=tb)
        d = out["image"][:, 1:, :3] - tgt
        return float(np.sum(d * d))

    h = 2.0 ** -12
    rel = []
    t0 = time.perf_counter()
    for flat in idx:
        m, c = divmod(int(flat), 3)
        mp, mm = base.copy(), base.copy()
        mp["albedo"][m, c] += h
        mm["albedo"][m, c] -= h
        fd = (L64(mp) - L64(mm)) / float(np.float32(mp["albedo"][m, c]) - np.float32(mm["albedo"][m, c]))
        rel.append(abs(g_alb[m, c] - fd) / abs(fd))
    return {"max_rel_err": max(rel), "step": h, "components": len(rel),
            "host_seconds": time.perf_counter() - t0}


def small_configs_section(local: int, steps: int, cpu: bool) -> dict:
    """The reference's own frame (Ref: constant scene, linear scan, reference
    ties, 1024^2, 4 spp, depth 4) and c0 (64 spheres, median BVH, 512^2,
    1 spp, depth 2): device-timed Mrays/s of the wavefront and plain kernels,
    and, with cpu, the oracle's on all host cores (the whole frame)."""
    import torch
    from vktrace import abi, configs
    from vktrace import scene as S
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    out = {}
    for wl in (configs.ref(), configs.c0()):
        tr = abi.Tracer(local)
        tr.upload_scene(wl.scene)
        res = {}
        rays = None
        for name, kern in (("plain", abi.KERNEL_PLAIN), ("wavefront", abi.KERNEL_WAVEFRONT)):
            p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                                  sky=wl.sky, tie_mode=wl.tie_mode, kernel=kern, stats=rays is None)
            if rays is None:  # canonical counts from the plain kernel
                tr.trace(wl.frame, p, sptr)
                st = tr.stats()
                rays = st["closest_rays"] + st["shadow_rays"]
                p.stats = 0
            for _ in range(3):
                tr.trace(wl.frame, p, sptr)
            tr.synchronize()
            torch.cuda.synchronize()
            tot = 0.0
            for _ in range(steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                tr.trace(wl.frame, p, sptr)
                e1.record(stream)
                torch.cuda.synchronize()
                tot += e0.elapsed_time(e1)
            ms = tot / steps
            res[name] = {"value": rays / (ms / 1e3) / 1e6, "ms_per_frame": ms}
        tr.close()
        res["rays_per_frame"] = rays
        if cpu:
            import pyoracle
            pyoracle.build()
            prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                                  sky=wl.sky, tie_mode=wl.tie_mode, trig_mode=0, threads=os.cpu_count() or 1)
            tb, sb = None, None
            if wl.scene.bvh != 0:
                sb = abi.build_bvh(wl.scene.bvh, wl.scene.spheres, wl.scene.leaf_size, wl.scene.sah_bins)[:2]
            t0 = time.perf_counter()
            o = pyoracle.render(wl.scene, wl.frame, prm, tri_bvh=tb, sphere_bvh=sb)
            dt = time.perf_counter() - t0
            r = o["stats"]["closest_rays"] + o["stats"]["shadow_rays"]
            res["cpu_oracle"] = {"value": r / dt / 1e6, "cores": os.cpu_count() or 1, "sample": "whole frame",
                                 "kind": "port"}
        out[wl.name] = res
    # the legacy Whitted shader (Raytracer.comp) on its own scene, the
    # start-up frame at the reference's 1024^2
    tr = abi.Tracer(local)
    fr = S.reference_frame(0.5)
    p = abi.Tracer.params(1024, 1024, stats=True)
    tr.trace_whitted(fr, p, sptr)
    st = tr.stats()
    rays = st["closest_rays"] + st["shadow_rays"]
    p.stats = 0
    for _ in range(3):
        tr.trace_whitted(fr, p, sptr)
    tr.synchronize()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tr.trace_whitted(fr, p, sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    tr.close()
    ms = tot / steps
    res = {"gpu": {"value": rays / (ms / 1e3) / 1e6, "ms_per_frame": ms}, "rays_per_frame": rays}
    if cpu:
        import pyoracle
        t0 = time.perf_counter()
        o = pyoracle.whitted(fr, 1024, 1024)
        dt = time.perf_counter() - t0
        r = o["stats"]["closest_rays"] + o["stats"]["shadow_rays"]
        res["cpu_oracle"] = {"value": r / dt / 1e6, "cores": os.cpu_count() or 1, "sample": "whole frame",
                             "kind": "port"}
    out["whitted-raytracer.comp-1024x1024"] = res
    return out


def present_section(local: int, steps: int) -> dict:
    """The present pass (Fullscreen.frag) on device images: the reference's
    sizes (1024^2 RGBA8 images -> 1024x768 framebuffer) and c1's (1920x1080
    -> 1920x1080).  Per launch: CUDA events around one launch with L2 flushed
    before it; algorithmic bytes = both source images + the framebuffer."""
    import numpy as np
    import torch
    from vktrace import abi
    hbm, src = peaks()
    tr = abi.Tracer(local)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    out = {}
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    for name, (sw, sh, w, h) in (("ref_1024_to_1024x768", (1024, 1024, 1024, 768)),
                                 ("c1_1920x1080", (1920, 1080, 1920, 1080))):
        a = torch.randint(0, 256, (sh, sw, 4), dtype=torch.uint8, device="cuda", generator=g)
        b = torch.randint(0, 256, (sh, sw, 4), dtype=torch.uint8, device="cuda", generator=g)
        fb = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
        call = lambda: tr.present((a.data_ptr(), sw, sh, abi.AOV_RGBA8), (b.data_ptr(),), w, h, abi.AOV_RGBA8,
                                  out=fb.data_ptr(), stream=sptr)
        for _ in range(3):
            call()
        torch.cuda.synchronize()
        # the library's CUDA events bracket the kernel alone (the call's host
        # work -- argument checks, pointer queries -- stays outside)
        tr.set_profiling(True)
        times = []
        for _ in range(steps):
            flush.zero_()
            call()
            times.append(tr.timings()["total_ms"])
        tr.set_profiling(False)
        ms = float(np.median(times))
        nbytes = 2 * sw * sh * 4 + w * h * 4
        gbs = nbytes / (ms / 1e3) / 1e9
        out[name] = {"us_per_launch": ms * 1e3, "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
                     "frac_of_hbm": gbs / hbm, "peak_source": src}
    tr.close()
    return {"kernel": "k_present<uchar4>", "l2": "flushed before each launch", **out}


def gd_section(local: int, gd_steps: int, width: int, spp: int, n_tris: int, checkpoint: str | None = None,
               every: int = 10, resume: bool = False, hit_log: bool = False) -> dict:
    """c4: recover perturbed albedos by gradient descent on an L2 image loss
    (1024^2, 64 spp, depth 12, 1M triangles, 1024 materials by default).
    Each step: forward (wavefront, RGBA32F + LINEAR) and adjoint, device-timed;
    Adam on the albedo table, clamped to [1e-3, 1] (vktrace.descent).  With a
    checkpoint path the optimiser state is saved every `every` steps and at
    the end; resume continues from that file.  hit_log: the adjoint keeps
    pass 1's hits of the current sample (tracer_set_adjoint_hit_log) instead
    of pure path replay."""
    import numpy as np
    import torch
    from vktrace import abi, configs
    from vktrace.descent import AlbedoDescent
    wl = configs.c4(width=width, spp=spp, n_tris=n_tris)
    tr = abi.Tracer(local)
    tr.upload_scene(wl.scene)
    if hit_log:
        tr.set_adjoint_hit_log(4 << 30)
    truth = wl.scene.materials.copy()
    nm = len(truth)
    p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                          sky=wl.sky, aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR), stats=True)
    tr.trace(wl.frame, p)
    target = torch.from_numpy(tr.readback(abi.AOV_RGBA32F)).cuda()
    start = _perturbed_albedo(truth, 4)
    if resume and checkpoint and os.path.exists(checkpoint):
        opt = AlbedoDescent.load(checkpoint)
    else:
        opt = AlbedoDescent(start["albedo"], lr=0.01, lo=1e-3, hi=1.0)
    first = opt.t
    ga = torch.zeros((nm, 3), device="cuda")
    ge = torch.zeros((nm, 3), device="cuda")
    gc = torch.zeros(3, device="cuda")
    free0, _ = torch.cuda.mem_get_info()
    # a dedicated stream: the events must be recorded on the stream the tracer
    # launches on (handle 0 would select the tracer's own stream instead)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    mats = truth.copy()
    npx = wl.width * wl.height
    peak_extra = 0
    for step in range(first, gd_steps):
        mats["albedo"] = opt.albedo
        tr.set_materials(mats)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        tr.trace(wl.frame, p, sptr)
        e1.record(stream)
        tr.synchronize()
        f_rays = sum(tr.stats()[k] for k in ("closest_rays", "shadow_rays"))
        ptr, _ = tr.device_image(abi.AOV_RGBA32F)
        img = torch.empty((wl.height, wl.width, 4), device="cuda")
        lin = torch.empty((wl.height, wl.width, 4), device="cuda")
        torch.cuda.synchronize()
        from vktrace.autograd import _DeviceView
        img.copy_(torch.as_tensor(_DeviceView(ptr, img.shape, "<f4"), device="cuda"))
        lptr, _ = tr.device_image(abi.AOV_LINEAR)
        lin.copy_(torch.as_tensor(_DeviceView(lptr, lin.shape, "<f4"), device="cuda"))
        dl = torch.zeros_like(img)
        dl[:, 1:, :3] = 2.0 * (img[:, 1:, :3] - target[:, 1:, :3]) / npx
        torch.cuda.synchronize()
        e1b = torch.cuda.Event(enable_timing=True)
        e1b.record(stream)
        tr.trace_adjoint(wl.frame, p, dl.data_ptr(), lin.data_ptr(),
                         outputs=(ga.data_ptr(), ge.data_ptr(), gc.data_ptr()), stream=sptr)
        e2.record(stream)
        tr.synchronize()
        torch.cuda.synchronize()
        peak_extra = max(peak_extra, free0 - torch.cuda.mem_get_info()[0])
        a_rays = sum(tr.stats()[k] for k in ("closest_rays", "shadow_rays"))
        opt.record(fwd=f_rays / (e0.elapsed_time(e1) / 1e3) / 1e6,
                   adj=f_rays / (e1b.elapsed_time(e2) / 1e3) / 1e6,
                   replay=a_rays / (e1b.elapsed_time(e2) / 1e3) / 1e6)
        opt.step(ga.cpu().numpy())
        if checkpoint and (opt.t % every == 0 or opt.t == gd_steps):
            opt.save(checkpoint)
    tr.close()
    seen = opt.seen
    fwd_rates, adj_rates = opt.log.get("fwd", [0.0]), opt.log.get("adj", [0.0])
    err0 = np.abs(start["albedo"] - truth["albedo"])[seen]
    err1 = np.abs(opt.albedo - truth["albedo"])[seen]
    return {"metric": "gradient descent on albedos (c4 shape)", "steps": gd_steps, "resumed_at_step": first,
            "forward_mrays_s": {"median": float(np.median(fwd_rates)), "min": float(np.min(fwd_rates))},
            # forward rays per adjoint second
            "adjoint_mrays_s": {"median": float(np.median(adj_rates)), "min": float(np.min(adj_rates))},
            "adjoint_to_forward": float(np.median(adj_rates) / np.median(fwd_rates)),
            "albedo_mae": {"initial": float(err0.mean()), "final": float(err1.mean()),
                           "materials_with_gradient": int(seen.sum()), "materials": nm},
            "checkpoint": checkpoint,
            "peak_extra_device_memory_bytes": int(peak_extra),
            "config": {"workload": wl.name, "optimizer": "Adam lr 0.01, albedo clamped to [1e-3, 1]",
                       "adjoint": "hit log (pass 1's hits of the current sample kept)" if hit_log
                       else "pure path replay (no stored path vertices)"}}


def run_reference(args):
    """CPU restatement of the reference shader (oracle port, same BVH), timed
    on the host cores.  Rank 0 alone works under torchrun."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    from vktrace import configs
    import pyoracle
    pyoracle.build()
    wl = configs.c1(width=args.width, height=args.height, spp=args.spp)
    # the oracle's own builder (node for node the product's; no product code here)
    nodes, idx, _ = pyoracle.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)
    threads = os.cpu_count() or 1
    step = 128
    times, rays_tot = [], 0
    for k in range(args.warmup + args.steps):
        prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                              sky=wl.sky, tie_mode=1, trig_mode=0, threads=threads,
                              rows=((k * 7) % step, wl.height, step))
        t0 = time.perf_counter()
        out = pyoracle.render(wl.scene, wl.frame, prm, tri_bvh=(nodes, idx))
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            rays_tot += out["stats"]["closest_rays"] + out["stats"]["shadow_rays"]
    total = sum(times)
    value = rays_tot / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(wl, args.gpus),
        "impl_config": {"kind": "CPU restatement of Tracer.comp (oracle), OpenMP over scanlines",
                        "bvh": "built by the oracle's own builder", "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: every {step}th scanline of the frame (offset varies), full width, "
                                   f"{wl.spp} spp; CPU restatement of Tracer.comp with the same BVH"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    from vktrace import abi, configs
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    wl = configs.c1(width=args.width, height=args.height, spp=args.spp)
    # weak scaling: each rank its own frame (different seed)
    wl.frame["seed"] = np.float32(rank_seed(wl.frame["seed"], rank))
    nodes, idx, bvh_depth = abi.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)
    tr = abi.Tracer(local)
    tr.upload_scene(wl.scene, tri_bvh=(nodes, idx))
    # A dedicated stream: the kernel, the L2 flush and the timing events all
    # run on it (a legacy-default-stream handle of 0 would mean "the context's
    # own stream" to the C ABI).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    kern = abi.KERNEL_WAVEFRONT if args.kernel == "wavefront" else abi.KERNEL_PLAIN
    common = dict(spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start, sky=wl.sky, kernel=kern,
                  block=args.block, wavefront=args.wavefront, bvh_width=args.bvh_width, tail_paths=args.tail_paths)
    p_run = abi.Tracer.params(wl.width, wl.height, aovs=(abi.AOV_RGBA8,), stats=False, **common)
    # counting pass (untimed) with the plain kernel, whose node-visiting order
    # is the oracle's: the canonical ray / node / primitive counts of the frame.
    # Every kernel traces exactly these rays (the wavefront's speculative
    # traversal fetches ~1.5 % more nodes than this canonical count).
    p_count = abi.Tracer.params(wl.width, wl.height, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F), stats=True,
                                **dict(common, kernel=abi.KERNEL_PLAIN, block=0))
    tr.trace(wl.frame, p_count, sptr)
    st = tr.stats()
    rays = st["closest_rays"] + st["shadow_rays"]
    plain_img = tr.readback(abi.AOV_RGBA32F)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        flush.zero_()
        tr.trace(wl.frame, p_run, sptr)
    tr.synchronize()
    torch.cuda.synchronize()

    clk = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(stream)
        tr.trace(wl.frame, p_run, sptr)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    tr.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = sum(step_ms) / args.steps
    value, max_s, _ = aggregate(world, rays, ms / 1e3)
    ms = max_s * 1e3

    # per-kernel breakdown of one frame (untimed run with CUDA events around
    # every extend and shade launch)
    tr.set_profiling(True)
    flush.zero_()
    tr.trace(wl.frame, p_run, sptr)
    breakdown = tr.timings()
    rounds = tr.rounds() if kern == abi.KERNEL_WAVEFRONT else None
    tr.set_profiling(False)

    # end to end through the C ABI with host buffers
    pinned = torch.empty((wl.height, wl.width, 4), dtype=torch.uint8, pin_memory=True)
    img = pinned.numpy()
    for _ in range(2):
        tr.trace(wl.frame, p_run)
        tr.readback(abi.AOV_RGBA8, img)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        tr.trace(wl.frame, p_run)
        tr.readback(abi.AOV_RGBA8, img)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e, e2e_s, _ = aggregate(world, rays, e2e_s)

    # the benchmarked frame itself (same kernel and launch shape), untimed,
    # with the float image and primary hits for the parity checks: against
    # the plain kernel's image (the metric is quoted at <= 1e-3 RMSE vs the
    # plain trace) and, below, against the oracle's frame
    p_chk = abi.Tracer.params(wl.width, wl.height, aovs=(abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT), stats=False,
                              **common)
    tr.trace(wl.frame, p_chk, sptr)
    hit = tr.readback(abi.AOV_PRIMARY_HIT)
    frame_out = {"rgba32f": tr.readback(abi.AOV_RGBA32F), "hit_id": hit[..., 0].copy(),
                 "hit_t": hit[..., 1].copy().view(np.float32)}
    d = frame_out["rgba32f"][:, 1:, :3].astype(np.float64) - plain_img[:, 1:, :3].astype(np.float64)
    rmse_vs_plain = float(np.sqrt(np.mean(d * d)))

    if rank == 0:
        peak, peak_kind = peaks()
        l2_gbs = tr.measure_l2_read(32 << 20, 64)
        ab = algorithmic_bytes(st, wl.pixels, 4)
        # dominant kernel: the traversal (extend) kernel of the wavefront, one
        # launch per round; its algorithmic bytes are the traversal bytes of
        # the frame, its time the sum of its launches (CUDA events)
        # (the finishing kernel traces the last ~1 % of the rays: its time
        # is counted with the extend launches')
        if kern == abi.KERNEL_WAVEFRONT and breakdown["extend_ms"] > 0:
            k_ms = breakdown["extend_ms"] + breakdown["finish_ms"]
            k_bytes = ab - 4 * wl.pixels
        else:
            k_ms, k_bytes = ms, ab
        achieved = k_bytes / (k_ms / 1e3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(wl, world),
            "impl_config": {"kernel": args.kernel, "block": args.block, "bvh_depth": bvh_depth,
                            "traversal": TRAVERSAL_LABEL[args.bvh_width], "tail_paths": args.tail_paths},
            "rays_per_step": rays,
            "max_image_rmse_vs_plain": rmse_vs_plain,
            "stats": st,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 96,
                    "d2h_bytes_per_step": wl.pixels * 4},
            # the traversal's working set (4.8 MB of triangles, 2.1 MB of nodes)
            # stays in L2: what bounds it is instruction issue (the integer
            # pipe of the slab tests), the warps' SIMD efficiency and the
            # latency of dependent L1/L2 node fetches, not HBM bandwidth.
            # peak/frac: against the measured HBM copy bandwidth (the common
            # denominator); l2.frac: against L2 read bandwidth
            "roofline": {"bound": "instruction issue (integer ALU, 68 % issue active in ncu) with L1/L2 latency "
                                  "behind it; scene L2-resident", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": (NCU_EXTEND_DRAM_BYTES_PER_RAY * rays
                                     if kern == abi.KERNEL_WAVEFRONT else None),
                         "kernel": (("wf_extend_cw8" if args.bvh_width in (0, 8) else "wf_extend_bvh")
                                    + " (+ wf_finish for the last paths)" if kern == abi.KERNEL_WAVEFRONT
                                    else "k_plain"),
                         "algorithmic_bytes_per_frame": k_bytes, "kernel_ms_per_frame": k_ms,
                         "launches_per_frame": breakdown["rounds"] if kern == abi.KERNEL_WAVEFRONT else 1,
                         "peak_source": peak_kind,
                         "l2": {"peak": l2_gbs, "frac": achieved / l2_gbs,
                                "peak_source": "measured here: reads of a 32 MiB L2-resident buffer, L1 bypassed"},
                         "note": "scene is L2-resident; algorithmic bytes are served mostly by L1/L2"},
            "breakdown": breakdown,
            "tail": tail_summary(rounds, args.tail_paths),
            "clocks": clocks,
            "gpu_launches": args.steps * int(breakdown["launches"]),
        }
        if world == 1 and not args.no_cpu_baseline:
            import pyoracle
            pyoracle.build()
            onodes, oidx, _ = pyoracle.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)
            v, cores, sample, ora, rows = cpu_baseline_sample(wl, (onodes, oidx))
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
            # the oracle's frame from the baseline run is the checker of the
            # benchmarked GPU frame (same seed, same BVH)
            line["parity"] = parity_summary(frame_out, ora, rows)
        if world == 1 and not args.no_batched:
            line["batched"] = batched_section(local, max(3, args.steps // 2), 2)
        if world == 1 and not args.no_adjoint:
            line["adjoint"] = adjoint_section(local, max(3, args.steps // 2))
        if world == 1:
            line["present"] = present_section(local, 20)
            line["small_configs"] = small_configs_section(local, 5, not args.no_cpu_baseline)
        print(json.dumps(line), flush=True)
    tr.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--kernel", choices=["wavefront", "plain"], default="wavefront")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--wavefront", type=int, default=0)
    ap.add_argument("--bvh-width", type=int, default=0, choices=[0, 2, 4, 8],
                    help="wavefront traversal: 0 auto (= 8-wide for triangle-only scenes), 2 binary, 4 4-wide, "
                         "8 compressed 8-wide")
    ap.add_argument("--tail-paths", type=int, default=0,
                    help="wavefront hand-over to the finishing kernel below this many live paths (0 auto, 1 never)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched section")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint section")
    ap.add_argument("--gd-steps", type=int, default=0,
                    help="run only the gradient-descent workload (c4 shape) for this many steps")
    ap.add_argument("--gd-tris", type=int, default=1_000_000)
    ap.add_argument("--gd-checkpoint", default=None, help="gradient descent: .npz file for the optimiser state")
    ap.add_argument("--gd-checkpoint-every", type=int, default=10)
    ap.add_argument("--gd-resume", action="store_true", help="gradient descent: continue from --gd-checkpoint")
    ap.add_argument("--gd-hit-log", action="store_true",
                    help="gradient descent: the adjoint keeps pass 1's hits (tracer_set_adjoint_hit_log)")
    ap.add_argument("--present-only", action="store_true", help="time the present pass alone (--steps launches)")
    # smaller variants of the workload (profiling captures); defaults = c1
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=16)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.gd_steps:
        import torch
        torch.cuda.set_device(dist_setup()[2])
        w = args.width if args.width != 1920 else 1024
        spp = args.spp if args.spp != 16 else 64
        print(json.dumps(gd_section(dist_setup()[2], args.gd_steps, w, spp, args.gd_tris, args.gd_checkpoint,
                                    args.gd_checkpoint_every, args.gd_resume, args.gd_hit_log)), flush=True)
    elif args.present_only:
        import torch
        torch.cuda.set_device(dist_setup()[2])
        print(json.dumps(present_section(dist_setup()[2], args.steps)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
