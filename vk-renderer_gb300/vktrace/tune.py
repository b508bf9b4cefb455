"""Autotuner for the wavefront launch shape.

Sweeps the extend kernel's block size, the traversal stack depth (0 = the
bound the BVH needs), the traversal width (compressed 8-wide, 4-wide or
binary nodes) and the "wavefront size" (resident extend CTAs per SM, i.e.
how many rays are in flight at once), timing each candidate on the device
with CUDA events (tracer_last_timings); then times the `refine` fastest
candidates again, `refine_reps` times each, and returns the one with the
smallest median, so that one noisy sample does not pick the launch shape.
Candidates the library refuses (a stack shallower than the BVH, a shape that
cannot be resident, a width the scenes lack) are recorded as skipped.
Results are deterministic given the timings.
"""
from __future__ import annotations

import itertools
import time

from . import abi


def _set(params, block, stack, wave, width, tail=0):
    for p in params:
        p.block, p.stack_depth, p.wavefront, p.bvh_width, p.tail_paths = block, stack, wave, width, tail


def autotune_batched(tr: abi.Tracer, frames, params, blocks=(64, 128, 256), stacks=(0, 16, 32, 64),
                     wavefronts=(0, 6, 4), widths=(8, 4, 2), tails=(0,), reps: int = 1, use_graph: bool = True,
                     budget_s: float = 60.0, refine: int = 3, refine_reps: int = 5):
    """Returns (best, table): best = dict(block, stack_depth, wavefront,
    bvh_width, tail_paths, ms); table = one dict per candidate (ms or
    skipped reason; the re-timed ones also ms_refined).  tails: tail_paths
    values (live paths below which the rest goes to the finishing kernel;
    0 = the library's choice)."""
    table = []
    best = None
    t_start = time.perf_counter()
    saved = [(p.block, p.stack_depth, p.wavefront, p.bvh_width, p.tail_paths) for p in params]
    tr.set_profiling(True)
    try:
        for width, block, stack, wave, tail in itertools.product(widths, blocks, stacks, wavefronts, tails):
            cand = {"block": block, "stack_depth": stack, "wavefront": wave, "bvh_width": width, "tail_paths": tail}
            if time.perf_counter() - t_start > budget_s:
                table.append(dict(cand, skipped="time budget"))
                continue
            _set(params, block, stack, wave, width, tail)
            try:
                tr.trace_batched(frames, params, use_graph=use_graph)  # first run: graph capture, caches warm
                tr.synchronize()
                times = []
                for _ in range(reps):
                    tr.trace_batched(frames, params, use_graph=use_graph)
                    times.append(tr.timings()["total_ms"])
                ms = sorted(times)[len(times) // 2]
            except abi.TracerError as e:
                table.append(dict(cand, skipped=str(e)))
                continue
            row = dict(cand, ms=ms)
            table.append(row)
            if best is None or ms < best["ms"]:
                best = dict(row)
        # second stage: the fastest few again, several times each
        timed = sorted((r for r in table if "ms" in r), key=lambda r: r["ms"])[:max(0, refine)]
        if len(timed) > 1 and refine_reps > 0:
            for row in timed:
                _set(params, row["block"], row["stack_depth"], row["wavefront"], row["bvh_width"], row["tail_paths"])
                tr.trace_batched(frames, params, use_graph=use_graph)
                tr.synchronize()
                times = []
                for _ in range(refine_reps):
                    tr.trace_batched(frames, params, use_graph=use_graph)
                    times.append(tr.timings()["total_ms"])
                row["ms_refined"] = sorted(times)[len(times) // 2]
            top = min(timed, key=lambda r: r["ms_refined"])
            best = dict(top, ms=top["ms_refined"])
    finally:
        tr.set_profiling(False)
        for p, (b, s, w, wd, tl) in zip(params, saved):
            p.block, p.stack_depth, p.wavefront, p.bvh_width, p.tail_paths = b, s, w, wd, tl
    return best, table


def autotune_single(tr: abi.Tracer, frame, params, blocks=(64, 128, 256), stacks=(0,), wavefronts=(0, 6, 4),
                    reps: int = 1, budget_s: float = 60.0):
    """The same sweep for one scene (tracer_trace, wavefront kernel)."""
    table = []
    best = None
    t_start = time.perf_counter()
    saved = (params.block, params.stack_depth, params.wavefront)
    tr.set_profiling(True)
    try:
        for block, stack, wave in itertools.product(blocks, stacks, wavefronts):
            if time.perf_counter() - t_start > budget_s:
                table.append({"block": block, "stack_depth": stack, "wavefront": wave, "skipped": "time budget"})
                continue
            params.block, params.stack_depth, params.wavefront = block, stack, wave
            try:
                tr.trace(frame, params)
                tr.synchronize()
                times = []
                for _ in range(reps):
                    tr.trace(frame, params)
                    times.append(tr.timings()["total_ms"])
                ms = sorted(times)[len(times) // 2]
            except abi.TracerError as e:
                table.append({"block": block, "stack_depth": stack, "wavefront": wave, "skipped": str(e)})
                continue
            row = {"block": block, "stack_depth": stack, "wavefront": wave, "ms": ms}
            table.append(row)
            if best is None or ms < best["ms"]:
                best = dict(row)
    finally:
        tr.set_profiling(False)
        params.block, params.stack_depth, params.wavefront = saved
    return best, table
