"""Host-side logic of the autotuner and of the bench's round summary, on CPU
with a stand-in for the tracer (no GPU, no CUDA library calls)."""
import sys

import numpy as np
import pytest

from conftest import REPO

sys.path.insert(0, REPO)

from vktrace import abi, tune  # noqa: E402


class FakeTracer:
    """Records the launch shape of every batched trace and reports a time
    that depends on it; refuses stacks below a minimum, as the library does."""

    def __init__(self, min_stack=8, slow_call=None):
        self.calls = []
        self.min_stack = min_stack
        self.profiling = False
        self.last_ms = 0.0
        self.slow_call = slow_call

    def set_profiling(self, on):
        self.profiling = on

    def synchronize(self):
        pass

    def trace_batched(self, frames, params, use_graph=True):
        p = params[0]
        shape = (p.block, p.stack_depth, p.wavefront, p.bvh_width, p.tail_paths)
        self.calls.append(shape)
        if self.slow_call is not None:
            self.slow_call()
        if p.stack_depth and p.stack_depth < self.min_stack:
            raise abi.TracerError(abi.ERR_STACK_OVERFLOW, "stack depth below the BVH depth")
        # fastest: block 128, stack 0, wavefront 6, width 2, tail 1000
        self.last_ms = (10.0 + abs(p.block - 128) / 64 + (p.stack_depth != 0) + abs(p.wavefront - 6) / 2
                        + (p.bvh_width != 2) * 3 + (p.tail_paths != 1000) * 0.5)

    def timings(self):
        assert self.profiling
        return {"total_ms": self.last_ms}


def _params(n=3):
    return [abi.Tracer.params(64, 64, spp=2, max_depth=3, block=0, stack_depth=0, wavefront=0, bvh_width=0,
                              tail_paths=0) for _ in range(n)]


def test_autotune_picks_fastest_and_restores_params():
    tr = FakeTracer()
    params = _params()
    best, table = tune.autotune_batched(tr, [None] * 3, params, blocks=(64, 128, 256), stacks=(0, 4, 16),
                                        wavefronts=(0, 6), widths=(4, 2), tails=(0, 1000), reps=2)
    assert len(table) == 3 * 3 * 2 * 2 * 2
    assert best["block"] == 128 and best["stack_depth"] == 0 and best["wavefront"] == 6
    assert best["bvh_width"] == 2 and best["tail_paths"] == 1000
    assert best["ms"] == pytest.approx(10.0)
    skipped = [r for r in table if "skipped" in r]
    assert skipped and all(r["stack_depth"] == 4 for r in skipped)
    assert all("stack depth" in r["skipped"] for r in skipped)
    # every candidate traced once to capture and reps times to time (refused ones once), then
    # the 3 fastest once more to capture and 5 times each
    assert len(tr.calls) == (len(table) - len(skipped)) * 3 + len(skipped) + 3 * (1 + 5)
    refined = [r for r in table if "ms_refined" in r]
    assert len(refined) == 3 and min(r["ms_refined"] for r in refined) == best["ms"]
    for p in params:
        assert (p.block, p.stack_depth, p.wavefront, p.bvh_width, p.tail_paths) == (0, 0, 0, 0, 0)
    assert not tr.profiling


def test_autotune_refine_overrules_a_noisy_first_sample():
    """A candidate that was lucky once loses to the one whose repeated
    timings are faster."""
    tr = FakeTracer()
    lucky = {"n": 0}
    base_trace = tr.trace_batched

    def trace(frames, params, use_graph=True):
        base_trace(frames, params, use_graph)
        p = params[0]
        if p.block == 256:  # a slow shape with one lucky sample in the sweep
            lucky["n"] += 1
            tr.last_ms = 5.0 if lucky["n"] == 2 else 30.0
    tr.trace_batched = trace
    best, table = tune.autotune_batched(tr, [None], _params(1), blocks=(128, 256), stacks=(0,), wavefronts=(6,),
                                        widths=(2,), tails=(1000,), reps=1)
    assert [r["ms"] for r in table if r["block"] == 256] == [5.0]
    assert best["block"] == 128 and best["ms"] == pytest.approx(10.0)


def test_autotune_time_budget():
    import time
    tr = FakeTracer(slow_call=lambda: time.sleep(0.02))
    best, table = tune.autotune_batched(tr, [None], _params(1), blocks=(64, 128, 256), stacks=(0,),
                                        wavefronts=(0, 6, 4), widths=(2,), budget_s=0.05)
    assert best is not None
    assert any(r.get("skipped") == "time budget" for r in table)
    assert len(table) == 9


def _rounds(paths, ext, sh, finish_last):
    dt = np.dtype([("paths", np.uint32), ("finish", np.uint32), ("extend_ms", np.float32),
                   ("shade_ms", np.float32)])
    r = np.zeros(len(paths), dt)
    r["paths"], r["extend_ms"], r["shade_ms"] = paths, ext, sh
    if finish_last:
        r["finish"][-1] = 1
        r["shade_ms"][-1] = 0.0
    return r


def test_tail_summary():
    import bench
    r = _rounds([1000, 1000, 600, 400, 90, 80], [2.0, 2.0, 1.5, 1.0, 0.5, 0.7], [0.1, 0.1, 0.1, 0.1, 0.05, 0.0],
                finish_last=True)
    s = bench.tail_summary(r, 0)
    assert s["rounds"] == 5 and s["first_round_paths"] == 1000
    assert s["handover_paths"] == 80 and s["finish_ms"] == pytest.approx(0.7)
    assert s["ms_in_rounds_with_half_the_paths_or_more"] == pytest.approx(2.1 + 2.1 + 1.6)
    assert "auto" in s["tail_paths"]
    s = bench.tail_summary(_rounds([10, 5, 0], [1.0, 1.0, 0.1], [0.1, 0.1, 0.1], finish_last=False), 1)
    assert s["rounds"] == 3 and "handover_paths" not in s and s["tail_paths"] == 1
    assert bench.tail_summary(None, 0) is None
