"""tracer_trace_noalloc: the entry point for callers that must not allocate
device memory while rendering (a frame loop that cannot afford the device-wide
synchronization a cudaMalloc/cudaFree may cause, or an engine that hands the
library only buffers it allocated itself).  It must give the same image as
the regular entry point, call after call, while writing only into the
caller's buffers and its own fixed scratch array.

This file is collected last (its name) so that a run stopping at the first
failure has already run every other test; it also passes on its own in a
fresh process."""
import ctypes

import numpy as np
import pytest

from gpu_cases import IMAGE_RMSE_TOL, rmse, soup_scene
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def _case(emitters=False):
    if emitters:  # the reference's spheres (one emitter: next-event shadow rays) and planes
        ref = S.reference_scene()
        sc = soup_scene(44, 400, extent=30.0, sigma=4.0)
        sc.spheres, sc.planes = ref.spheres, ref.planes
        return sc, S.reference_frame(0.35), 100, 80
    sc = soup_scene(21, 2500, extent=10.0, sigma=0.5)
    fr = S.frame(S.look_at((0.0, 2.0, 30.0), (0.0, 0.0, 0.0), 40.0), 120 / 96, 0.75)
    return sc, fr, 120, 96


@pytest.mark.parametrize("emitters", [False, True])
@pytest.mark.parametrize("tail_paths", [0, 1])
def test_noalloc_matches_regular_trace_twice(gpu_tracer, tail_paths, emitters):
    """Two calls in a row, each equal to tracer_trace's image: the finishing
    kernel after generate (tail_paths 0) and every round launched
    (tail_paths 1), on a triangle soup and on a scene with an emissive sphere
    and planes."""
    import torch
    sc, fr, w, h = _case(emitters)
    tr = gpu_tracer
    tr.upload_scene(sc)
    p = abi.Tracer.params(w, h, spp=3, max_depth=6, rr_start=3, sky=(1.0, 1.0, 1.0),
                          aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F), kernel=abi.KERNEL_WAVEFRONT, tail_paths=tail_paths)
    tr.trace(fr, p)
    ref8 = tr.readback(abi.AOV_RGBA8)
    ref32 = tr.readback(abi.AOV_RGBA32F)
    # caller-owned output buffers (the caller allocated them; the call does not)
    out8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    out32 = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    for call in range(2):
        out8.fill_(7)
        out32.fill_(-5.0)
        torch.cuda.synchronize()
        tr.trace_noalloc(fr, p, out8.data_ptr(), out32.data_ptr())
        torch.cuda.synchronize()
        got8 = out8.cpu().numpy()
        got32 = out32.cpu().numpy()
        e = rmse(got32, ref32)
        assert e <= IMAGE_RMSE_TOL, (call, e)
        assert np.array_equal(got8, ref8), call
        assert np.array_equal(np.isnan(got32[:, 0]), np.isnan(ref32[:, 0]))


def test_noalloc_device_memory_unchanged(gpu_tracer):
    """The property the entry point exists for: once the library's code and
    its fixed array are resident (a first call), further calls take no device
    memory -- the device's free memory is the same before and after a run of
    calls, with both branches (finishing kernel, every round)."""
    import torch
    sc, fr, w, h = _case()
    tr = gpu_tracer
    tr.upload_scene(sc)
    out8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    prm = [abi.Tracer.params(w, h, spp=2, max_depth=4, rr_start=3, sky=(1.0, 1.0, 1.0), tail_paths=t)
           for t in (0, 1)]
    for p in prm:  # first calls: module code and kernels loaded
        tr.trace_noalloc(fr, p, out8.data_ptr(), None)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        for p in prm:
            tr.trace_noalloc(fr, p, out8.data_ptr(), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_single_output_and_limits(gpu_tracer):
    import torch
    sc, fr, w, h = _case()
    tr = gpu_tracer
    tr.upload_scene(sc)
    p = abi.Tracer.params(w, h, spp=2, max_depth=4, rr_start=3, sky=(1.0, 1.0, 1.0), aovs=(abi.AOV_RGBA8,))
    tr.trace(fr, p)
    ref8 = tr.readback(abi.AOV_RGBA8)
    out8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    tr.trace_noalloc(fr, p, out8.data_ptr(), None)
    torch.cuda.synchronize()
    assert np.array_equal(out8.cpu().numpy(), ref8)
    # beyond the scratch array: refused with a message, nothing launched
    big = abi.Tracer.params(256, 256, spp=1, max_depth=2)
    with pytest.raises(abi.TracerError) as e:
        tr.trace_noalloc(fr, big, out8.data_ptr(), None)
    assert e.value.status == abi.ERR_NO_SUITABLE_SURFACE and "no-alloc limit" in str(e.value)
    deep = abi.Tracer.params(16, 16, spp=4096, max_depth=4)
    with pytest.raises(abi.TracerError) as e:
        tr.trace_noalloc(fr, deep, out8.data_ptr(), None)
    assert e.value.status == abi.ERR_INVALID_ARG
    with pytest.raises(abi.TracerError):
        tr.trace_noalloc(fr, p, None, None)
    # binary traversal only: a 4-wide (or unknown) width is refused
    for width in (4, 3):
        wide = abi.Tracer.params(w, h, spp=2, max_depth=4, bvh_width=width)
        with pytest.raises(abi.TracerError) as e:
            tr.trace_noalloc(fr, wide, out8.data_ptr(), None)
        assert e.value.status == abi.ERR_INVALID_ARG
