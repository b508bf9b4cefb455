"""Failure paths that need a GPU but fault nothing: a bounded wait that runs
out returns TRACER_ERR_TIMEOUT and leaves the context usable (the kernel
itself finishes normally); argument checks refuse bad launches before any
kernel runs."""
import numpy as np
import pytest

from gpu_cases import soup_scene
from vktrace import abi, configs
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_then_recovers():
    """A 1 ms wait on a ~200 ms frame (the plain kernel: one launch, so the
    trace call itself never waits): the readback reports a timeout instead of
    blocking; with the default limit back, the same frame completes and
    matches a trace that was never interrupted."""
    wl = configs.c1()
    with abi.Tracer(0) as tr:
        tr.upload_scene(wl.scene)
        p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                              sky=wl.sky, kernel=abi.KERNEL_PLAIN, aovs=(abi.AOV_RGBA8,))
        tr.trace(wl.frame, p)
        tr.synchronize()
        ref = tr.readback(abi.AOV_RGBA8)
        tr.set_timeout(1)
        tr.trace(wl.frame, p)
        with pytest.raises(abi.TracerError) as e:
            tr.readback(abi.AOV_RGBA8)
        assert e.value.status == abi.ERR_TIMEOUT
        tr.set_timeout(60000)
        tr.synchronize()
        again = tr.readback(abi.AOV_RGBA8)
        assert np.array_equal(again, ref)


def test_refused_launches_leave_context_usable(gpu_tracer):
    tr = gpu_tracer
    sc = soup_scene(9, 800)
    tr.upload_scene(sc)
    fr = S.frame(S.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    bad = [
        abi.Tracer.params(0, 16),                                   # empty image
        abi.Tracer.params(16, 16, spp=0),                           # no samples
        abi.Tracer.params(16, 16, tie_mode=abi.TIES_REFERENCE),     # reference ties need a linear scan
        abi.Tracer.params(16, 16, kernel=7),                        # unknown kernel
        abi.Tracer.params(16, 16, kernel=abi.KERNEL_WAVEFRONT, block=96),
        abi.Tracer.params(16, 16, stack_depth=1),                   # below the BVH depth
        abi.Tracer.params(16, 16, aovs=(9,)),                       # unknown AOV
    ]
    for p in bad:
        with pytest.raises(abi.TracerError):
            tr.trace(fr, p)
    p = abi.Tracer.params(16, 16, spp=2, max_depth=3)
    tr.trace(fr, p)
    assert tr.readback(abi.AOV_RGBA8).shape == (16, 16, 4)


def test_no_scene():
    with abi.Tracer(0) as tr:
        with pytest.raises(abi.TracerError) as e:
            tr.trace(S.reference_frame(0.5), abi.Tracer.params(8, 8))
        assert e.value.status == abi.ERR_NO_SCENE


def test_measure_l2_read(gpu_tracer):
    """The L2 read-bandwidth probe: rejects malformed sizes, returns a rate."""
    for nbytes, passes in ((0, 1), (15, 1), (1 << 20, 0), ((1 << 20) + 8, 4)):
        with pytest.raises(abi.TracerError):
            gpu_tracer.measure_l2_read(nbytes, passes)
    gbs = gpu_tracer.measure_l2_read(8 << 20, 16)
    assert 100.0 < gbs < 1e6


@pytest.mark.parametrize("kernel,tail", [(abi.KERNEL_PLAIN, 0), (abi.KERNEL_WAVEFRONT, 1),
                                         (abi.KERNEL_WAVEFRONT, 0)])
def test_traversal_limit_fires_then_recovers(gpu_tracer, kernel, tail):
    """The device-side traversal step cap, lowered to a handful of steps,
    stops rays mid-traversal: the kernels finish, the wait reports
    TRACER_ERR_TRAVERSAL_LIMIT, and with the automatic cap back the same
    context traces the frame as before (the plain kernel, the wavefront's
    rounds, and its finishing kernel)."""
    tr = gpu_tracer
    sc = soup_scene(12, 3000, extent=10.0, sigma=0.5)
    tr.upload_scene(sc)
    fr = S.frame(S.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.5)
    p = abi.Tracer.params(64, 64, spp=2, max_depth=4, rr_start=3, sky=(1, 1, 1), kernel=kernel, tail_paths=tail,
                          aovs=(abi.AOV_RGBA32F,))
    tr.trace(fr, p)
    ref = tr.readback(abi.AOV_RGBA32F)
    try:
        tr.set_traversal_limit(3)
        tr.trace(fr, p)
        with pytest.raises(abi.TracerError) as e:
            tr.synchronize()
        assert e.value.status == abi.ERR_TRAVERSAL_LIMIT
    finally:
        tr.set_traversal_limit(0)
    tr.trace(fr, p)
    again = tr.readback(abi.AOV_RGBA32F)
    assert np.array_equal(np.nan_to_num(again, nan=-7.0), np.nan_to_num(ref, nan=-7.0))
