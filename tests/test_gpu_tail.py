"""The wavefront's finishing kernel (tracer_trace_params.tail_paths): once few
paths are live, one launch runs each of them to the end of its pixel.  The
image, hits and ray counts must not depend on where the hand-over happens:
never, before any round (every path still live) or part-way through."""
import numpy as np
import pytest

from conftest import fbits

from gpu_cases import compare, run_gpu, run_oracle, soup_scene, sphere_scene
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu

NEVER = 1  # no path count is below 1 while paths remain
ALWAYS = 0xFFFFFFFF  # more than any frame's pixels: no round, the finishing kernel after generate


def _same(a, b, what):
    assert np.array_equal(fbits(a["rgba32f"]), fbits(b["rgba32f"])), what
    assert np.array_equal(a["rgba8"], b["rgba8"]), what
    assert np.array_equal(a["hit_id"], b["hit_id"]), what
    assert np.array_equal(fbits(a["hit_t"]), fbits(b["hit_t"])), what
    for k in ("closest_rays", "shadow_rays", "hits"):
        assert a["stats"][k] == b["stats"][k], (what, k)


def _mixed_scene():
    sc = soup_scene(7, 3000, extent=12.0, sigma=0.6)
    ref = S.reference_scene()
    sc.spheres = ref.spheres  # one emitter: next-event shadow rays inside the finishing kernel
    sc.planes = ref.planes
    return sc


@pytest.mark.parametrize("tail", [ALWAYS, 3000, 300])
def test_tail_soup_identical(gpu_tracer, tail):
    sc = soup_scene(5, 4000, extent=12.0, sigma=0.5)
    fr = S.frame(S.look_at((0.0, 3.0, 30.0), (0.0, 0.0, 0.0), 40.0), 96 / 80, 0.7)
    args = (sc, fr, 96, 80, 4, 8)
    kw = dict(rr_start=3, sky=(1.0, 0.95, 0.9))
    plain = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_PLAIN, **kw)
    rounds = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=NEVER, **kw)
    tailed = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=tail, **kw)
    _same(rounds, plain, "rounds vs plain")
    _same(tailed, plain, f"tail {tail} vs plain")


def test_tail_emitters_and_planes(gpu_tracer):
    """BVH + spheres + planes + an emitter (shadow rays in the finishing kernel)."""
    sc = _mixed_scene()
    fr = S.frame(S.look_at((0.0, 4.0, 28.0), (0.0, 0.0, 0.0), 45.0), 1.25, 0.2)
    args = (sc, fr, 80, 64, 3, 6)
    kw = dict(rr_start=2, sky=(0.5, 0.6, 0.7))
    plain = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_PLAIN, **kw)
    for tail in (ALWAYS, 1000):
        _same(run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=tail, **kw), plain, tail)
    o = run_oracle(sc, fr, 80, 64, 3, 6, **kw)
    compare(run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=ALWAYS, **kw), o)


def test_tail_reference_scene(gpu_tracer):
    """Linear scan with the reference's tie rule, emitter, RR at every depth."""
    sc = S.reference_scene()
    fr = S.reference_frame(0.5)
    args = (sc, fr, 160, 128, 4, 4)
    kw = dict(tie=abi.TIES_REFERENCE)
    plain = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_PLAIN, **kw)
    for tail in (NEVER, ALWAYS, 5000):
        _same(run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=tail, **kw), plain, tail)


def test_tail_spheres(gpu_tracer):
    sc = sphere_scene(9)
    fr = S.frame(S.look_at((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.0)
    args = (sc, fr, 64, 64, 2, 5)
    kw = dict(rr_start=1, sky=(1.0, 1.0, 1.0))
    plain = run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_PLAIN, **kw)
    _same(run_gpu(gpu_tracer, *args, kernel=abi.KERNEL_WAVEFRONT, tail_paths=ALWAYS, **kw), plain, "spheres")


def test_round_statistics(gpu_tracer):
    """tracer_last_rounds: live paths per round (all pixels first, never
    growing), the finishing kernel as the last entry, times recorded."""
    sc = soup_scene(5, 4000, extent=12.0, sigma=0.5)
    fr = S.frame(S.look_at((0.0, 3.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.7)
    gpu_tracer.upload_scene(sc)
    gpu_tracer.set_profiling(True)
    try:
        for tail in (NEVER, 2000, ALWAYS):
            p = abi.Tracer.params(64, 64, spp=4, max_depth=8, rr_start=3, sky=(1.0, 1.0, 1.0),
                                  kernel=abi.KERNEL_WAVEFRONT, tail_paths=tail)
            gpu_tracer.trace(fr, p)
            r = gpu_tracer.rounds()
            t = gpu_tracer.timings()
            assert len(r) >= 1
            assert r["paths"][0] == 64 * 64
            assert np.all(np.diff(r["paths"].astype(np.int64)) <= 0)
            assert np.all(r["extend_ms"] > 0)
            fin = r["finish"] == 1
            if tail == NEVER:
                assert not fin.any() and t["finish_ms"] == 0.0
                # the loop notices the empty queue three rounds late: at most
                # three empty rounds, all at the end
                empty = r["paths"] == 0
                assert 1 <= empty.sum() <= 3 and empty[-1]
            else:
                assert fin[-1] and fin.sum() == 1
                assert r["shade_ms"][-1] == 0.0 and t["finish_ms"] > 0.0
                f = len(r) - 1
                if tail == ALWAYS:
                    assert f == 0  # fewer pixels than the threshold: no round at all
                else:
                    # the count that triggered the hand-over is read three rounds late
                    assert r["paths"][f - 3] < tail
                    if f >= 5:
                        assert r["paths"][f - 4] >= tail
            assert t["rounds"] == int((~fin).sum())
    finally:
        gpu_tracer.set_profiling(False)


def test_tail_batched_rounds_equal_graph(gpu_tracer):
    """Batched without a graph hands over to the finishing kernel too; the
    graph (fixed rounds) must give the same bits."""
    scenes = [soup_scene(40, 600), soup_scene(41, 3000, extent=20.0), _mixed_scene()]
    sizes = [(24, 16), (64, 48), (40, 32)]
    frames = [S.frame(S.look_at((1.0 * i, 2.0, 30.0), (0.0, 0.0, 0.0), 40.0), w / h, 0.1 * i)
              for i, (w, h) in enumerate(sizes)]
    params = [abi.Tracer.params(w, h, spp=2 + i, max_depth=4 + i, rr_start=2, sky=(1.0, 0.9, 0.8),
                                aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F), tail_paths=ALWAYS)
              for i, (w, h) in enumerate(sizes)]
    tr = gpu_tracer
    tr.upload_scenes(scenes)
    tr.trace_batched(frames, params, use_graph=False)
    tailed = [tr.readback_scene(i, abi.AOV_RGBA32F).copy() for i in range(len(scenes))]
    tr.trace_batched(frames, params, use_graph=True)
    graph = [tr.readback_scene(i, abi.AOV_RGBA32F).copy() for i in range(len(scenes))]
    for i in range(len(scenes)):
        assert np.array_equal(fbits(tailed[i]), fbits(graph[i])), i


def test_graph_handover_replayed_for_other_frames(gpu_tracer):
    """A batch graph takes its hand-over round from the run that captured it;
    replayed for other frames (other cameras and seeds, so other path
    lengths) it must still trace them completely."""
    scenes = [soup_scene(40, 600), soup_scene(41, 3000, extent=20.0), _mixed_scene()]
    sizes = [(48, 32), (64, 48), (40, 32)]

    def frames(shift):
        return [S.frame(S.look_at((1.0 * i + shift, 2.0 - shift, 30.0), (0.0, 0.0, 0.0), 40.0), w / h,
                        0.1 * i + shift) for i, (w, h) in enumerate(sizes)]

    def params(tail):
        return [abi.Tracer.params(w, h, spp=3, max_depth=5 + i, rr_start=2, sky=(1.0, 0.9, 0.8),
                                  aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F), tail_paths=tail)
                for i, (w, h) in enumerate(sizes)]

    tr = gpu_tracer
    tr.upload_scenes(scenes)
    tr.trace_batched(frames(0.0), params(1500), use_graph=True)  # capture
    for shift in (0.0, 3.0, -2.5):
        tr.trace_batched(frames(shift), params(1500), use_graph=True)  # replay
        got = [tr.readback_scene(i, abi.AOV_RGBA32F).copy() for i in range(len(scenes))]
        tr.trace_batched(frames(shift), params(NEVER), use_graph=False)
        want = [tr.readback_scene(i, abi.AOV_RGBA32F).copy() for i in range(len(scenes))]
        for i in range(len(scenes)):
            assert np.array_equal(fbits(got[i]), fbits(want[i])), (shift, i)


def test_auto_kernel_choice(gpu_tracer):
    """TRACER_KERNEL_AUTO: the wavefront (more than one launch) for BVH scenes
    from 2^16 pixel x spp x depth when the scene has an 8-wide BVH (triangles
    only; bvh_width 0 or 8), from 2^22 otherwise (bvh_width 2 asked for, or
    spheres in the scene), else the plain kernel (one launch); linear-scan
    scenes plain."""
    sc = soup_scene(5, 4000, extent=12.0, sigma=0.5)
    sph = soup_scene(5, 4000, extent=12.0, sigma=0.5)
    sph.spheres = S.random_spheres(9, 4)  # spheres: no 8-wide BVH
    fr = S.frame(S.look_at((0.0, 3.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.7)
    gpu_tracer.set_profiling(True)
    try:
        for scene, width, (w, h, spp, depth), wavefront in (
                ("tris", 0, (64, 64, 2, 4), False),        # 2^15
                ("tris", 0, (128, 128, 1, 4), True),       # 2^16
                ("tris", 0, (256, 256, 4, 4), True),
                ("tris", 2, (256, 256, 4, 4), False),
                ("tris", 2, (512, 512, 4, 4), True),
                ("spheres", 0, (256, 256, 4, 4), False),
                ("spheres", 0, (512, 512, 4, 4), True),
                ("linear", 0, (512, 512, 4, 4), False)):
            if scene == "tris":
                gpu_tracer.upload_scene(sc)
            elif scene == "spheres":
                gpu_tracer.upload_scene(sph)
            else:
                gpu_tracer.upload_scene(S.Scene(triangles=sc.triangles[:200], materials=sc.materials,
                                                bvh=S.BVH_NONE))
            p = abi.Tracer.params(w, h, spp=spp, max_depth=depth, rr_start=2, sky=(1.0, 1.0, 1.0),
                                  kernel=abi.KERNEL_AUTO, bvh_width=width)
            gpu_tracer.trace(fr, p)
            assert (gpu_tracer.timings()["launches"] > 1) == wavefront, (scene, width, w, h, spp, depth)
    finally:
        gpu_tracer.set_profiling(False)
