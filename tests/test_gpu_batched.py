"""Batched tracing: many scenes of uneven size and resolution in one device
arena and one wavefront (optionally one CUDA graph).  Every scene's image
must equal, bit for bit, its single-scene trace, and the per-scene plain
baseline must equal both."""
import numpy as np
import pytest

from conftest import fbits

from gpu_cases import compare, run_oracle, scene_bvhs, soup_scene, sphere_scene
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def _batch():
    ref = S.reference_scene()
    mixed = soup_scene(44, 400, extent=30.0, sigma=4.0)
    mixed.spheres = ref.spheres
    mixed.planes = ref.planes
    scenes = [soup_scene(40, 600), soup_scene(41, 5000, extent=20.0), sphere_scene(42), soup_scene(43, 1500),
              mixed]
    sizes = [(16, 16), (96, 64), (33, 17), (64, 64), (48, 40)]
    frames = []
    for i, (w, h) in enumerate(sizes):
        if i == 4:
            frames.append(S.reference_frame(0.1 * i))
        else:
            frames.append(S.frame(S.look_at((1.0 * i, 2.0, 30.0), (0.0, 0.0, 0.0), 40.0), w / h, 0.1 * i))
    params = [abi.Tracer.params(w, h, spp=2 + (i % 2), max_depth=3 + i, rr_start=2, sky=(1.0, 0.9, 0.8),
                                aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT))
              for i, (w, h) in enumerate(sizes)]
    return scenes, frames, params


def _single(tr, sc, fr, p):
    tr.upload_scene(sc)
    tr.trace(fr, p)
    return tr.readback(abi.AOV_RGBA32F), tr.readback(abi.AOV_PRIMARY_HIT)


def _bits(a):
    return fbits(a)


@pytest.mark.parametrize("width", [2, 4])
def test_batched_equals_single_scene(gpu_tracer, width):
    """Binary and 4-wide traversal of the batch; the single-scene references
    use the other width, so the two widths are compared too."""
    tr = gpu_tracer
    scenes, frames, params = _batch()
    for p in params:
        p.bvh_width = 6 - width
    singles = [_single(tr, sc, fr, p) for sc, fr, p in zip(scenes, frames, params)]
    for p in params:
        p.bvh_width = width
    tr.upload_scenes(scenes)
    for use_graph in (False, True, True):  # the second graph run replays the captured graph
        tr.trace_batched(frames, params, use_graph=use_graph)
        for k in range(len(scenes)):
            img = tr.readback_scene(k, abi.AOV_RGBA32F)
            hit = tr.readback_scene(k, abi.AOV_PRIMARY_HIT)
            assert np.array_equal(_bits(img), _bits(singles[k][0])), (use_graph, k)
            assert np.array_equal(hit, singles[k][1]), (use_graph, k)
    for p in params:
        p.kernel = abi.KERNEL_PLAIN
    tr.trace_batched(frames, params, use_graph=False)
    for k in range(len(scenes)):
        assert np.array_equal(_bits(tr.readback_scene(k, abi.AOV_RGBA32F)), _bits(singles[k][0])), ("plain", k)


def test_batched_cw8_equals_single_scene(gpu_tracer):
    """A batch of triangle-only scenes through the compressed 8-wide
    traversal (each scene's nodes and triangles packed in the arena) equals
    every scene's single-scene binary trace, graph and non-graph."""
    tr = gpu_tracer
    scenes = [soup_scene(60, 700), soup_scene(61, 6000, extent=25.0), soup_scene(62, 1), soup_scene(63, 2500)]
    sizes = [(24, 20), (80, 64), (9, 7), (64, 48)]
    frames = [S.frame(S.look_at((1.5 * i, 2.0, 30.0), (0.0, 0.0, 0.0), 40.0), w / h, 0.2 * i)
              for i, (w, h) in enumerate(sizes)]
    params = [abi.Tracer.params(w, h, spp=2, max_depth=4 + i, rr_start=2, sky=(1.0, 0.9, 0.8),
                                aovs=(abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT), kernel=abi.KERNEL_WAVEFRONT,
                                bvh_width=2, tail_paths=1)
              for i, (w, h) in enumerate(sizes)]
    singles = [_single(tr, sc, fr, p) for sc, fr, p in zip(scenes, frames, params)]
    for p in params:
        p.bvh_width = 8
    tr.upload_scenes(scenes)
    for use_graph in (False, True):
        tr.trace_batched(frames, params, use_graph=use_graph)
        for k in range(len(scenes)):
            assert np.array_equal(_bits(tr.readback_scene(k, abi.AOV_RGBA32F)), _bits(singles[k][0])), (use_graph, k)
            assert np.array_equal(tr.readback_scene(k, abi.AOV_PRIMARY_HIT), singles[k][1]), (use_graph, k)


def test_batched_against_oracle(gpu_tracer):
    tr = gpu_tracer
    scenes, frames, params = _batch()
    tr.upload_scenes(scenes)
    tr.trace_batched(frames, params, use_graph=True)
    for k in (1, 2, 4):
        p = params[k]
        g = {"rgba32f": tr.readback_scene(k, abi.AOV_RGBA32F)}
        hit = tr.readback_scene(k, abi.AOV_PRIMARY_HIT)
        g["hit_id"], g["hit_t"] = hit[..., 0].copy(), hit[..., 1].copy().view(np.float32)
        o = run_oracle(scenes[k], frames[k], p.width, p.height, p.spp, p.max_depth, rr_start=p.rr_start,
                       sky=tuple(p.sky))
        compare(g, o, check_stats=False)


def test_graph_replay_follows_new_frames(gpu_tracer):
    """A replayed graph reads the per-scene table written for this call: a
    moved camera gives the moved image."""
    tr = gpu_tracer
    scenes, frames, params = _batch()
    tr.upload_scenes(scenes)
    tr.trace_batched(frames, params, use_graph=True)
    moved = list(frames)
    moved[0] = S.frame(S.look_at((5.0, -3.0, 28.0), (1.0, 0.0, 0.0), 35.0), 1.0, 0.9)
    tr.trace_batched(moved, params, use_graph=True)
    a = tr.readback_scene(0, abi.AOV_RGBA32F)
    tr.trace_batched(moved, params, use_graph=False)
    b = tr.readback_scene(0, abi.AOV_RGBA32F)
    assert np.array_equal(_bits(a), _bits(b))
    single, _ = _single(tr, scenes[0], moved[0], params[0])
    assert np.array_equal(_bits(a), _bits(single))


def test_timings_after_graph_and_autotune(gpu_tracer):
    """Per-kernel timings after a graph replay (no per-round events exist) and
    the autotuner's sweep over launch shapes."""
    from vktrace import tune
    tr = gpu_tracer
    scenes, frames, params = _batch()
    tr.upload_scenes(scenes)
    for p in params:
        p.tail_paths = 1  # rounds to the end (this small batch would otherwise run no round)
    tr.set_profiling(True)
    try:
        tr.trace_batched(frames, params, use_graph=True)
        t = tr.timings()
        assert t["total_ms"] > 0 and t["extend_ms"] == 0 and t["rounds"] > 0
        tr.trace_batched(frames, params, use_graph=False)
        t = tr.timings()
        assert t["extend_ms"] > 0 and t["shade_ms"] > 0
    finally:
        tr.set_profiling(False)
    for p in params:
        p.tail_paths = 0
    best, table = tune.autotune_batched(tr, frames, params, blocks=(64, 128), stacks=(4, 32), wavefronts=(0, 2),
                                        tails=(0, 1))
    assert best is not None and best["ms"] > 0
    assert any("skipped" in r for r in table)  # stack 4 is below the BVH depth
    assert len(table) == 48  # widths 8, 4 and 2, tails auto and never
    # the batch has spheres: no 8-wide BVH, those candidates are refused
    assert all("skipped" in r for r in table if r["bvh_width"] == 8)
    assert best["bvh_width"] in (2, 4) and best["tail_paths"] in (0, 1)
    assert all(p.tail_paths == 0 for p in params)  # the parameters are restored


def test_batched_argument_errors(gpu_tracer):
    tr = gpu_tracer
    scenes, frames, params = _batch()
    with pytest.raises(abi.TracerError):
        tr.upload_scenes([S.Scene(triangles=scenes[0].triangles, materials=scenes[0].materials, bvh=S.BVH_NONE)])
    tr.upload_scenes(scenes)
    with pytest.raises(abi.TracerError):
        tr.trace_batched(frames[:2], params[:2])  # wrong scene count
    bad = [abi.Tracer.params(p.width, p.height, spp=1, max_depth=2, tie_mode=abi.TIES_REFERENCE) for p in params]
    with pytest.raises(abi.TracerError):
        tr.trace_batched(frames, bad)
