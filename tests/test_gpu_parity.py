"""GPU parity: the CUDA kernels against the oracle, through the C ABI.

Bar (the benchmark spec): primary-hit primitive ids bit-exact except ties within
1e-6 in t; hit t within 1e-5 relative; float image RMSE <= 1e-3 at equal
sample counts; the ray / node / primitive-test counters equal the oracle's.
"""
import numpy as np
import pytest

from conftest import fbits

from gpu_cases import compare, run_gpu, run_oracle, soup_scene, sphere_scene
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu

KERNELS = [abi.KERNEL_PLAIN, abi.KERNEL_WAVEFRONT]


@pytest.mark.parametrize("kernel", KERNELS)
def test_reference_scene(gpu_tracer, kernel):
    """The reference's own configuration (linear scan, reference ties,
    emitter with next-event estimation, RR at every depth), reduced size."""
    sc = S.reference_scene()
    fr = S.reference_frame(0.5)
    g = run_gpu(gpu_tracer, sc, fr, 160, 128, 4, 4, tie=abi.TIES_REFERENCE, kernel=kernel)
    o = run_oracle(sc, fr, 160, 128, 4, 4, tie=0)
    r = compare(g, o)
    # Paths are identical; remaining differences are last-ulp powf results
    # (CUDA vs the host C library) in next-event shading and the 1/2.2 gamma.
    assert r["rmse"] < 1e-6, r


def test_reference_scene_full_size(gpu_tracer):
    """Ref: 1024x1024, 4 spp, depth 4 (Source/Main.cpp:112, Tracer.comp:179-180)."""
    sc = S.reference_scene()
    fr = S.reference_frame(0.5)
    g = run_gpu(gpu_tracer, sc, fr, 1024, 1024, 4, 4, tie=abi.TIES_REFERENCE, kernel=abi.KERNEL_WAVEFRONT)
    o = run_oracle(sc, fr, 1024, 1024, 4, 4, tie=0)
    compare(g, o)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("sky", [(0.0, 0.0, 0.0), (1.0, 1.0, 1.0)])
def test_spheres_median_bvh(gpu_tracer, kernel, sky):
    """64 spheres, median-split BVH leaf 2, 1 spp, depth 2 (spheres workload,
    reduced resolution).  sky = 0 is the workload as specified (black plus
    dither: hits are the meaningful check); sky = 1 exercises the image."""
    sc = sphere_scene(0)
    nodes, idx, _ = abi.build_bvh(S.BVH_MEDIAN, sc.spheres, leaf_size=2)
    fr = S.frame(S.look_at((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.0)
    g = run_gpu(gpu_tracer, sc, fr, 128, 128, 1, 2, sky=sky, kernel=kernel, sphere_bvh=(nodes, idx))
    o = run_oracle(sc, fr, 128, 128, 1, 2, sky=sky, sphere_bvh=(nodes, idx))
    compare(g, o)
    assert (g["hit_id"] != 0xFFFFFFFF).mean() > 0.05


@pytest.mark.parametrize("kernel", KERNELS)
def test_triangle_soup_sah(gpu_tracer, kernel):
    """Triangle soup with a 16-bin SAH BVH (leaf 4), sky 1, RR from depth 3."""
    sc = soup_scene(1, 3000, extent=10.0, sigma=0.5)
    nodes, idx, _ = abi.build_bvh(S.BVH_SAH, sc.triangles, leaf_size=4, sah_bins=16)
    fr = S.frame(S.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), 40.0), 96 / 80, 1.0)
    g = run_gpu(gpu_tracer, sc, fr, 96, 80, 4, 8, rr_start=3, sky=(1, 1, 1), kernel=kernel, tri_bvh=(nodes, idx))
    o = run_oracle(sc, fr, 96, 80, 4, 8, rr_start=3, sky=(1, 1, 1), tri_bvh=(nodes, idx))
    compare(g, o)


def test_kernels_identical(gpu_tracer):
    """The plain and wavefront kernels compute the same bits."""
    sc = soup_scene(2, 2000)
    fr = S.frame(S.look_at((0.0, 5.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    a = run_gpu(gpu_tracer, sc, fr, 77, 61, 3, 6, rr_start=2, sky=(0.8, 0.9, 1.0), kernel=abi.KERNEL_PLAIN)
    b = run_gpu(gpu_tracer, sc, fr, 77, 61, 3, 6, rr_start=2, sky=(0.8, 0.9, 1.0), kernel=abi.KERNEL_WAVEFRONT)
    assert np.array_equal(fbits(a["rgba32f"]), fbits(b["rgba32f"]))
    assert np.array_equal(a["rgba8"], b["rgba8"])
    assert np.array_equal(a["hit_id"], b["hit_id"])
    for k in ("closest_rays", "shadow_rays", "hits"):
        assert a["stats"][k] == b["stats"][k]


@pytest.mark.parametrize("prims", ["triangles", "spheres", "mixed"])
def test_wide_traversal_identical(gpu_tracer, prims):
    """The wavefront's 4-wide traversal (nodes collapsed from the binary BVH,
    same boxes) and, for triangle-only scenes, its compressed 8-wide traversal
    (quantised boxes containing the binary ones) give the binary traversal's
    and the plain kernel's bits."""
    ref = S.reference_scene()
    if prims == "spheres":
        sc = sphere_scene(3)
    else:
        sc = soup_scene(6, 4000, extent=12.0, sigma=0.5)
        if prims == "mixed":
            sc.spheres = ref.spheres  # one emitter: next-event shadow rays too
    fr = S.frame(S.look_at((0.0, 3.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.2, 0.4)
    out = {}
    runs = [("plain", abi.KERNEL_PLAIN, 0), ("binary", abi.KERNEL_WAVEFRONT, 2), ("wide", abi.KERNEL_WAVEFRONT, 4)]
    if prims == "triangles":
        runs.append(("cw8", abi.KERNEL_WAVEFRONT, 8))
    for name, kernel, width in runs:
        gpu_tracer.upload_scene(sc)
        p = abi.Tracer.params(72, 60, spp=3, max_depth=5, rr_start=2, sky=(0.9, 0.95, 1.0), kernel=kernel,
                              aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT), stats=True,
                              bvh_width=width)
        gpu_tracer.trace(fr, p)
        out[name] = (gpu_tracer.readback(abi.AOV_RGBA32F), gpu_tracer.readback(abi.AOV_PRIMARY_HIT),
                     gpu_tracer.stats())
    for name, _, _ in runs[1:]:
        assert np.array_equal(fbits(out[name][0]), fbits(out["plain"][0])), name
        assert np.array_equal(out[name][1], out["plain"][1]), name
        for k in ("closest_rays", "shadow_rays", "hits"):
            assert out[name][2][k] == out["plain"][2][k], (name, k)


def test_wide_traversal_stack_check(gpu_tracer):
    sc = soup_scene(6, 4000, extent=12.0, sigma=0.5)
    gpu_tracer.upload_scene(sc)
    fr = S.frame(S.look_at((0.0, 3.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.4)
    p = abi.Tracer.params(16, 16, spp=1, max_depth=2, kernel=abi.KERNEL_WAVEFRONT, stack_depth=4, bvh_width=4)
    with pytest.raises(abi.TracerError) as e:
        gpu_tracer.trace(fr, p)
    assert e.value.status in (abi.ERR_STACK_OVERFLOW,)
    p.bvh_width = 3
    with pytest.raises(abi.TracerError):
        gpu_tracer.trace(fr, p)
    # an 8-wide traversal needs a triangle-only scene
    mixed = soup_scene(6, 400)
    mixed.spheres = sphere_scene(3).spheres
    gpu_tracer.upload_scene(mixed)
    p = abi.Tracer.params(16, 16, spp=1, max_depth=2, kernel=abi.KERNEL_WAVEFRONT, bvh_width=8)
    with pytest.raises(abi.TracerError) as e:
        gpu_tracer.trace(fr, p)
    assert e.value.status == abi.ERR_INVALID_ARG


def test_bvh_equals_linear_strict(gpu_tracer):
    """Strict ties make the result independent of traversal order: the BVH
    image equals the linear-scan image."""
    sc = soup_scene(3, 600)
    fr = S.frame(S.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.1)
    a = run_gpu(gpu_tracer, sc, fr, 64, 64, 2, 4, sky=(1, 1, 1), stats=False)
    lin = S.Scene(triangles=sc.triangles, materials=sc.materials, bvh=S.BVH_NONE)
    b = run_gpu(gpu_tracer, lin, fr, 64, 64, 2, 4, sky=(1, 1, 1), stats=False)
    assert np.array_equal(fbits(a["rgba32f"]), fbits(b["rgba32f"]))
    assert np.array_equal(a["hit_id"], b["hit_id"])


@pytest.mark.parametrize("wh", [(1, 1), (17, 5), (33, 65), (250, 3)])
def test_ragged_sizes(gpu_tracer, wh):
    w, h = wh
    sc = soup_scene(4, 500)
    fr = S.frame(S.look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), 40.0), w / h, 0.6)
    for k in KERNELS:
        g = run_gpu(gpu_tracer, sc, fr, w, h, 2, 3, sky=(1, 1, 1), kernel=k)
        o = run_oracle(sc, fr, w, h, 2, 3, sky=(1, 1, 1))
        compare(g, o)


def test_planes_only_and_mixed(gpu_tracer):
    """Planes are scanned linearly after the BVHs; spheres and triangles in one scene."""
    ref = S.reference_scene()
    sc = soup_scene(5, 300, extent=30.0, sigma=4.0)
    sc.spheres = ref.spheres
    sc.planes = ref.planes
    fr = S.reference_frame(0.2)
    tnodes, tidx, _ = abi.build_bvh(S.BVH_SAH, sc.triangles)
    snodes, sidx, _ = abi.build_bvh(S.BVH_SAH, sc.spheres)
    g = run_gpu(gpu_tracer, sc, fr, 96, 96, 2, 4, tri_bvh=(tnodes, tidx), sphere_bvh=(snodes, sidx))
    o = run_oracle(sc, fr, 96, 96, 2, 4, tri_bvh=(tnodes, tidx), sphere_bvh=(snodes, sidx))
    compare(g, o)
    only = S.Scene(planes=ref.planes)
    g = run_gpu(gpu_tracer, only, fr, 40, 40, 2, 3)
    o = run_oracle(only, fr, 40, 40, 2, 3)
    compare(g, o)


def test_empty_scene_sky_only(gpu_tracer):
    sc = S.Scene()
    fr = S.frame(S.look_at((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.5)
    g = run_gpu(gpu_tracer, sc, fr, 32, 32, 2, 3, sky=(0.5, 0.25, 1.0))
    o = run_oracle(sc, fr, 32, 32, 2, 3, sky=(0.5, 0.25, 1.0))
    compare(g, o)
    assert (g["hit_id"] == 0xFFFFFFFF).all()
