"""GPU parity at the benchmarked workloads' own sizes (through the C ABI).

The other GPU parity tests use reduced sizes; these run the workloads as the
benchmark runs them and hold them to the same bar against the oracle:
  c0  512^2, 1 spp, depth 2, 64 spheres, median BVH (every pixel)
  c1  1920x1080, 16 spp, depth 8, 100k triangles, SAH (every 16th scanline)
  c2  all 64 scenes of the batch, one CUDA-graph wavefront (every 32nd
      scanline of every scene), and every scene equal to its plain trace
  c3  the adjoint at 256^2, 4 spp, depth 4, 10k triangles, 64 materials:
      its largest albedo gradients against central differences of the FP64
      host evaluation
"""
import numpy as np
import pytest

import pyoracle
from conftest import fbits
from gpu_cases import IMAGE_RMSE_TOL, compare
from vktrace import abi, configs
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def _gpu_frame(tr, wl, kernel, aovs=(abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT), stats=True, tri_bvh=None,
               sphere_bvh=None):
    tr.upload_scene(wl.scene, tri_bvh=tri_bvh, sphere_bvh=sphere_bvh)
    p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start, sky=wl.sky,
                          tie_mode=wl.tie_mode, kernel=kernel, aovs=aovs, stats=stats)
    tr.trace(wl.frame, p)
    hit = tr.readback(abi.AOV_PRIMARY_HIT)
    out = {"rgba32f": tr.readback(abi.AOV_RGBA32F), "hit_id": hit[..., 0].copy(),
           "hit_t": hit[..., 1].copy().view(np.float32), "kernel": kernel}
    if stats:
        out["stats"] = tr.stats()
    return out


def _rows(d, rows):
    return {k: (v[rows] if isinstance(v, np.ndarray) else v) for k, v in d.items()}


@pytest.mark.parametrize("kernel", [abi.KERNEL_PLAIN, abi.KERNEL_WAVEFRONT])
@pytest.mark.parametrize("sky", [None, (1.0, 1.0, 1.0)])
def test_c0_full_size(gpu_tracer, kernel, sky):
    """c0 as specified (sky 0: black plus dither, hits carry the check), and
    the same frame with sky 1 so that the image carries it too."""
    wl = configs.c0()
    if sky is not None:
        wl.sky = sky
    sb = pyoracle.build_bvh(1, wl.scene.spheres, leaf_size=2)[:2]
    g = _gpu_frame(gpu_tracer, wl, kernel, sphere_bvh=sb)
    o = pyoracle.render(wl.scene, wl.frame, pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth,
                                                            rr_start=wl.rr_start, sky=wl.sky), sphere_bvh=sb)
    r = compare(g, o)
    assert r["id_mismatch"] == 0
    assert (g["hit_id"] != 0xFFFFFFFF).mean() > 0.05


def test_c1_full_frame(gpu_tracer):
    """The benchmarked frame itself (wavefront, automatic launch shape) on
    every 16th scanline of the oracle."""
    wl = configs.c1()
    tb = pyoracle.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)[:2]
    g = _gpu_frame(gpu_tracer, wl, abi.KERNEL_WAVEFRONT, stats=False, tri_bvh=tb)
    rows = slice(3, wl.height, 16)
    o = pyoracle.render(wl.scene, wl.frame, pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth,
                                                            rr_start=wl.rr_start, sky=wl.sky,
                                                            rows=(rows.start, wl.height, rows.step)), tri_bvh=tb)
    r = compare(_rows(g, rows), _rows(o, rows), check_stats=False)
    assert r["id_mismatch"] == 0, r


def test_c2_all_scenes(gpu_tracer):
    """All 64 scenes of the batch in one CUDA-graph wavefront: every scene
    bit-identical to its per-scene plain trace and, on every 32nd scanline, to
    the oracle."""
    tr = gpu_tracer
    wls = configs.c2()
    tr.upload_scenes([w.scene for w in wls])
    frames = [w.frame for w in wls]

    def prm(kernel):
        return [abi.Tracer.params(w.width, w.height, spp=w.spp, max_depth=w.max_depth, rr_start=w.rr_start,
                                  sky=w.sky, kernel=kernel, aovs=(abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT))
                for w in wls]

    tr.trace_batched(frames, prm(abi.KERNEL_PLAIN), use_graph=False)
    plain = [tr.readback_scene(k, abi.AOV_RGBA32F) for k in range(len(wls))]
    tr.trace_batched(frames, prm(abi.KERNEL_WAVEFRONT), use_graph=True)
    worst = 0.0
    for k, w in enumerate(wls):
        img = tr.readback_scene(k, abi.AOV_RGBA32F)
        hit = tr.readback_scene(k, abi.AOV_PRIMARY_HIT)
        assert np.array_equal(fbits(img), fbits(plain[k])), k
        tb = pyoracle.build_bvh(2, w.scene.triangles, leaf_size=4, sah_bins=16)[:2]
        start = k % 32
        rows = slice(start, w.height, 32)
        o = pyoracle.render(w.scene, w.frame, pyoracle.params(w.width, w.height, spp=w.spp, max_depth=w.max_depth,
                                                              rr_start=w.rr_start, sky=w.sky,
                                                              rows=(start, w.height, 32)), tri_bvh=tb)
        g = {"rgba32f": img, "hit_id": hit[..., 0].copy(), "hit_t": hit[..., 1].copy().view(np.float32)}
        r = compare(_rows(g, rows), _rows(o, rows), check_stats=False)
        assert r["id_mismatch"] == 0, (k, r)
        worst = max(worst, r["rmse"])
    assert worst <= IMAGE_RMSE_TOL


def test_c3_adjoint_vs_fp64_host(gpu_tracer):
    """c3 as specified: target rendered with albedos + N(0, 0.1^2) (clamped),
    L2 image loss; the 8 largest albedo gradient components against central
    differences (step 2^-12, measured in float) of the FP64 host evaluation.
    Bar: relative error <= 1e-3."""
    from bench import _perturbed_albedo
    tr = gpu_tracer
    wl = configs.c3()
    tb = pyoracle.build_bvh(2, wl.scene.triangles, leaf_size=4, sah_bins=16)[:2]
    tr.upload_scene(wl.scene, tri_bvh=tb)
    base = wl.scene.materials.copy()
    p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start,
                          sky=wl.sky, aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR))
    tr.set_materials(_perturbed_albedo(base, 3))
    tr.trace(wl.frame, p)
    target = tr.readback(abi.AOV_RGBA32F)
    tr.set_materials(base)
    tr.trace(wl.frame, p)
    img, lin = tr.readback(abi.AOV_RGBA32F), tr.readback(abi.AOV_LINEAR)
    d = img[:, 1:, :3].astype(np.float64) - target[:, 1:, :3]
    dl = np.zeros(img.shape, np.float32)
    dl[:, 1:, :3] = 2 * d
    ga, ge, gc = tr.trace_adjoint(wl.frame, p, dl, lin, num_materials=len(base))
    prm = pyoracle.params(wl.width, wl.height, spp=wl.spp, max_depth=wl.max_depth, rr_start=wl.rr_start, sky=wl.sky)
    tgt = target[:, 1:, :3].astype(np.float64)

    def L64(mats):
        sc = S.Scene(triangles=wl.scene.triangles, materials=mats, bvh=wl.scene.bvh)
        out = pyoracle.render_f64(sc, wl.frame, prm, tri_bvh=tb)
        e = out["image"][:, 1:, :3] - tgt
        return float(np.sum(e * e))

    h = 2.0 ** -12
    rel = []
    for flat in np.argsort(-np.abs(ga).ravel())[:8]:
        m, c = divmod(int(flat), 3)
        mp, mm = base.copy(), base.copy()
        mp["albedo"][m, c] += h
        mm["albedo"][m, c] -= h
        fd = (L64(mp) - L64(mm)) / float(np.float32(mp["albedo"][m, c]) - np.float32(mm["albedo"][m, c]))
        rel.append(abs(float(ga[m, c]) - fd) / abs(fd))
    assert max(rel) <= 1e-3, rel
