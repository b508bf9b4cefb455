"""Scenes and comparisons shared by the GPU parity tests."""
from __future__ import annotations

import numpy as np

from conftest import fbits

import pyoracle
from vktrace import abi
from vktrace import scene as S

# Image parity bar: RMSE of the float image before 8-bit conversion.
IMAGE_RMSE_TOL = 1e-3
# Hit distances: the same IEEE operations in the same order, so equal; the
# stated bar is 1e-5 relative.
T_REL_TOL = 1e-5


def soup_scene(seed: int, n: int, extent: float = 10.0, sigma: float = 0.5, n_mat: int = 16, bvh=S.BVH_SAH):
    tris, mats = S.triangle_soup(seed, n, extent=extent, sigma=sigma, n_materials=n_mat)
    return S.Scene(triangles=tris, materials=mats, bvh=bvh)


def sphere_scene(seed: int, n: int = 64, bvh=S.BVH_MEDIAN):
    return S.Scene(spheres=S.random_spheres(seed, n), bvh=bvh)


def scene_bvhs(sc: S.Scene, tri_bvh=None, sphere_bvh=None):
    """The BVHs the library builds for sc (same host builder, deterministic)."""
    if sc.bvh != S.BVH_NONE:
        if tri_bvh is None and len(sc.triangles):
            tri_bvh = abi.build_bvh(sc.bvh, sc.triangles, sc.leaf_size, sc.sah_bins)[:2]
        if sphere_bvh is None and len(sc.spheres):
            sphere_bvh = abi.build_bvh(sc.bvh, sc.spheres, sc.leaf_size, sc.sah_bins)[:2]
    return tri_bvh, sphere_bvh


def run_gpu(tr: abi.Tracer, sc: S.Scene, fr, w, h, spp, depth, rr_start=0, sky=(0, 0, 0), tie=abi.TIES_STRICT,
            kernel=abi.KERNEL_PLAIN, block=0, tri_bvh=None, sphere_bvh=None, stats=True, tail_paths=0):
    tri_bvh, sphere_bvh = scene_bvhs(sc, tri_bvh, sphere_bvh)
    tr.upload_scene(sc, tri_bvh=tri_bvh, sphere_bvh=sphere_bvh)
    p = abi.Tracer.params(w, h, spp=spp, max_depth=depth, rr_start=rr_start, sky=sky, tie_mode=tie, kernel=kernel,
                          block=block, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F, abi.AOV_PRIMARY_HIT), stats=stats,
                          tail_paths=tail_paths)
    tr.trace(fr, p)
    out = {"rgba32f": tr.readback(abi.AOV_RGBA32F), "rgba8": tr.readback(abi.AOV_RGBA8)}
    hit = tr.readback(abi.AOV_PRIMARY_HIT)
    out["hit_id"] = hit[..., 0].copy()
    out["hit_t"] = hit[..., 1].copy().view(np.float32)
    if stats:
        out["stats"] = tr.stats()
        out["kernel"] = kernel
    return out


def run_oracle(sc: S.Scene, fr, w, h, spp, depth, rr_start=0, sky=(0, 0, 0), tie=1, tri_bvh=None, sphere_bvh=None):
    tri_bvh, sphere_bvh = scene_bvhs(sc, tri_bvh, sphere_bvh)
    return pyoracle.render(sc, fr, pyoracle.params(w, h, spp=spp, max_depth=depth, rr_start=rr_start, sky=sky,
                                                   tie_mode=tie, trig_mode=0), tri_bvh=tri_bvh, sphere_bvh=sphere_bvh)


def rmse(a, b, skip_col0=True):
    a = a[..., :3].astype(np.float64)
    b = b[..., :3].astype(np.float64)
    if skip_col0:  # column 0 is NaN by construction (uv.x = 0), reported separately
        a, b = a[:, 1:], b[:, 1:]
    if a.size == 0:
        return 0.0
    return float(np.sqrt(np.mean((a - b) ** 2)))


def compare(gpu, ora, check_stats=True):
    """Asserts the parity bar; returns a summary dict."""
    gid, oid = gpu["hit_id"], ora["hit_id"]
    gt, ot = gpu["hit_t"], ora["hit_t"]
    mism = gid != oid
    if mism.any():
        # the only allowed id mismatches are ties: both hits within 1e-6 in t
        assert np.all(np.abs(gt[mism] - ot[mism]) <= 1e-6), f"{int(mism.sum())} primary-hit id mismatches"
    both = (gid == oid) & (gid != 0xFFFFFFFF)
    rel = np.abs(gt[both] - ot[both]) / np.maximum(np.abs(ot[both]), 1e-30)
    assert rel.size == 0 or rel.max() <= T_REL_TOL
    e = rmse(gpu["rgba32f"], ora["rgba32f"])
    assert e <= IMAGE_RMSE_TOL, f"image RMSE {e}"
    # column 0: NaN exactly where the oracle has NaN
    assert np.array_equal(np.isnan(gpu["rgba32f"][:, 0]), np.isnan(ora["rgba32f"][:, 0]))
    exact = float(np.mean(np.all(fbits(gpu["rgba32f"]) == fbits(ora["rgba32f"]), axis=-1)))
    if check_stats and "stats" in gpu:
        if gpu["kernel"] == abi.KERNEL_PLAIN:
            # the plain kernel visits nodes in the oracle's order: every counter equal
            assert gpu["stats"] == ora["stats"], (gpu["stats"], ora["stats"])
        else:
            # the wavefront traversal order depends on the warp; rays, hits
            # and the (unordered) plane scans must still agree
            for k in ("closest_rays", "shadow_rays", "hits", "plane_tests"):
                assert gpu["stats"][k] == ora["stats"][k], (k, gpu["stats"], ora["stats"])
    return {"rmse": e, "bit_exact_pixels": exact, "id_mismatch": int(mism.sum())}
