"""BVH builder properties and the oracle's BVH traversal (no GPU)."""
import numpy as np
import pytest

from conftest import fbits

from vktrace import abi, configs
from vktrace import scene as S


@pytest.mark.parametrize("kind,leaf", [(S.BVH_MEDIAN, 2), (S.BVH_SAH, 4), (S.BVH_SAH, 1)])
def test_bvh_valid_and_deterministic(tracer_lib, kind, leaf):
    tris, _ = S.triangle_soup(3, 5000, extent=20.0)
    n1, i1, d1 = abi.build_bvh(kind, tris, leaf_size=leaf, sah_bins=16)
    n2, i2, d2 = abi.build_bvh(kind, tris, leaf_size=leaf, sah_bins=16)
    assert n1.tobytes() == n2.tobytes() and np.array_equal(i1, i2) and d1 == d2
    assert abi.validate_bvh(tris, n1, i1) == d1
    assert (n1["count"] <= leaf).all()
    assert len(n1) <= 2 * len(tris) - 1
    assert sorted(i1.tolist()) == list(range(len(tris)))


def test_sphere_bvh_c0(tracer_lib):
    wl = configs.c0()
    nodes, idx, depth = abi.build_bvh(S.BVH_MEDIAN, wl.scene.spheres, leaf_size=2)
    assert abi.validate_bvh(wl.scene.spheres, nodes, idx) == depth
    assert len(nodes) == 63  # 64 spheres, leaf size 2 -> 32 leaves, 31 interior


def test_degenerate_inputs(tracer_lib):
    # all triangles identical: no SAH split exists, the median fallback must still build a valid tree
    t = np.zeros(37, S.TRIANGLE)
    t["v0"] = (0, 0, 0)
    t["v1"] = (1, 0, 0)
    t["v2"] = (0, 1, 0)
    nodes, idx, depth = abi.build_bvh(S.BVH_SAH, t, leaf_size=4)
    assert abi.validate_bvh(t, nodes, idx) == depth
    one = t[:1]
    nodes, idx, depth = abi.build_bvh(S.BVH_SAH, one)
    assert len(nodes) == 1 and nodes[0]["count"] == 1 and depth == 1


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_bvh_equals_linear_strict(oracle_lib, tracer_lib, seed):
    """With strict ties the closest hit does not depend on traversal order, so
    the oracle's BVH traversal must reproduce its linear scan exactly."""
    tris, mats = S.triangle_soup(100 + seed, 800, extent=8.0, sigma=0.8, n_materials=8)
    sph = S.random_spheres(200 + seed, 24, extent=8.0)
    sc = S.Scene(triangles=tris, materials=mats, spheres=sph, planes=S.reference_scene().planes[:1])
    tb = abi.build_bvh(S.BVH_SAH, tris)[:2]
    sb = abi.build_bvh(S.BVH_MEDIAN, sph, leaf_size=2)[:2]
    fr = S.frame(S.look_at((3.0, 4.0, 25.0), (0.0, 0.0, 0.0), 45.0), 1.0, 0.4)
    prm = oracle_lib.params(48, 40, spp=2, max_depth=5, rr_start=2, sky=(1.0, 0.9, 0.8), tie_mode=1)
    a = oracle_lib.render(sc, fr, prm)
    b = oracle_lib.render(sc, fr, prm, tri_bvh=tb, sphere_bvh=sb)
    assert np.array_equal(fbits(a["rgba32f"]), fbits(b["rgba32f"]))
    assert np.array_equal(a["hit_id"], b["hit_id"])
    assert a["stats"]["closest_rays"] == b["stats"]["closest_rays"]
    assert b["stats"]["node_fetches"] > 0 and b["stats"]["tri_tests"] < a["stats"]["tri_tests"]


def test_oracle_trace_ray_bvh_matches_linear(oracle_lib, tracer_lib):
    tris, mats = S.triangle_soup(5, 2000, extent=10.0)
    sc = S.Scene(triangles=tris, materials=mats)
    tb = abi.build_bvh(S.BVH_SAH, tris)[:2]
    g = S.SplitMix64(77)
    o = g.uniform(3 * 300, -15, 15).reshape(300, 3).astype(np.float32)
    d = g.uniform(3 * 300, -1, 1).reshape(300, 3)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    hits = 0
    for i in range(300):
        a = oracle_lib.trace_ray(sc, o[i], d[i], 3000.0, tie_mode=1)
        b = oracle_lib.trace_ray(sc, o[i], d[i], 3000.0, tie_mode=1, tri_bvh=tb)
        assert a["found"] == b["found"] and a["prim"] == b["prim"]
        if a["found"]:
            hits += 1
            assert a["t"] == b["t"]
        s = oracle_lib.trace_ray(sc, o[i], d[i], 3000.0, tie_mode=1, shadow=True, tri_bvh=tb)
        assert s["found"] == a["found"]
    assert hits > 20


def test_nan_ray_is_not_traversed(oracle_lib, tracer_lib):
    tris, mats = S.triangle_soup(6, 300, extent=10.0)
    sc = S.Scene(triangles=tris, materials=mats)
    tb = abi.build_bvh(S.BVH_SAH, tris)[:2]
    r = oracle_lib.trace_ray(sc, (0, 0, 20), (np.nan, np.nan, np.nan), 3000.0, tri_bvh=tb)
    assert not r["found"] and r["stats"]["node_fetches"] == 0 and r["stats"]["closest_rays"] == 1


@pytest.mark.parametrize("case", ["c1-soup", "c3-soup", "c0-spheres", "degenerate", "one", "median-tris", "leaf1"])
def test_oracle_builder_equals_product(oracle_lib, tracer_lib, case):
    """The oracle builds its BVHs with its own code (so the CPU baseline needs
    nothing from the product library); node for node, index for index, it
    must equal the product's builder."""
    kind, leaf, bins = S.BVH_SAH, 4, 16
    if case == "c1-soup":
        prims = configs.c1().scene.triangles
    elif case == "c3-soup":
        prims = configs.c3().scene.triangles
    elif case == "c0-spheres":
        prims, kind, leaf = configs.c0().scene.spheres, S.BVH_MEDIAN, 2
    elif case == "degenerate":
        prims = np.zeros(37, S.TRIANGLE)
        prims["v1"] = (1, 0, 0)
        prims["v2"] = (0, 1, 0)
    elif case == "one":
        prims = S.triangle_soup(5, 1)[0]
    elif case == "median-tris":
        prims, kind, leaf = S.triangle_soup(6, 3000, extent=20.0)[0], S.BVH_MEDIAN, 2
    else:
        prims, leaf, bins = S.triangle_soup(7, 2000, extent=5.0, sigma=2.0)[0], 1, 8
    pn, pi, pd = abi.build_bvh(kind, prims, leaf_size=leaf, sah_bins=bins)
    on, oi, od = oracle_lib.build_bvh(kind, prims, leaf_size=leaf, sah_bins=bins)
    assert len(on) == len(pn) and od == pd
    assert on.tobytes() == pn.tobytes()
    assert np.array_equal(oi, pi)
