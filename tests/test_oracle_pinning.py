"""Pins the oracle to the reference: its outputs must equal, bit for bit, the
golden vectors recorded from the reference shader compiled for the host
(tests/golden/make_golden.py).  In portable-trig mode this holds on any IEEE
host; libm mode is checked only on the host whose C library made the goldens
(cos in libm is not bit-identical across C libraries / CPUs)."""
import hashlib

import numpy as np
import pytest

from conftest import fbits, golden

from vktrace import scene as S


def _libm_matches(pyoracle):
    """True when this host's libm cos gives the rand() stream the goldens were made with."""
    kr = golden("kat_rand.npz")
    c = kr["cases"][3]
    return np.array_equal(pyoracle.rand(c[0], c[1], c[2], 64, trig_mode=1).view(np.uint32),
                          kr["libm"][3].view(np.uint32))


def _bits_equal(a, b):
    """Bitwise equality of float32 arrays; any two NaNs count as equal (the
    NaN payload an operation returns depends on the operand order a compiler
    picks for a commutative +/*, and carries no meaning)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    nan = np.isnan(a) & np.isnan(b)
    return np.array_equal(np.where(nan, 0, a.view(np.uint32)), np.where(nan, 0, b.view(np.uint32)))


def test_reference_scene_table_matches_shader_constants():
    g = golden("ref_scene.npz")
    sc = S.reference_scene()
    assert _bits_equal(np.frombuffer(sc.spheres.tobytes(), np.float32).reshape(-1, 16), g["spheres"])
    assert _bits_equal(np.frombuffer(sc.planes.tobytes(), np.float32).reshape(-1, 16), g["planes"])
    assert _bits_equal(np.frombuffer(sc.materials.tobytes(), np.float32), g["tri_material"])
    assert int(g["depth"]) == 4 and int(g["samples"]) == 4


def test_reference_camera_matches_camera_cpp():
    g = golden("ref_scene.npz")
    assert _bits_equal(np.frombuffer(S.reference_camera().tobytes(), np.float32), g["camera"])


@pytest.mark.parametrize("trig", [0, 1])
def test_rand_kat(oracle_lib, trig):
    if trig == 1 and not _libm_matches(oracle_lib):
        pytest.skip("this host's libm cos differs from the one the goldens were made with")
    kr = golden("kat_rand.npz")
    ref = kr["rng" if trig == 0 else "libm"]
    for i, c in enumerate(kr["cases"]):
        got = oracle_lib.rand(c[0], c[1], c[2], 64, trig_mode=trig)
        assert _bits_equal(got, ref[i]), f"case {i} {c}"


def test_rand_column_zero_is_nan(oracle_lib):
    # uv.x = 0 makes rand_salt = uv.y / 0 = +inf (NaN at the origin pixel),
    # Tracer.comp:565, so every rand() of pixel column 0 is NaN.
    with np.errstate(divide="ignore", invalid="ignore"):
        for cy in (0.0, 0.3):
            salt = np.float32(cy) / np.float32(0.0) + np.float32(0.5)
            assert np.isnan(oracle_lib.rand(0.0, cy, salt, 4)).all()


def test_intersection_kats(oracle_lib):
    k = golden("kat_intersect.npz")
    L = oracle_lib.lib()
    P = oracle_lib._p
    n = len(k["o"])
    ti = np.array([L.oracle_tri_intersect(P(k["o"][i]), P(k["d"][i]), P(k["tri48"][i])) for i in range(n)], np.float32)
    si = np.array([L.oracle_sphere_intersect(P(k["o"][i]), P(k["d"][i]), P(k["centers"][i]), k["radii"][i])
                   for i in range(n)], np.float32)
    pi = np.array([L.oracle_plane_intersect(P(k["o"][i]), P(k["d_plane"][i]), P(k["normals"][i]), k["lens"][i])
                   for i in range(n)], np.float32)
    assert _bits_equal(ti, k["tri_t"])
    assert _bits_equal(si, k["sphere_t"])
    assert _bits_equal(pi, k["plane_t"])
    assert (k["tri_t"] > 0).sum() > 20  # the KAT set exercises hits as well as misses


def test_trace_ray_kat(oracle_lib):
    k = golden("kat_trace.npz")
    sc = S.reference_scene()
    sc.triangles = k["triangles"]
    for i in range(len(k["o"])):
        r = oracle_lib.trace_ray(sc, k["o"][i], k["d"][i], float(k["tmax"][i]), tie_mode=0)
        ref = k["out"][i]
        assert r["found"] == bool(ref[0])
        if r["found"]:
            assert _bits_equal(np.array([r["t"]], np.float32), ref[1:2])
            assert _bits_equal(r["P"], ref[2:5]) and _bits_equal(r["N"], ref[5:8])
            assert _bits_equal(r["material"][:9], ref[8:17])


@pytest.mark.parametrize("trig", [0, 1])
def test_reference_render_64(oracle_lib, trig):
    if trig == 1 and not _libm_matches(oracle_lib):
        pytest.skip("this host's libm cos differs from the one the goldens were made with")
    g = golden("ref_render.npz")
    tag = "rng" if trig == 0 else "libm"
    out = oracle_lib.render(S.reference_scene(), S.reference_frame(0.5),
                            oracle_lib.params(64, 64, spp=4, max_depth=4, rr_start=0, tie_mode=0, trig_mode=trig))
    assert _bits_equal(out["rgba32f"], g[f"{tag}_64_rgba32f"])
    assert np.array_equal(out["rgba8"], g[f"{tag}_64_rgba8"])


def test_reference_render_full_size(oracle_lib):
    """The Ref configuration itself: 1024x1024, 4 spp, depth 4, portable trig."""
    g = golden("ref_render.npz")
    out = oracle_lib.render(S.reference_scene(), S.reference_frame(0.5),
                            oracle_lib.params(1024, 1024, spp=4, max_depth=4, rr_start=0, tie_mode=0, trig_mode=0))
    img = out["rgba32f"]
    for (y, x), crop in zip(g["crops_yx"], g["rng_1024_crops"]):
        assert _bits_equal(img[y:y + 32, x:x + 32], crop)
    assert hashlib.sha256(fbits(img).tobytes()).hexdigest() == str(g["rng_1024_sha_rgba32f"])
    assert hashlib.sha256(out["rgba8"].tobytes()).hexdigest() == str(g["rng_1024_sha_rgba8"])


@pytest.mark.parametrize("trig", [0, 1])
def test_random_triangle_ssbo(oracle_lib, trig):
    if trig == 1 and not _libm_matches(oracle_lib):
        pytest.skip("this host's libm cos differs from the one the goldens were made with")
    g = golden("ref_tris.npz")
    sc = S.reference_scene()
    sc.triangles = g["triangles"]
    out = oracle_lib.render(sc, g["frame"], oracle_lib.params(48, 48, spp=4, max_depth=4, tie_mode=0,
                                                              trig_mode=trig))
    assert _bits_equal(out["rgba32f"], g[("rng" if trig == 0 else "libm") + "_rgba32f"])


def test_live_harness_if_present(oracle_lib):
    """When the reference tree is mounted, compare against the compiled shader
    live on a fresh random scene and camera (not only the committed vectors)."""
    if not oracle_lib.reference_present():
        pytest.skip("reference tree not mounted")
    oracle_lib.build_ref()
    h = oracle_lib.RefHarness(rng_trig=True)
    g = S.SplitMix64(99)
    n = 16
    t = np.zeros(n, S.TRIANGLE)
    c = g.uniform(3 * n, -30, 30).reshape(n, 1, 3) + np.array([0, 30, 0])
    v = (c + g.uniform(9 * n, -15, 15).reshape(n, 3, 3)).astype(np.float32)
    t["v0"], t["v1"], t["v2"] = v[:, 0], v[:, 1], v[:, 2]
    sc = S.reference_scene()
    sc.triangles = t
    fr = S.frame(S.look_at((20.0, 60.0, -100.0), (-10.0, 30.0, 0.0), 50.0), 1.3, 0.7)
    ref_img, ref_u8 = h.render(fr, t, 40, 30)
    out = oracle_lib.render(sc, fr, oracle_lib.params(40, 30, spp=4, max_depth=4, tie_mode=0, trig_mode=0))
    assert _bits_equal(out["rgba32f"], ref_img)
    assert np.array_equal(out["rgba8"], ref_u8)
