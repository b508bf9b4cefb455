"""Generates the golden vectors in tests/golden/ from the reference itself.

The reference ships no tests or fixtures.  Its hot path is a GLSL compute
shader (Assets/Tracer.comp); oracle/ref/Makefile compiles that shader source,
as it stands in the reference tree, into a host library against the
reference's vendored glm, and Source/Camera.cpp likewise.  This script calls
those libraries and records their outputs:

  ref_scene.npz      the shader's constant spheres/planes/triangle material,
                     DEPTH/SAMPLES, and the start-up camera from Camera.cpp
  ref_render.npz     Ref-scene renders (64x64 and crops of 1024x1024, plus
                     SHA-256 of the full 1024x1024 images), libm and portable
                     trig
  ref_tris.npz       a 48x48 render with 40 random triangles in the SSBO
  kat_rand.npz       rand() sequences, including the uv.x = 0 column
  kat_intersect.npz  calc_tri/sphere/plane_intersect on random rays
  kat_trace.npz      trace_ray on random rays through the Ref scene + triangles

  ref_present.npz    the present pass (Assets/Fullscreen.frag) on random image
                     pairs, RGBA8 and float
  ref_camera.npz     Camera.cpp operations from the default camera
  ref_whitted.npz    the legacy Assets/Raytracer.comp on two frames

Run here (needs the reference tree):  python tests/golden/make_golden.py
(--present: only the last three)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "vk-renderer_gb300"))

import pyoracle  # noqa: E402
from vktrace import scene as S  # noqa: E402

CROPS = [(0, 0), (0, 480), (500, 500), (992, 992), (300, 10)]  # (y, x) of 32x32 crops at 1024^2


def sha(a: np.ndarray) -> str:
    """SHA-256 of the array's bytes; float32 NaNs are first mapped to one
    canonical NaN (their payload depends on compiler operand order)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = np.where(np.isnan(a), np.uint32(0x7FC00000), a.view(np.uint32))
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def random_tris(seed: int, n: int) -> np.ndarray:
    g = S.SplitMix64(seed)
    c = g.uniform(3 * n, -40.0, 40.0).reshape(n, 1, 3) + np.array([0.0, 40.0, 0.0])
    off = g.uniform(9 * n, -12.0, 12.0).reshape(n, 3, 3)
    v = (c + off).astype(np.float32)
    t = np.zeros(n, S.TRIANGLE)
    t["v0"], t["v1"], t["v2"] = v[:, 0], v[:, 1], v[:, 2]
    return t


def present_and_camera():
    """ref_present.npz: Fullscreen.frag compiled for the host over random
    image pairs (RGBA8 and float, equal and differing regions, the Ref sizes
    1024^2 -> 1024x768 and ragged ones).  ref_camera.npz: Camera.cpp
    operations from the default camera (moves, pitch/yaw changes past the
    +-89 clamp, the start-up camera)."""
    g = np.random.default_rng(20240)
    pres = {}
    cases = [(64, 64, 48, 40), (37, 23, 50, 71), (1, 1, 3, 2), (1024, 1024, 1024, 768)]
    for k, (sw, sh, w, h) in enumerate(cases):
        a8 = g.integers(0, 256, (sh, sw, 4), dtype=np.uint8)
        b8 = a8.copy()
        noisy = g.random((sh, sw)) < 0.5  # half the texels differ from the previous frame
        b8[noisy] = g.integers(0, 256, (int(noisy.sum()), 4), dtype=np.uint8)
        af = g.random((sh, sw, 4), dtype=np.float32)
        bf = af + np.where(g.random((sh, sw, 1)) < 0.5, np.float32(0.05), np.float32(0.0)).astype(np.float32)
        out8 = pyoracle.ref_present(a8, b8, w, h)
        outf = pyoracle.ref_present(af, bf, w, h)
        if sw * sh > 4096:  # large case: seeds regenerate the inputs; store hashes and crops
            pres[f"c{k}_seed_note"] = np.array("inputs regenerated by the test from the same generator")
            pres[f"c{k}_u8_sha"] = np.array(sha(out8))
            pres[f"c{k}_f32_sha"] = np.array(sha(outf))
            pres[f"c{k}_u8_crop"] = out8[300:332, 500:532]
            pres[f"c{k}_f32_crop"] = outf[300:332, 500:532]
        else:
            pres[f"c{k}_a8"], pres[f"c{k}_b8"], pres[f"c{k}_af"], pres[f"c{k}_bf"] = a8, b8, af, bf
            pres[f"c{k}_u8"], pres[f"c{k}_f32"] = out8, outf
    pres["cases"] = np.array(cases, np.int32)
    pres["rng_seed"] = np.int64(20240)
    np.savez_compressed(os.path.join(HERE, "ref_present.npz"), **pres)

    ops = [0, 2, 6, 6, 4, 1, 3, 5, 6, 6, 7, 0, 6, 2]
    args = [3.5, 0, 2.25, 0, 10.5, -3.25, 0.0, 200.0, 1.5, 0, 0.75, 0, 5.0, 0, 2.0, 0, -7.0, -150.0,
            33.3, 71.2, 0, 0, 1.1, 0, 4.2, -1.7, 0.6, 0]
    states = pyoracle.ref_camera_ops(ops, args)
    np.savez(os.path.join(HERE, "ref_camera.npz"), ops=np.array(ops, np.int32),
             args=np.array(args, np.float32).reshape(-1, 2), states=states)

    # the legacy Whitted shader (Assets/Raytracer.comp): the start-up frame and
    # a second camera/light, small sizes in full, 1024^2 as hashes
    fr2 = S.frame(S.look_at((0.0, 40.0, -60.0), (0.0, 20.0, 30.0), 60.0), 4 / 3, 0.2, (10.0, 60.0, 10.0))
    frames = [S.reference_frame(0.5), fr2]
    # frames as raw 96-byte records (24 floats): a stacked structured array
    # would lose its field offsets in the .npz
    wh = {"frames": np.stack([np.frombuffer(f.tobytes(), np.float32) for f in frames])}
    for k, fr in enumerate(frames):
        for w, h in ((64, 48), (97, 61)):
            img, u8 = pyoracle.ref_whitted(fr, w, h)
            wh[f"f{k}_{w}x{h}_rgba32f"], wh[f"f{k}_{w}x{h}_rgba8"] = img, u8
        img, u8 = pyoracle.ref_whitted(fr, 1024, 1024)
        wh[f"f{k}_1024_sha_rgba32f"], wh[f"f{k}_1024_sha_rgba8"] = np.array(sha(img)), np.array(sha(u8))
    np.savez_compressed(os.path.join(HERE, "ref_whitted.npz"), **wh)


def main():
    if not pyoracle.build_ref():
        raise SystemExit("reference tree not found")
    if "--present" in sys.argv:
        present_and_camera()
        print("present and camera vectors written to", HERE)
        return
    present_and_camera()
    out = {}
    H = {False: pyoracle.RefHarness(False), True: pyoracle.RefHarness(True)}
    sph, pl, tm, (depth, samples) = H[False].scene_constants()
    cam = pyoracle.ref_camera(S.REF_CAMERA_POS, S.REF_CAMERA_PITCH, S.REF_CAMERA_YAW)
    np.savez(os.path.join(HERE, "ref_scene.npz"), spheres=sph, planes=pl, tri_material=tm,
             depth=np.int32(depth), samples=np.int32(samples), camera=cam)

    ref = S.reference_scene()
    fr = S.reference_frame(seed=0.5)
    assert (np.frombuffer(fr["camera"].tobytes(), np.float32) == cam).all()
    rend = {}
    for rng in (False, True):
        tag = "rng" if rng else "libm"
        img, u8 = H[rng].render(fr, ref.triangles, 64, 64)
        rend[f"{tag}_64_rgba32f"] = img
        rend[f"{tag}_64_rgba8"] = u8
        img, u8 = H[rng].render(fr, ref.triangles, 1024, 1024)
        rend[f"{tag}_1024_sha_rgba32f"] = np.array(sha(img))
        rend[f"{tag}_1024_sha_rgba8"] = np.array(sha(u8))
        rend[f"{tag}_1024_crops"] = np.stack([img[y:y + 32, x:x + 32] for y, x in CROPS])
    rend["crops_yx"] = np.array(CROPS, np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_render.npz"), **rend)

    tris = random_tris(11, 40)
    cam2 = S.look_at((0.0, 50.0, -120.0), (0.0, 40.0, 0.0), None if False else 40.0)
    fr2 = S.frame(cam2, 1.0, 0.25)
    tr = {"triangles": tris, "frame": fr2}
    for rng in (False, True):
        tag = "rng" if rng else "libm"
        img, u8 = H[rng].render(fr2, tris, 48, 48)
        tr[f"{tag}_rgba32f"] = img
    np.savez_compressed(os.path.join(HERE, "ref_tris.npz"), **tr)

    g = S.SplitMix64(5)
    cases = [(0.0, 0.0, 0.0), (0.0, 0.5, 0.5), (1.0 / 512, 511.0 / 512, 0.0), (0.5, 0.5, 0.37),
             (1.0 / 1920, 1079.0 / 1080, 0.9), (0.25, 0.75, 2000.0)]
    cases += [tuple(x) for x in np.c_[g.uniform(20), g.uniform(20), g.uniform(20, 0.0, 600.0)]]
    cases = np.array(cases, np.float32)
    kr = {"cases": cases}
    for rng in (False, True):
        kr["rng" if rng else "libm"] = np.stack([H[rng].rand(c[0], c[1], c[2], 64) for c in cases])
    np.savez(os.path.join(HERE, "kat_rand.npz"), **kr)

    n = 256
    o = g.uniform(3 * n, -30.0, 30.0).reshape(n, 3).astype(np.float32)
    d = g.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tri48 = np.zeros((n, 12), np.float32)
    tri48[:, 0:3] = g.uniform(3 * n, -10.0, 10.0).reshape(n, 3)
    tri48[:, 4:7] = g.uniform(3 * n, -10.0, 10.0).reshape(n, 3)
    tri48[:, 8:11] = g.uniform(3 * n, -10.0, 10.0).reshape(n, 3)
    # aim half of the rays at their triangle's centroid so hits occur
    cen = (tri48[:, 0:3] + tri48[:, 4:7] + tri48[:, 8:11]) / 3
    aim = cen - o
    aim = (aim / np.linalg.norm(aim, axis=1, keepdims=True)).astype(np.float32)
    d[::2] = aim[::2]
    cs = g.uniform(3 * n, -10.0, 10.0).reshape(n, 3).astype(np.float32)
    rs = g.uniform(n, 0.5, 8.0).astype(np.float32)
    pn = g.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    pn = (pn / np.linalg.norm(pn, axis=1, keepdims=True)).astype(np.float32)
    pn[5] = (0, 1, 0)
    pl_len = g.uniform(n, -20.0, 20.0).astype(np.float32)
    L = H[False].L
    P = pyoracle._p
    ti = np.array([L.ref_tri_intersect(P(o[i]), P(d[i]), P(tri48[i])) for i in range(n)], np.float32)
    si = np.array([L.ref_sphere_intersect(P(o[i]), P(d[i]), P(cs[i]), rs[i]) for i in range(n)], np.float32)
    d_par = d.copy()
    d_par[5] = (1, 0, 0)  # parallel to the plane y = const: when_neq guard
    pi = np.array([L.ref_plane_intersect(P(o[i]), P(d_par[i]), P(pn[i]), pl_len[i]) for i in range(n)], np.float32)
    np.savez(os.path.join(HERE, "kat_intersect.npz"), o=o, d=d, d_plane=d_par, tri48=tri48, tri_t=ti, centers=cs,
             radii=rs, sphere_t=si, normals=pn, lens=pl_len, plane_t=pi)

    m = 200
    allt = np.concatenate([ref.triangles, random_tris(12, 24)])
    allt["material"] = 0
    o2 = np.c_[g.uniform(m, -60, 60), g.uniform(m, 2, 120), g.uniform(m, -60, 60)].astype(np.float32)
    d2 = g.uniform(3 * m, -1.0, 1.0).reshape(m, 3)
    d2 = (d2 / np.linalg.norm(d2, axis=1, keepdims=True)).astype(np.float32)
    tmax = np.array([3000.0, 750.0, 333.33334, 187.5] * (m // 4), np.float32)
    res = np.stack([H[False].trace_ray(allt, o2[i], d2[i], tmax[i]) for i in range(m)])
    np.savez(os.path.join(HERE, "kat_trace.npz"), triangles=allt, o=o2, d=d2, tmax=tmax, out=res)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
