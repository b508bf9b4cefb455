"""The steps around the dispatch, on the host: the oracle's present pass and
the product's camera controller against vectors recorded from the reference
(tests/golden/make_golden.py: Assets/Fullscreen.frag and Source/Camera.cpp
compiled for the host), and the progressive-accumulation restatement."""
import hashlib

import numpy as np
import pytest

import pyoracle
from conftest import golden

from vktrace import abi


def _sha(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = np.where(np.isnan(a), np.uint32(0x7FC00000), a.view(np.uint32))
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _regenerate_inputs():
    """The generator calls of make_golden.present_and_camera, in order."""
    g = np.random.default_rng(20240)
    out = []
    for sw, sh, w, h in golden("ref_present.npz")["cases"]:
        a8 = g.integers(0, 256, (sh, sw, 4), dtype=np.uint8)
        b8 = a8.copy()
        noisy = g.random((sh, sw)) < 0.5
        b8[noisy] = g.integers(0, 256, (int(noisy.sum()), 4), dtype=np.uint8)
        af = g.random((sh, sw, 4), dtype=np.float32)
        bf = af + np.where(g.random((sh, sw, 1)) < 0.5, np.float32(0.05), np.float32(0.0)).astype(np.float32)
        out.append((int(w), int(h), a8, b8, af, bf))
    return out


def test_present_oracle_matches_fullscreen_frag(oracle_lib):
    gp = golden("ref_present.npz")
    for k, (w, h, a8, b8, af, bf) in enumerate(_regenerate_inputs()):
        o8, _ = pyoracle.present(a8, b8, w, h)
        of, _ = pyoracle.present(af, bf, w, h)
        if f"c{k}_u8" in gp:
            assert np.array_equal(gp[f"c{k}_a8"], a8) and np.array_equal(gp[f"c{k}_bf"], bf)
            assert np.array_equal(o8.view(np.uint32), gp[f"c{k}_u8"].view(np.uint32)), k
            assert np.array_equal(of.view(np.uint32), gp[f"c{k}_f32"].view(np.uint32)), k
        else:
            assert _sha(o8) == str(gp[f"c{k}_u8_sha"]), k
            assert _sha(of) == str(gp[f"c{k}_f32_sha"]), k
            assert np.array_equal(o8[300:332, 500:532], gp[f"c{k}_u8_crop"])


def test_present_filter_behaviour(oracle_lib):
    """Identical frames: the centre tap (bilinear at the pixel's uv), so a
    constant image passes through; differing frames: the four-tap mean."""
    a = np.full((16, 16, 4), 200, np.uint8)
    out, out8 = pyoracle.present(a, a, 16, 16)
    inner = out[2:-2, 2:-2, :3]
    assert np.allclose(inner, 200 / 255, atol=1e-6) and (out8[2:-2, 2:-2, :3] == 200).all()
    # border: at twice the resolution the outermost pixels sample a quarter
    # of the clamp-to-border black
    up, _ = pyoracle.present(a, a, 32, 32)
    assert abs(up[0, 5, 0] - 0.75 * 200 / 255) < 1e-6 and abs(up[5, 5, 0] - 200 / 255) < 1e-6
    b = a.copy()
    b[..., :3] = 0
    blur, _ = pyoracle.present(a, b, 16, 16)
    # constant image: the four-tap mean equals the centre tap away from the border
    assert np.allclose(blur[3:-3, 3:-3, :3], 200 / 255, atol=1e-6)
    assert (out[..., 3] == 1.0).all()


def test_present_oracle_vflip(oracle_lib):
    """Row 0 of the traced image is its bottom: it appears at the bottom of
    the framebuffer."""
    a = np.zeros((8, 8, 4), np.uint8)
    a[0, :, 0] = 255  # bottom row red
    out, _ = pyoracle.present(a, a, 8, 8)
    assert out[-1, 4, 0] > 0.4 and out[0, 4, 0] == 0.0


def test_accumulate_restatement(oracle_lib):
    g = np.random.default_rng(3)
    lin = [g.random((5, 7, 4), dtype=np.float32) * 3 for _ in range(4)]
    s = np.zeros((5, 7, 4), np.float32)
    for n, l in enumerate(lin, 1):
        disp = pyoracle.accumulate(l, s, n)
    mean = (((lin[0][..., :3] + lin[1][..., :3]) + lin[2][..., :3]) + lin[3][..., :3]) / np.float32(4)
    ref = np.power(mean / (mean + 1), np.float32(1 / 2.2))
    assert np.allclose(disp[..., :3], ref, rtol=2e-6, atol=0)
    assert np.allclose(s[..., :3], ((lin[0] + lin[1]) + lin[2] + lin[3])[..., :3], rtol=1e-6)


def test_camera_controller_matches_camera_cpp(tracer_lib):
    gc = golden("ref_camera.npz")
    cam = abi.Camera(lib=tracer_lib)
    got = []
    for op, (a, b) in zip(gc["ops"], gc["args"]):
        if op == 7:
            cam = abi.Camera(startup=True, lib=tracer_lib)
        elif op == 6:
            cam.c.yaw = np.float32(np.float32(cam.c.yaw) - a)
            cam.c.pitch = np.float32(np.float32(cam.c.pitch) + b)
            cam.update()
        else:
            cam.move(int(op), float(a))
        got.append(cam.state())
    got = np.array(got)
    assert np.array_equal(got.view(np.uint32), gc["states"].view(np.uint32))


def _script(seed, n):
    g = np.random.default_rng(seed)
    x, y = 512.0, 384.0
    frames = []
    for i in range(n):
        d = {"dt": float(np.float32(g.uniform(0.004, 0.03))), "keys": int(g.integers(0, 64)),
             "toggle_light": bool(g.random() < 0.1)}
        if g.random() < 0.7:
            x += g.normal(0, 40)
            y += g.normal(0, 25)
            d["cursor"] = (x, y)
        frames.append(d)
    return frames


def test_camera_script_matches_oracle(tracer_lib, oracle_lib):
    """Scripted input (cursor, keys, light lock) through the product's
    controller and through the oracle's restatement of Main.cpp."""
    inputs = _script(5, 200)
    cam = abi.Camera(startup=True, lib=tracer_lib)
    frames = cam.script(inputs)
    o = pyoracle.CameraCtl()
    o.c.cam[0], o.c.cam[1], o.c.cam[2] = 32.8509, 30.6991, -106.389
    o.c.pitch, o.c.yaw = 4.44998, -602.79
    o.update()
    locked = False
    light = np.array([0.0, 64.0, 0.0], np.float32)
    for i, d in enumerate(inputs):
        if "cursor" in d:
            o.mouse(*d["cursor"])
        if d["toggle_light"]:
            locked = not locked
        o.keyboard(d["keys"], d["dt"])
        st = o.state()
        assert np.array_equal(np.frombuffer(frames[i]["camera"].tobytes(), np.float32).view(np.uint32),
                              st[:16].view(np.uint32)), i
        if locked:
            light = (st[:3] + np.array([0.0, -1.0, 0.0], np.float32)).astype(np.float32)
        assert np.array_equal(frames[i]["light_pos"], light), i
    # pitch stays clamped
    assert abs(float(cam.c.pitch)) <= 89.0


def test_camera_keys_exclusive(tracer_lib):
    """W wins over S, A over D, R over F (else-if chains, Main.cpp:27-50)."""
    a = abi.Camera(lib=tracer_lib)
    b = abi.Camera(lib=tracer_lib)
    a.keys(abi.KEY_W | abi.KEY_S | abi.KEY_A | abi.KEY_D | abi.KEY_R | abi.KEY_F, 0.01)
    b.keys(abi.KEY_W | abi.KEY_A | abi.KEY_R, 0.01)
    assert np.array_equal(a.state(), b.state())
    with pytest.raises(abi.TracerError):
        a.move(6, 1.0)
