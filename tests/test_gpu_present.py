"""GPU present pass and draw loop against the oracle, through the C ABI.

The present kernel restates Assets/Fullscreen.frag with the sampler of
Source/GraphicsDevice.cpp:770-790: its output must equal the oracle's bit for
bit.  tracer_draw in ping-pong mode must equal the oracle's present pass over
the frames the GPU traced (slot k % 2, read as bound); in accumulation mode
the running mean must equal the oracle's (the tonemap's powf may differ from
the host C library in the last ulp: tolerance 2e-7 absolute on the float
output, one 8-bit step on RGBA8)."""
import numpy as np
import pytest

import pyoracle
from gpu_cases import soup_scene
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def _pair(g, sw, sh, dtype):
    if dtype == np.uint8:
        a = g.integers(0, 256, (sh, sw, 4), dtype=np.uint8)
        b = a.copy()
        m = g.random((sh, sw)) < 0.5
        b[m] = g.integers(0, 256, (int(m.sum()), 4), dtype=np.uint8)
    else:
        a = g.random((sh, sw, 4), dtype=np.float32)
        b = (a + np.where(g.random((sh, sw, 1)) < 0.5, 0.05, 0.0)).astype(np.float32)
    return a, b


@pytest.mark.parametrize("dtype", [np.uint8, np.float32])
@pytest.mark.parametrize("case", [(64, 64, 48, 40), (37, 23, 50, 71), (1, 1, 3, 2), (1024, 1024, 1024, 768),
                                  (1920, 1080, 1920, 1080)])
def test_present_bit_exact(gpu_tracer, dtype, case):
    sw, sh, w, h = case
    g = np.random.default_rng(sw * 7 + h)
    a, b = _pair(g, sw, sh, dtype)
    o32, o8 = pyoracle.present(a, b, w, h)
    got8 = gpu_tracer.present(a, b, w, h, abi.AOV_RGBA8)
    got32 = gpu_tracer.present(a, b, w, h, abi.AOV_RGBA32F)
    assert np.array_equal(got32.view(np.uint32), o32.view(np.uint32))
    assert np.array_equal(got8, o8)


def test_present_device_buffers(gpu_tracer):
    torch = pytest.importorskip("torch")
    g = np.random.default_rng(4)
    a, b = _pair(g, 300, 200, np.uint8)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros((150, 400, 4), dtype=torch.float32, device="cuda")
    gpu_tracer.present((da.data_ptr(), 300, 200, abi.AOV_RGBA8), (db.data_ptr(),), 400, 150, abi.AOV_RGBA32F,
                       out=out.data_ptr())
    gpu_tracer.synchronize()
    torch.cuda.synchronize()
    o32, _ = pyoracle.present(a, b, 400, 150)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), o32.view(np.uint32))


def _scene_frame(seed):
    sc = soup_scene(seed, 1500, extent=10.0, sigma=0.6)
    fr = S.frame(S.look_at((0.0, 2.0, 28.0), (0.0, 0.0, 0.0), 40.0), 64 / 48, 0.1)
    return sc, fr


def test_draw_pingpong_matches_reference_binding(gpu_tracer):
    """Frames k = 0..3 traced into slot k % 2; every present reads slot 0 as
    the current image and slot 1 as the previous one."""
    tr = gpu_tracer
    sc, fr = _scene_frame(31)
    tr.upload_scene(sc)
    tr.draw_reset()
    p = abi.Tracer.params(64, 48, spp=2, max_depth=4, rr_start=2, sky=(1.0, 1.0, 1.0),
                          aovs=(abi.AOV_RGBA8,))
    slots = [np.zeros((48, 64, 4), np.uint8), np.zeros((48, 64, 4), np.uint8)]
    for k in range(4):
        f = fr.copy()
        f["seed"] = np.float32(0.1 + 0.173 * k)
        out8 = tr.draw(f, p, 80, 60, abi.PRESENT_PINGPONG, abi.AOV_RGBA8)
        slots[k % 2] = tr.readback(abi.AOV_RGBA8)
        _, o8 = pyoracle.present(slots[0], slots[1], 80, 60)
        assert np.array_equal(out8, o8), k
    # frames with different seeds differ, so the variance test fires somewhere
    assert not np.array_equal(slots[0], slots[1])


def test_draw_accumulate(gpu_tracer):
    tr = gpu_tracer
    sc, fr = _scene_frame(32)
    tr.upload_scene(sc)
    tr.draw_reset()
    w, h = 64, 48
    p = abi.Tracer.params(w, h, spp=1, max_depth=4, rr_start=2, sky=(1.0, 1.0, 1.0))
    s = np.zeros((h, w, 4), np.float32)
    prev = np.zeros((h, w, 4), np.float32)
    for k in range(5):
        f = fr.copy()
        f["seed"] = np.float32(0.05 + 0.11 * k)
        out = tr.draw(f, p, w, h, abi.PRESENT_ACCUMULATE, abi.AOV_RGBA32F)
        lin = tr.readback(abi.AOV_LINEAR)
        disp = pyoracle.accumulate(lin, s, k + 1)
        o32, _ = pyoracle.present(disp, prev, w, h)
        ok = np.abs(out - o32) <= 2e-7
        # a last-ulp tonemap difference can flip the variance test of a pixel
        assert ok.mean() > 0.999, (k, float(np.abs(out - o32).max()))
        prev = disp
    # a camera change restarts the mean: frame 1 of the new sequence
    f = fr.copy()
    f["camera"]["pos"] = f["camera"]["pos"] + np.float32(0.5)
    f["seed"] = np.float32(0.9)
    out = tr.draw(f, p, w, h, abi.PRESENT_ACCUMULATE, abi.AOV_RGBA32F)
    lin = tr.readback(abi.AOV_LINEAR)
    disp = pyoracle.accumulate(lin, np.zeros((h, w, 4), np.float32), 1)
    o32, _ = pyoracle.present(disp, np.zeros_like(disp), w, h)
    assert (np.abs(out - o32) <= 2e-7).mean() > 0.999


def test_present_rejects_bad_arguments(gpu_tracer):
    a = np.zeros((4, 4, 4), np.uint8)
    with pytest.raises(abi.TracerError) as e:
        gpu_tracer.present(a, a, 40000, 4)  # wider than 32768
    assert e.value.status == abi.ERR_NO_SUITABLE_SURFACE
    with pytest.raises(abi.TracerError) as e:
        gpu_tracer.present(a, a, 0, 4)  # nothing to write: no output buffer
    assert e.value.status == abi.ERR_INVALID_ARG
    with pytest.raises(abi.TracerError):
        gpu_tracer.present(a, a, 4, 4, out_aov=abi.AOV_PRIMARY_HIT)
