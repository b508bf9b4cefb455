"""The legacy Whitted shader (Assets/Raytracer.comp): the oracle's restatement
against vectors recorded from the shader compiled for the host, and the CUDA
kernel (through tracer_trace_whitted) against the oracle.

Bar: the oracle bit for bit against the recorded vectors; the GPU bit for bit
except the specular term's powf (CUDA vs the host C library may differ in
the last ulp): float RMSE <= 1e-6, RGBA8 within one step, and every pixel's
ray and hit counts equal."""
import hashlib

import numpy as np
import pytest

import pyoracle
from conftest import fbits, golden

from vktrace import abi
from vktrace import scene as S


def _sha(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = np.where(np.isnan(a), np.uint32(0x7FC00000), a.view(np.uint32))
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _frame(k):
    """Frame k of the vectors (stored as 24 floats: the 96-byte FrameData)."""
    return np.frombuffer(golden("ref_whitted.npz")["frames"][k].tobytes(), S.FRAME).reshape(()).copy()


def test_oracle_matches_raytracer_comp(oracle_lib):
    g = golden("ref_whitted.npz")
    for k in range(len(g["frames"])):
        fr = _frame(k)
        for w, h in ((64, 48), (97, 61)):
            o = pyoracle.whitted(fr, w, h)
            assert np.array_equal(fbits(o["rgba32f"]), fbits(g[f"f{k}_{w}x{h}_rgba32f"])), (k, w, h)
            assert np.array_equal(o["rgba8"], g[f"f{k}_{w}x{h}_rgba8"]), (k, w, h)
        o = pyoracle.whitted(fr, 1024, 1024)
        assert _sha(o["rgba32f"]) == str(g[f"f{k}_1024_sha_rgba32f"])
        assert _sha(o["rgba8"]) == str(g[f"f{k}_1024_sha_rgba8"])


@pytest.mark.gpu
@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("wh", [(64, 48), (97, 61), (1, 1), (1024, 1024)])
def test_gpu_whitted_vs_oracle(gpu_tracer, k, wh):
    w, h = wh
    fr = _frame(k)
    p = abi.Tracer.params(w, h, aovs=(abi.AOV_RGBA8, abi.AOV_RGBA32F), stats=True)
    gpu_tracer.trace_whitted(fr, p)
    img = gpu_tracer.readback(abi.AOV_RGBA32F)
    u8 = gpu_tracer.readback(abi.AOV_RGBA8)
    st = gpu_tracer.stats()
    o = pyoracle.whitted(fr, w, h)
    d = img.astype(np.float64) - o["rgba32f"]
    assert np.sqrt(np.mean(d * d)) <= 1e-6
    assert np.abs(u8.astype(int) - o["rgba8"].astype(int)).max() <= 1
    # the same paths: ray and hit counts equal
    for key in ("closest_rays", "shadow_rays", "hits"):
        assert st[key] == o["stats"][key], key
    # most pixels bit-identical (powf only enters lit, non-shadowed hits)
    assert (fbits(img) == fbits(o["rgba32f"])).mean() > 0.5


@pytest.mark.gpu
def test_gpu_whitted_needs_no_scene():
    t = abi.Tracer(0)
    try:
        p = abi.Tracer.params(32, 32)
        t.trace_whitted(S.reference_frame(0.5), p)
        assert t.readback(abi.AOV_RGBA8).shape == (32, 32, 4)
        with pytest.raises(abi.TracerError):
            t.trace_whitted(S.reference_frame(0.5), abi.Tracer.params(32, 32, aovs=(abi.AOV_PRIMARY_HIT,)))
    finally:
        t.close()
