"""Camera-position gradient, boundary part (edge sampling of triangle
outlines), through the C ABI.

The forward image is point-sampled: each pixel's samples all pass through
one point, so as the camera moves a pixel keeps its value until an outline
crosses that point, then jumps.  Central differences of the loss with step h
therefore count crossing events; averaged over where outlines fall relative
to the pixel grid, their expectation is the boundary integral the adjoint
computes (the derivative of each pixel averaged over a one-pixel box around
its sample point).  The check renders the differences at 32 x 32 stratified
sub-pixel offsets of all sample points (the camera's dir moved by a fraction
of a pixel along right and up), which averages over that box; their
standard error comes from the spread of 16 random groups of the offsets
(interleaved grids of offsets see nearly the same events and understate
it), and the gradient must lie within 4 standard errors plus a few per cent
of them.  The step must be small against the triangles' images: on c3's
~2-pixel triangles a step of 0.02 (0.28 pixel) lets a sample point cross
both sides of a triangle and biases the quotient towards zero.  Common random numbers: every render uses the same seed, so only the
geometry moves.  A linear loss (fixed random weights per pixel) makes dL/dI
exact at every camera position.
"""
import numpy as np
import pytest

from vktrace import abi, configs
from vktrace import scene as S

pytestmark = pytest.mark.gpu


def _adjoint_with_edges(tr, frame, p, dl, lin, nm, pieces=4):
    """tracer_trace_adjoint with the boundary part on, then off again (the
    default)."""
    tr.set_edge_sampling(pieces)
    try:
        return tr.trace_adjoint(frame, p, dl, lin, num_materials=nm)
    finally:
        tr.set_edge_sampling(0)


def _weights(h, w, seed=5):
    g = np.random.default_rng(seed)
    dl = np.zeros((h, w, 4), np.float32)
    dl[:, 1:, :3] = g.normal(size=(h, w - 1, 3)).astype(np.float32)  # column 0 is NaN by construction
    return dl


def _render(tr, frame, p, pos=None, offset=(0.0, 0.0)):
    """The frame, optionally with the camera at pos and every sample point
    moved by offset (in pixels) along the camera's right and up vectors."""
    f = np.array(frame, S.FRAME).reshape(())
    if pos is not None:
        f["camera"]["pos"] = pos
    if offset != (0.0, 0.0):
        cam = f["camera"]
        cam["dir"] = (cam["dir"].astype(np.float64) + cam["right"] * (2.0 * offset[0] / p.width)
                      + cam["up"] * (2.0 * offset[1] / p.height)).astype(np.float32)
    tr.trace(f, p)
    return tr.readback(abi.AOV_RGBA32F)


def box_averaged_fd(tr, frame, p, dl, axis, h, k_side=32):
    """Central differences of the linear loss sum(dl * image) along the
    camera axis, averaged over k_side^2 stratified sub-pixel offsets; returns
    (mean, its standard error, crossing events).  The standard error comes
    from 16 random groups of the offsets: the spread of their means over 4."""
    pos = np.array(frame["camera"]["pos"], np.float64).reshape(3)
    up, dn = pos.copy(), pos.copy()
    up[axis] += h
    dn[axis] -= h
    step = float(np.float32(up[axis]) - np.float32(dn[axis]))
    per = np.zeros((k_side, k_side))
    events = 0
    for i in range(k_side):
        for j in range(k_side):
            off = ((i + 0.5) / k_side - 0.5, (j + 0.5) / k_side - 0.5)
            a = _render(tr, frame, p, up.astype(np.float32), off)
            b = _render(tr, frame, p, dn.astype(np.float32), off)
            d = ((a[:, 1:, :3].astype(np.float64) - b[:, 1:, :3]) * dl[:, 1:, :3]).sum(axis=-1) / step
            per[i, j] = d.sum()
            events += int((d != 0.0).sum())
    groups = np.random.default_rng(1).permutation(k_side * k_side).reshape(16, -1)
    flat = per.ravel()
    subs = [flat[q].mean() for q in groups]
    return float(per.mean()), float(np.std(subs, ddof=1) / 4.0), events


def _c3_like(depth, width=256):
    wl = configs.c3(width=width)
    p = abi.Tracer.params(wl.width, wl.height, spp=wl.spp, max_depth=depth, rr_start=wl.rr_start, sky=wl.sky,
                          aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR))
    return wl, p


def _layers(seed=11, n=40):
    """Large triangles facing the camera at distinct depths (they overlap in
    the image but never intersect), one diffuse material."""
    g = np.random.default_rng(seed)
    tris = np.zeros(n, S.TRIANGLE)
    for i in range(n):
        c = np.r_[g.uniform(-8.0, 8.0, 2), -8.0 + 16.0 * i / n]
        v = c + g.normal(0.0, 2.5, (3, 3))
        v[:, 2] = c[2]
        if np.cross(v[1] - v[0], v[2] - v[0])[2] < 0:  # front face towards the camera at +z
            v[[1, 2]] = v[[2, 1]]
        tris[i]["v0"], tris[i]["v1"], tris[i]["v2"] = v
    mats = np.zeros(1, S.MATERIAL)
    mats[0] = S.material((0.5, 0.6, 0.7), (0, 0, 0), 0.5, 0.0, S.MAT_DIFFUSE)
    return S.Scene(triangles=tris, materials=mats, bvh=S.BVH_SAH)


def test_campos_boundary_layers_vs_box_averaged_fd(gpu_tracer):
    """Pure primary visibility (depth 1, sky 1): 40 large overlapping
    triangles at distinct depths, random per-pixel loss weights, all three
    camera axes.  The boundary term is the whole camera gradient here, and
    its estimate is exact up to the integration along each outline."""
    tr = gpu_tracer
    sc = _layers()
    tr.upload_scene(sc)
    fr = S.frame(S.look_at((1.0, 2.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    p = abi.Tracer.params(192, 192, spp=2, max_depth=1, rr_start=3, sky=(1.0, 1.0, 1.0),
                          aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR))
    _render(tr, fr, p)
    lin = tr.readback(abi.AOV_LINEAR)
    dl = _weights(p.height, p.width, seed=7)
    _, _, gc = _adjoint_with_edges(tr, fr, p, dl, lin, 1)
    rows = []
    for axis in range(3):
        fd, se, events = box_averaged_fd(tr, fr, p, dl, axis, h=0.02, k_side=16)
        rows.append((axis, float(gc[axis]), fd, se, events))
    for axis, g, fd, se, events in rows:
        assert events > 10000, rows
        assert abs(g - fd) <= 4.0 * se + 0.03 * abs(fd), rows


@pytest.mark.parametrize("depth", [1, 4])
def test_campos_boundary_c3_dolly(gpu_tracer, depth):
    """c3's scene and frame (256^2, 4 spp, 10k triangles, sky 1, no emitters:
    the camera enters the image only through visibility), moving along the
    view axis, loss = the image's sum (every outline moves coherently as
    the projected triangles grow or shrink).  Depth 1 is pure primary
    visibility, which the boundary term models; at depth 4 outlines seen by
    bounce rays also move (not modelled), so the bound there is 15 % of the
    difference quotient."""
    tr = gpu_tracer
    wl, p = _c3_like(depth)
    tr.upload_scene(wl.scene)
    _render(tr, wl.frame, p)
    lin = tr.readback(abi.AOV_LINEAR)
    dl = np.zeros((wl.height, wl.width, 4), np.float32)
    dl[:, 1:, :3] = 1.0
    _, _, gc = _adjoint_with_edges(tr, wl.frame, p, dl, lin, len(wl.scene.materials), pieces=16)
    fd, se, events = box_averaged_fd(tr, wl.frame, p, dl, 2, h=0.02, k_side=16)
    slack = 0.05 if depth == 1 else 0.15
    assert events > 10000, (fd, se, events)
    assert abs(float(gc[2]) - fd) <= 4.0 * se + slack * abs(fd), (depth, float(gc[2]), fd, se, events)


def _smooth_weights(h, w):
    """Positive weights varying smoothly over the image: the loss moves with
    every outline coherently instead of as a sum of random signs."""
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    dl = np.zeros((h, w, 4), np.float32)
    for c in range(3):
        dl[:, :, c] = 1.0 + 0.5 * np.sin(2 * np.pi * (xx / w + c / 3.0)) + 0.5 * np.cos(2 * np.pi * yy / h)
    dl[:, 0] = 0.0
    return dl


@pytest.mark.parametrize("depth", [1, 4])
def test_campos_boundary_c3_all_axes(gpu_tracer, depth):
    """c3's scene and frame, all three camera axes, smooth loss weights,
    step 0.01 (0.14 pixel: small against the ~2-pixel triangles): the
    gradient within 4 standard errors of the box-averaged differences at
    depth 1 (primary visibility only) and at c3's depth 4 (outlines seen by
    bounce rays are not modelled; their part is within the noise here)."""
    tr = gpu_tracer
    wl, p = _c3_like(depth)
    tr.upload_scene(wl.scene)
    _render(tr, wl.frame, p)
    lin = tr.readback(abi.AOV_LINEAR)
    dl = _smooth_weights(wl.height, wl.width)
    _, _, gc = _adjoint_with_edges(tr, wl.frame, p, dl, lin, len(wl.scene.materials), pieces=16)
    rows = []
    for axis in range(3):
        fd, se, events = box_averaged_fd(tr, wl.frame, p, dl, axis, h=0.01, k_side=32)
        rows.append((axis, float(gc[axis]), fd, se, events))
    for axis, g, fd, se, events in rows:
        assert events > 10000, rows
        assert abs(g - fd) <= 4.0 * se, (depth, rows)


def test_edge_sampling_off_leaves_interior_part(gpu_tracer):
    """Off (the default), an emitter-free scene's camera gradient is the
    interior part alone, zero; on, the outlines make it nonzero (with one
    piece per edge and with four); the albedo gradient does not depend on
    the setting."""
    tr = gpu_tracer
    tr.upload_scene(_layers())
    fr = S.frame(S.look_at((1.0, 2.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    p = abi.Tracer.params(96, 96, spp=2, max_depth=1, rr_start=3, sky=(1.0, 1.0, 1.0),
                          aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR))
    _render(tr, fr, p)
    lin = tr.readback(abi.AOV_LINEAR)
    dl = _weights(p.height, p.width, seed=9)
    ga0, _, gc0 = tr.trace_adjoint(fr, p, dl, lin, num_materials=1)
    ga1, _, gc1 = _adjoint_with_edges(tr, fr, p, dl, lin, 1, pieces=1)
    ga4, _, gc4 = _adjoint_with_edges(tr, fr, p, dl, lin, 1, pieces=4)
    assert np.all(gc0 == 0.0)
    assert np.all(gc1 != 0.0) and np.all(gc4 != 0.0)
    assert np.array_equal(ga0, ga1) and np.array_equal(ga0, ga4)
    with pytest.raises(abi.TracerError):
        tr.set_edge_sampling(4096)
