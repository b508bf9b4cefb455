"""Adjoint trace: gradients of an L2 image loss with respect to material
albedo/emission and camera position, checked against central finite
differences (GPU forward, step 1e-3) and against an FP64 host evaluation
(the oracle in double precision).

Bar: relative error <= 1e-3 on the gradient components that carry the loss
(components below 1 % of the largest are compared in absolute terms)."""
import numpy as np
import pytest

import pyoracle
from gpu_cases import scene_bvhs
from vktrace import abi
from vktrace import scene as S

pytestmark = pytest.mark.gpu

GRAD_REL_TOL = 1e-3


def _scene(seed=7, n=1500, nm=12):
    tris, mats = S.triangle_soup(seed, n, extent=10.0, sigma=0.6, n_materials=nm)
    # a little emission on some materials (dielectric: linear; diffuse: normalised)
    g = S.SplitMix64(seed + 1)
    emit = g.uniform(nm) < 0.5
    mats["emissive"][emit] = np.c_[g.uniform(nm, 0.01, 0.05), g.uniform(nm, 0.01, 0.05), g.uniform(nm, 0.01, 0.05)][emit]
    return S.Scene(triangles=tris, materials=mats, bvh=S.BVH_SAH)


def _loss_and_dl(img, target):
    d = img[:, 1:, :3].astype(np.float64) - target[:, 1:, :3].astype(np.float64)
    dl = np.zeros(img.shape, np.float32)
    dl[:, 1:, :3] = 2.0 * d
    return float(np.sum(d * d)), dl


def _render(tr, sc, fr, p, mats=None, campos=None):
    if mats is not None:
        tr.set_materials(mats)
    f = np.array(fr, S.FRAME).reshape(())
    if campos is not None:
        f["camera"]["pos"] = campos
    tr.trace(f, p)
    return tr.readback(abi.AOV_RGBA32F), tr.readback(abi.AOV_LINEAR)


def _params(w, h, spp, depth, rr):
    return abi.Tracer.params(w, h, spp=spp, max_depth=depth, rr_start=rr, sky=(1.0, 1.0, 1.0),
                             aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR), kernel=abi.KERNEL_WAVEFRONT)


def _compare(grad, fd, what):
    grad, fd = np.asarray(grad, np.float64), np.asarray(fd, np.float64)
    scale = np.max(np.abs(fd))
    assert scale > 0, what
    big = np.abs(fd) >= 0.01 * scale
    rel = np.abs(grad[big] - fd[big]) / np.abs(fd[big])
    assert rel.max() <= GRAD_REL_TOL, (what, float(rel.max()), grad[big][:6], fd[big][:6])
    if (~big).any():
        assert np.max(np.abs(grad[~big] - fd[~big])) <= GRAD_REL_TOL * scale, what
    return float(rel.max())


def test_adjoint_vs_central_fd_gpu(gpu_tracer):
    """c3-shaped case (4 spp, depth 4, roulette only at the last depth, sky 1):
    albedo and emission gradients against central differences of the GPU
    forward image with step 1e-3."""
    tr = gpu_tracer
    sc = _scene()
    tr.upload_scene(sc)
    fr = S.frame(S.look_at((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    p = _params(96, 96, 4, 4, 3)
    base = sc.materials.copy()
    tgt_m = base.copy()
    g = S.SplitMix64(11)
    tgt_m["albedo"] = np.clip(base["albedo"] + 0.1 * g.normal(3 * len(base)).reshape(-1, 3), 0.0, 1.0)
    target, _ = _render(tr, sc, fr, p, tgt_m)
    img, lin = _render(tr, sc, fr, p, base)
    L0, dl = _loss_and_dl(img, target)
    ga, ge, gc = tr.trace_adjoint(fr, p, dl, lin, num_materials=len(base))  # the interior part alone
    assert np.all(gc == 0.0)  # no emitters: radiance does not depend on the camera away from edges
    # albedo: the stated step 1e-3.  Emission: diffuse emission enters as
    # normalize(e) with |e| ~ 0.03, whose curvature (and the acc clamp it
    # drives) makes a 1e-3 step ~3 % of |e|; a 1e-4 step keeps central
    # differences accurate there.
    steps = {"albedo": 1e-3, "emissive": 1e-4}
    fd_a = np.zeros_like(ga, dtype=np.float64)
    fd_e = np.zeros_like(ge, dtype=np.float64)
    for m in range(len(base)):
        for c in range(3):
            for field, fd in (("albedo", fd_a), ("emissive", fd_e)):
                if field == "emissive" and base["emissive"][m].min() <= 0:
                    continue  # zero emission: the normalised-emission branch is off on both sides of 0
                h = steps[field]
                mp, mm = base.copy(), base.copy()
                mp[field][m, c] += h
                mm[field][m, c] -= h
                Lp, _ = _loss_and_dl(_render(tr, sc, fr, p, mp)[0], target)
                Lm, _ = _loss_and_dl(_render(tr, sc, fr, p, mm)[0], target)
                step = float(np.float32(mp[field][m, c]) - np.float32(mm[field][m, c]))
                fd[m, c] = (Lp - Lm) / step
    tr.set_materials(base)
    _compare(ga, fd_a, "albedo")
    emit = base["emissive"].min(axis=1) > 0
    _compare(ge[emit], fd_e[emit], "emission")


def test_adjoint_vs_fp64_host(gpu_tracer):
    """The same gradient against central differences of the FP64 host
    evaluation (oracle in double precision, tiny step)."""
    tr = gpu_tracer
    sc = _scene(seed=9, n=800, nm=8)
    tb, _ = scene_bvhs(sc)
    tr.upload_scene(sc, tri_bvh=tb)
    fr = S.frame(S.look_at((1.0, 2.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.6)
    w = h = 40
    p = _params(w, h, 2, 4, 3)
    base = sc.materials.copy()
    tgt_m = base.copy()
    tgt_m["albedo"] = np.clip(base["albedo"] * 0.8 + 0.1, 0, 1)
    target, _ = _render(tr, sc, fr, p, tgt_m)
    img, lin = _render(tr, sc, fr, p, base)
    _, dl = _loss_and_dl(img, target)
    ga, ge, gc = tr.trace_adjoint(fr, p, dl, lin, num_materials=len(base))
    prm = pyoracle.params(w, h, spp=2, max_depth=4, rr_start=3, sky=(1, 1, 1))
    tgt64 = target[:, 1:, :3].astype(np.float64)

    def L64(mats):
        s2 = S.Scene(triangles=sc.triangles, materials=mats, bvh=sc.bvh)
        out = pyoracle.render_f64(s2, fr, prm, tri_bvh=tb)
        d = out["image"][:, 1:, :3] - tgt64
        return float(np.sum(d * d))

    hstep = 2.0 ** -12
    fd = np.zeros((len(base), 3))
    for m in range(len(base)):
        for c in range(3):
            mp, mm = base.copy(), base.copy()
            mp["albedo"][m, c] += hstep
            mm["albedo"][m, c] -= hstep
            fd[m, c] = (L64(mp) - L64(mm)) / (2 * hstep)
    tr.set_materials(base)
    _compare(ga, fd, "albedo vs FP64")


@pytest.mark.parametrize("hit_log", [True, False])
@pytest.mark.parametrize("case", ["sah-rr0", "sah-rr3-ragged", "linear-reference-ties"])
def test_wavefront_adjoint_equals_per_pixel(gpu_tracer, case, hit_log):
    """Scenes without emitters take the wavefront adjoint (closest hits
    through the forward extend kernel); the per-pixel adjoint kernel traces
    both passes of every sample.  With the hit log (opt-in) the wavefront
    traces pass 1 only and replays pass 2 from the logged hits: exactly half
    the per-pixel kernel's rays and hits; without it (limit 0, the default:
    pure path replay) it traces both passes: the same counts.  Gradients are
    equal up to the order of the FP64 sums either way."""
    tr = gpu_tracer
    tr.set_adjoint_hit_log((4 << 30) if hit_log else 0)
    sc = _scene(seed=21, n=2000, nm=16)
    tie = abi.TIES_STRICT
    if case.startswith("linear"):
        sc = S.Scene(triangles=sc.triangles[:300], materials=sc.materials, bvh=S.BVH_NONE)
        tie = abi.TIES_REFERENCE
    tr.upload_scene(sc)
    w, h = (77, 53) if "ragged" in case else (64, 64)
    rr = 0 if "rr0" in case or case.startswith("linear") else 3
    fr = S.frame(S.look_at((2.0, 1.0, 25.0), (0.0, 0.0, 0.0), 40.0), w / h, 0.45)
    p = abi.Tracer.params(w, h, spp=3, max_depth=5, rr_start=rr, sky=(1.0, 1.0, 1.0), tie_mode=tie,
                          aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR), kernel=abi.KERNEL_WAVEFRONT)
    base = sc.materials.copy()
    tgt_m = base.copy()
    tgt_m["albedo"] = np.clip(base["albedo"] * 0.7 + 0.2, 0, 1)
    target, _ = _render(tr, sc, fr, p, tgt_m)
    img, lin = _render(tr, sc, fr, p, base)
    _, dl = _loss_and_dl(img, target)
    out = {}
    # wavefront: rounds to the end (tail 1), the finishing kernel right after
    # generate (tail 2^32 - 1), and a hand-over part-way (700); the interior
    # part of the camera gradient (edge sampling off, the default), zero without emitters
    for k, tail in ((abi.KERNEL_PLAIN, 0), (abi.KERNEL_WAVEFRONT, 1), (abi.KERNEL_WAVEFRONT, 0xFFFFFFFF),
                    (abi.KERNEL_WAVEFRONT, 700)):
        p.kernel = k
        p.tail_paths = tail
        ga, ge, gc = tr.trace_adjoint(fr, p, dl, lin, num_materials=len(base))
        out[(k, tail)] = (ga, ge, gc, tr.stats())
    pa, pe, pc, ps = out[(abi.KERNEL_PLAIN, 0)]
    for key in ((abi.KERNEL_WAVEFRONT, 1), (abi.KERNEL_WAVEFRONT, 0xFFFFFFFF), (abi.KERNEL_WAVEFRONT, 700)):
        wa, we, wc, ws = out[key]
        if hit_log:
            assert ps["closest_rays"] == 2 * ws["closest_rays"] and ps["hits"] == 2 * ws["hits"], key
        else:
            assert ps["closest_rays"] == ws["closest_rays"] and ps["hits"] == ws["hits"], key
        assert ps["shadow_rays"] == ws["shadow_rays"] == 0
        assert np.all(wc == 0.0) and np.all(pc == 0.0)
        for a, b in ((pa, wa), (pe, we)):
            scale = float(np.max(np.abs(a))) if np.any(a) else 1.0
            np.testing.assert_allclose(b, a, rtol=1e-5, atol=1e-7 * scale, err_msg=str(key))
        assert np.any(wa != 0)
    tr.set_adjoint_hit_log(0)  # the default: pure replay


def _nee_scene(kind):
    """Scenes whose depth-1 image depends smoothly on the camera position
    (through the hit points, the sphere normals and the next-event view
    vector) with no occlusion boundary in view:
      floor:  a diffuse floor (two triangles, table material) lit by an
              emissive sphere outside the view;
      sphere: a lone diffuse sphere (inline material) lit the same way; the
              silhouette's pixels are excluded by primary-hit comparison."""
    mats = np.zeros(1, S.MATERIAL)
    mats[0] = S.material((0.7, 0.6, 0.5), (0, 0, 0), 0.6, 0.2, S.MAT_DIFFUSE)
    light = np.zeros(1, S.SPHERE)
    light[0]["mat"] = S.material((1, 1, 1), (60.0, 55.0, 50.0), 0.5, 0.0, S.MAT_DIFFUSE)
    light[0]["P"], light[0]["r"] = (45.0, 30.0, 5.0), 6.0
    if kind == "floor":
        tris = np.zeros(2, S.TRIANGLE)
        a, b, c_, d = (-60.0, 0.0, -60.0), (60.0, 0.0, -60.0), (60.0, 0.0, 60.0), (-60.0, 0.0, 60.0)
        tris[0]["v0"], tris[0]["v1"], tris[0]["v2"] = a, c_, b
        tris[1]["v0"], tris[1]["v1"], tris[1]["v2"] = a, d, c_
        return S.Scene(triangles=tris, materials=mats, spheres=light, bvh=S.BVH_NONE)
    sph = np.zeros(2, S.SPHERE)
    sph[0] = light[0]
    sph[1]["mat"] = S.material((0.3, 0.5, 0.7), (0, 0, 0), 0.4, 0.3, S.MAT_DIFFUSE)
    sph[1]["P"], sph[1]["r"] = (0.0, 4.0, 6.0), 9.0
    return S.Scene(materials=mats, spheres=sph, bvh=S.BVH_NONE)


@pytest.mark.parametrize("kind", ["floor", "sphere"])
def test_camera_and_nee_gradients_vs_fp64(gpu_tracer, kind):
    tr = gpu_tracer
    sc = _nee_scene(kind)
    tr.upload_scene(sc)
    cam = S.look_at((0.0, 30.0, -20.0), (0.0, 0.0, 8.0), 35.0)
    fr = S.frame(cam, 1.0, 0.2)
    w = h = 48
    p = abi.Tracer.params(w, h, spp=1, max_depth=1, rr_start=1, aovs=(abi.AOV_RGBA32F, abi.AOV_LINEAR),
                          tie_mode=abi.TIES_STRICT)
    base = sc.materials.copy()
    tgt_f = np.array(fr, S.FRAME).reshape(())
    tgt_f["camera"]["pos"] = (0.5, 29.0, -21.0)
    tr.trace(tgt_f, p)
    target = tr.readback(abi.AOV_RGBA32F)
    img, lin = _render(tr, sc, fr, p)
    _, dl = _loss_and_dl(img, target)
    # the interior part (edge sampling off, the default; the differences below
    # exclude pixels whose visible primitive changes); the boundary part has
    # tests of its own
    ga, ge, gc = tr.trace_adjoint(fr, p, dl, lin, num_materials=1)
    prm = pyoracle.params(w, h, spp=1, max_depth=1, rr_start=1, tie_mode=1)
    prm_f = pyoracle.params(w, h, spp=1, max_depth=1, rr_start=1, tie_mode=1)
    tgt64 = target[:, 1:, :3].astype(np.float64)
    pos0 = np.array(fr["camera"]["pos"], np.float32)

    def run(pos, mats=base):
        f = np.array(fr, S.FRAME).reshape(())
        f["camera"]["pos"] = pos
        s2 = S.Scene(triangles=sc.triangles, materials=mats, spheres=sc.spheres)
        o = pyoracle.render_f64(s2, f, prm)
        hid = pyoracle.render(s2, f, prm_f)["hit_id"][:, 1:]
        return o["image"][:, 1:, :3], hid

    hcam = 2.0 ** -12
    fd_c = np.zeros(3)
    for j in range(3):
        pp, pm = pos0.copy(), pos0.copy()
        pp[j] += hcam
        pm[j] -= hcam
        ip, hp = run(pp)
        im, hm = run(pm)
        same = (hp == hm)[..., None]  # pixels whose visible primitive did not change
        d = (np.sum(np.where(same, (ip - tgt64) ** 2, 0)) - np.sum(np.where(same, (im - tgt64) ** 2, 0)))
        fd_c[j] = d / (2 * hcam)
    _compare(gc, fd_c, "camera position")
    if kind != "floor":
        return  # the sphere's material is stored inline: no albedo gradient
    hstep = 2.0 ** -12
    fd_a = np.zeros(3)
    for c in range(3):
        mp, mm = base.copy(), base.copy()
        mp["albedo"][0, c] += hstep
        mm["albedo"][0, c] -= hstep
        ip, _ = run(pos0, mp)
        im, _ = run(pos0, mm)
        fd_a[c] = (np.sum((ip - tgt64) ** 2) - np.sum((im - tgt64) ** 2)) / (2 * hstep)
    _compare(ga[0], fd_a, "albedo through next-event estimation")


def test_autograd_function(gpu_tracer):
    torch = pytest.importorskip("torch")
    from vktrace.autograd import DifferentiableRenderer
    sc = _scene(seed=13, n=600, nm=6)
    fr = S.frame(S.look_at((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0), 1.0, 0.3)
    p = _params(48, 40, 2, 4, 3)
    r = DifferentiableRenderer(gpu_tracer, sc, fr, p)
    alb = torch.tensor(sc.materials["albedo"], device="cuda", requires_grad=True)
    emi = torch.tensor(sc.materials["emissive"], device="cuda", requires_grad=True)
    cam = torch.tensor(np.array(fr["camera"]["pos"]), device="cuda", requires_grad=True)
    target = torch.full((40, 48, 3), 0.5, device="cuda")
    img = r.render(alb, emi, cam)
    loss = ((img[:, 1:] - target[:, 1:]) ** 2).sum()
    loss.backward()
    # the same gradient through the C ABI directly
    dl = np.zeros((40, 48, 4), np.float32)
    dl[:, 1:, :3] = 2.0 * (img[:, 1:].detach().cpu().numpy() - 0.5)
    gpu_tracer.trace(fr, p)
    lin = gpu_tracer.readback(abi.AOV_LINEAR)
    ga, ge, gc = gpu_tracer.trace_adjoint(fr, p, dl, lin, num_materials=6)
    assert np.allclose(alb.grad.cpu().numpy(), ga, rtol=1e-5, atol=1e-6)
    assert np.allclose(emi.grad.cpu().numpy(), ge, rtol=1e-5, atol=1e-6)
