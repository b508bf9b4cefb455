"""Python wrapper of the CPU oracle and of the reference-shader harness.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, to check or time the CUDA path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

STATS_FIELDS = ["closest_rays", "shadow_rays", "node_fetches", "tri_tests", "sphere_tests", "plane_tests", "hits"]


class OScene(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_void_p), ("num_triangles", ctypes.c_uint32),
                ("materials", ctypes.c_void_p), ("num_materials", ctypes.c_uint32),
                ("spheres", ctypes.c_void_p), ("num_spheres", ctypes.c_uint32),
                ("planes", ctypes.c_void_p), ("num_planes", ctypes.c_uint32),
                ("tri_nodes", ctypes.c_void_p), ("num_tri_nodes", ctypes.c_uint32),
                ("tri_prim_index", ctypes.c_void_p),
                ("sphere_nodes", ctypes.c_void_p), ("num_sphere_nodes", ctypes.c_uint32),
                ("sphere_prim_index", ctypes.c_void_p)]


class OParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32), ("rr_start", ctypes.c_uint32), ("sky", ctypes.c_float * 3),
                ("tie_mode", ctypes.c_int32), ("trig_mode", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("row_begin", ctypes.c_uint32), ("row_end", ctypes.c_uint32), ("row_step", ctypes.c_uint32)]


class OStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in STATS_FIELDS]


class OCameraCtl(ctypes.Structure):
    _fields_ = [("cam", ctypes.c_float * 16), ("front", ctypes.c_float * 3), ("pitch", ctypes.c_float),
                ("yaw", ctypes.c_float), ("last_mouse", ctypes.c_float * 2)]


def build() -> str:
    """Builds liboracle.so (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def reference_root() -> str:
    """Where the reference tree is read from: $VKTRACE_REFERENCE_ROOT, else the
    harness recipe's default (its REF variable)."""
    env = os.environ.get("VKTRACE_REFERENCE_ROOT")
    if env:
        return env
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(HERE, "ref"), "ref-dir"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def reference_present() -> bool:
    root = reference_root()
    return bool(root) and os.path.isdir(os.path.join(root, "Assets"))


def build_ref() -> bool:
    """Builds the reference-shader harness when the reference tree exists."""
    if not reference_present():
        return False
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"OUT={REF_DIR}", f"REF={reference_root()}"],
                   check=True)
    return True


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, f32, i32 = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
        L.oracle_render.argtypes = [ctypes.POINTER(OScene), vp, ctypes.POINTER(OParams), vp, vp, vp, vp,
                                    ctypes.POINTER(OStats)]
        L.oracle_render_f64.argtypes = [ctypes.POINTER(OScene), vp, ctypes.POINTER(OParams), vp, vp,
                                        ctypes.POINTER(OStats)]
        L.oracle_rand.argtypes = [f32, f32, f32, i32, i32, vp]
        L.oracle_rand.restype = None
        L.oracle_cos.argtypes = [f32]
        L.oracle_cos.restype = f32
        L.oracle_sin.argtypes = [f32]
        L.oracle_sin.restype = f32
        for fn in ("oracle_tri_intersect",):
            getattr(L, fn).argtypes = [vp, vp, vp]
            getattr(L, fn).restype = f32
        L.oracle_sphere_intersect.argtypes = [vp, vp, vp, f32]
        L.oracle_sphere_intersect.restype = f32
        L.oracle_plane_intersect.argtypes = [vp, vp, vp, f32]
        L.oracle_plane_intersect.restype = f32
        L.oracle_trace_ray.argtypes = [ctypes.POINTER(OScene), i32, i32, vp, vp, f32, vp, ctypes.POINTER(OStats)]
        L.oracle_radiance.argtypes = [ctypes.POINTER(OScene), vp, ctypes.POINTER(OParams), vp, vp, f32, f32, f32,
                                      vp, vp]
        L.oracle_radiance.restype = None
        u32 = ctypes.c_uint32
        L.oracle_present.argtypes = [vp, vp, i32, u32, u32, u32, u32, vp, vp]
        L.oracle_present.restype = None
        L.oracle_accumulate.argtypes = [vp, vp, u32, u32, vp]
        L.oracle_accumulate.restype = None
        L.oracle_whitted.argtypes = [vp, u32, u32, vp, vp, ctypes.POINTER(OStats)]
        L.oracle_whitted.restype = None
        pc = ctypes.POINTER(OCameraCtl)
        for fn, args in (("oracle_camera_init", [pc]), ("oracle_camera_update", [pc]),
                         ("oracle_camera_move", [pc, i32, f32]),
                         ("oracle_camera_mouse", [pc, ctypes.c_double, ctypes.c_double]),
                         ("oracle_camera_keyboard", [pc, u32, f32])):
            getattr(L, fn).argtypes = args
            getattr(L, fn).restype = None
        L.oracle_build_bvh.argtypes = [i32, i32, vp, u32, u32, u32, vp, ctypes.POINTER(u32), vp,
                                       ctypes.POINTER(u32)]
        L.oracle_build_bvh.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None or a.size == 0 else a.ctypes.data_as(ctypes.c_void_p)


class _SceneRef:
    """Keeps numpy arrays alive while the oracle reads them."""

    def __init__(self, sc, tri_bvh=None, sphere_bvh=None):
        self.arrs = [np.ascontiguousarray(a) for a in (sc.triangles, sc.materials, sc.spheres, sc.planes)]
        self.s = OScene()
        s = self.s
        s.triangles, s.num_triangles = _p(self.arrs[0]), len(self.arrs[0])
        s.materials, s.num_materials = _p(self.arrs[1]), len(self.arrs[1])
        s.spheres, s.num_spheres = _p(self.arrs[2]), len(self.arrs[2])
        s.planes, s.num_planes = _p(self.arrs[3]), len(self.arrs[3])
        if tri_bvh is not None:
            n, i = np.ascontiguousarray(tri_bvh[0]), np.ascontiguousarray(tri_bvh[1], np.uint32)
            self.arrs += [n, i]
            s.tri_nodes, s.num_tri_nodes, s.tri_prim_index = _p(n), len(n), _p(i)
        if sphere_bvh is not None:
            n, i = np.ascontiguousarray(sphere_bvh[0]), np.ascontiguousarray(sphere_bvh[1], np.uint32)
            self.arrs += [n, i]
            s.sphere_nodes, s.num_sphere_nodes, s.sphere_prim_index = _p(n), len(n), _p(i)


def params(width, height, spp=4, max_depth=4, rr_start=0, sky=(0.0, 0.0, 0.0), tie_mode=1, trig_mode=0, threads=0,
           rows=None) -> OParams:
    p = OParams()
    p.width, p.height, p.spp, p.max_depth, p.rr_start = width, height, spp, max_depth, rr_start
    p.sky = (ctypes.c_float * 3)(*sky)
    p.tie_mode, p.trig_mode, p.threads = tie_mode, trig_mode, threads
    if rows is not None:
        p.row_begin, p.row_end, p.row_step = rows
    return p


# 32-byte BVH node record (bmin, left_or_first, bmax, count), as the product's
NODE = np.dtype({"names": ["bmin", "left_or_first", "bmax", "count"],
                 "formats": [("<f4", 3), "<i4", ("<f4", 3), "<i4"], "offsets": [0, 12, 16, 28], "itemsize": 32})


def build_bvh(kind: int, prims: np.ndarray, leaf_size: int = 0, sah_bins: int = 0):
    """The oracle's own BVH builder (bvh_oracle.cpp): kind 1 = median split,
    2 = binned SAH; prims = 48-byte triangle or 64-byte sphere records.
    Returns (nodes, prim_index, depth) like the product's builder."""
    L = lib()
    prims = np.ascontiguousarray(prims)
    ptype = 0 if prims.dtype.itemsize == 48 else 1
    n = len(prims)
    nodes = np.zeros(max(1, 2 * n), NODE)
    idx = np.zeros(n, np.uint32)
    nn, depth = ctypes.c_uint32(), ctypes.c_uint32()
    r = L.oracle_build_bvh(kind, ptype, _p(prims), n, leaf_size, sah_bins, _p(nodes), ctypes.byref(nn), _p(idx),
                           ctypes.byref(depth))
    if r != 0:
        raise ValueError("oracle_build_bvh: bad arguments")
    return nodes[: nn.value].copy(), idx, depth.value


def render(sc, frame, prm: OParams, tri_bvh=None, sphere_bvh=None):
    """Renders with the oracle; returns dict(rgba32f, rgba8, hit_id, hit_t, stats)."""
    L = lib()
    ref = _SceneRef(sc, tri_bvh, sphere_bvh)
    f = np.ascontiguousarray(frame).reshape(())
    h, w = prm.height, prm.width
    rgba = np.zeros((h, w, 4), np.float32)
    u8 = np.zeros((h, w, 4), np.uint8)
    hid = np.full((h, w), 0xFFFFFFFF, np.uint32)
    ht = np.full((h, w), -1.0, np.float32)
    st = OStats()
    L.oracle_render(ctypes.byref(ref.s), f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(prm), _p(rgba), _p(u8),
                    _p(hid), _p(ht), ctypes.byref(st))
    return {"rgba32f": rgba, "rgba8": u8, "hit_id": hid, "hit_t": ht,
            "stats": {k: int(getattr(st, k)) for k in STATS_FIELDS}}


def render_f64(sc, frame, prm: OParams, tri_bvh=None, sphere_bvh=None):
    """FP64 evaluation of the same paths (RNG in float): returns dict(lin =
    mean radiance (h, w, 3), image = tonemap(lin) + dither in double)."""
    L = lib()
    ref = _SceneRef(sc, tri_bvh, sphere_bvh)
    f = np.ascontiguousarray(frame).reshape(())
    h, w = prm.height, prm.width
    rgba = np.zeros((h, w, 4), np.float32)
    acc = np.zeros((h, w, 4), np.float64)
    st = OStats()
    L.oracle_render_f64(ctypes.byref(ref.s), f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(prm), _p(rgba), _p(acc),
                        ctypes.byref(st))
    lin = acc[..., :3]
    x = lin / (lin + 1.0)
    gamma = np.float64(np.float32(1.0) / np.float32(2.2))  # the shader's 1.0 / 2.2 in float
    with np.errstate(invalid="ignore"):
        img = np.power(x, gamma)
    return {"lin": lin, "image": img + acc[..., 3:4], "rgba32f": rgba}


def rand(cx, cy, salt, n, trig_mode=0):
    out = np.zeros(n, np.float32)
    lib().oracle_rand(cx, cy, salt, trig_mode, n, _p(out))
    return out


def trace_ray(sc, o, d, tmax, tie_mode=1, shadow=False, tri_bvh=None, sphere_bvh=None):
    L = lib()
    ref = _SceneRef(sc, tri_bvh, sphere_bvh)
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    out = np.zeros(21, np.float32)
    st = OStats()
    found = L.oracle_trace_ray(ctypes.byref(ref.s), tie_mode, int(shadow), _p(o), _p(d), tmax, _p(out),
                               ctypes.byref(st))
    return {"found": bool(found), "t": float(out[1]), "P": out[2:5].copy(), "N": out[5:8].copy(),
            "material": out[8:20].copy(), "prim": int(out[20:21].view(np.uint32)[0]),
            "stats": {k: int(getattr(st, k)) for k in STATS_FIELDS}}


# ------------------------------------------------------- reference harness --
class RefHarness:
    """The reference shader compiled for the host (oracle/ref/Makefile)."""

    def __init__(self, rng_trig: bool = False):
        name = "libref_tracer_rngtrig.so" if rng_trig else "libref_tracer.so"
        path = os.path.join(REF_DIR, name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        vp, f32, u32, i32 = ctypes.c_void_p, ctypes.c_float, ctypes.c_uint, ctypes.c_int
        L.ref_render.argtypes = [vp, vp, u32, i32, i32, vp, vp]
        L.ref_render.restype = None
        L.ref_radiance.argtypes = [vp, vp, u32, vp, vp, f32, f32, f32, vp, vp]
        L.ref_radiance.restype = None
        L.ref_rand.argtypes = [f32, f32, f32, i32, vp]
        L.ref_rand.restype = None
        L.ref_trace_ray.argtypes = [vp, u32, vp, vp, f32, vp]
        L.ref_trace_ray.restype = None
        L.ref_tri_intersect.argtypes = [vp, vp, vp]
        L.ref_tri_intersect.restype = f32
        L.ref_sphere_intersect.argtypes = [vp, vp, vp, f32]
        L.ref_sphere_intersect.restype = f32
        L.ref_plane_intersect.argtypes = [vp, vp, vp, f32]
        L.ref_plane_intersect.restype = f32
        L.ref_scene_constants.argtypes = [vp, vp, vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
        L.ref_scene_constants.restype = u32
        self.L = L

    def render(self, frame, triangles, w, h):
        f = np.ascontiguousarray(frame).reshape(())
        t = np.ascontiguousarray(triangles)
        rgba = np.zeros((h, w, 4), np.float32)
        u8 = np.zeros((h, w, 4), np.uint8)
        self.L.ref_render(f.ctypes.data_as(ctypes.c_void_p), _p(t), len(t), w, h, _p(rgba), _p(u8))
        return rgba, u8

    def rand(self, cx, cy, salt, n):
        out = np.zeros(n, np.float32)
        self.L.ref_rand(cx, cy, salt, n, _p(out))
        return out

    def trace_ray(self, triangles, o, d, tmax):
        t = np.ascontiguousarray(triangles)
        out = np.zeros(20, np.float32)
        self.L.ref_trace_ray(_p(t), len(t), _p(np.asarray(o, np.float32)), _p(np.asarray(d, np.float32)), tmax,
                             _p(out))
        return out

    def scene_constants(self):
        sph = np.zeros(16 * 16, np.float32)
        pl = np.zeros(16 * 16, np.float32)
        tm = np.zeros(12, np.float32)
        ns, npl = ctypes.c_uint(), ctypes.c_uint()
        code = self.L.ref_scene_constants(_p(sph), _p(pl), _p(tm), ctypes.byref(ns), ctypes.byref(npl))
        return (sph[: 16 * ns.value].reshape(ns.value, 16), pl[: 16 * npl.value].reshape(npl.value, 16), tm,
                divmod(code, 1000))


def ref_camera(pos, pitch, yaw):
    L = ctypes.CDLL(os.path.join(REF_DIR, "libref_camera.so"))
    out = np.zeros(16, np.float32)
    f32 = ctypes.c_float
    L.ref_camera.argtypes = [f32, f32, f32, f32, f32, ctypes.c_void_p]
    L.ref_camera.restype = None
    L.ref_camera(pos[0], pos[1], pos[2], pitch, yaw, _p(out))
    return out


# ------------------------------------------------ present / accumulate --
def present(image0, image1, width, height):
    """The present pass (Fullscreen.frag) over two (h, w, 4) source images,
    uint8 (RGBA8 UNORM) or float32; returns (rgba32f, rgba8) of the
    width x height framebuffer, row 0 at the top."""
    a = np.ascontiguousarray(image0)
    b = np.ascontiguousarray(image1)
    assert a.shape == b.shape and a.dtype == b.dtype and a.dtype in (np.uint8, np.float32)
    out32 = np.zeros((height, width, 4), np.float32)
    out8 = np.zeros((height, width, 4), np.uint8)
    lib().oracle_present(_p(a), _p(b), int(a.dtype == np.float32), a.shape[1], a.shape[0], width, height,
                         _p(out32), _p(out8))
    return out32, out8


def accumulate(linear, sum_rgba, n):
    """One frame of progressive accumulation: sum_rgba (h, w, 4) float32 is
    updated in place; returns the tonemapped mean after n frames."""
    lin = np.ascontiguousarray(linear, np.float32)
    assert sum_rgba.flags.c_contiguous and sum_rgba.dtype == np.float32
    disp = np.zeros_like(lin)
    lib().oracle_accumulate(_p(lin), _p(sum_rgba), lin.shape[0] * lin.shape[1], n, _p(disp))
    return disp


class CameraCtl:
    """The camera controller restated (Camera.cpp, Main.cpp input)."""

    def __init__(self):
        self.c = OCameraCtl()
        lib().oracle_camera_init(ctypes.byref(self.c))

    def update(self):
        lib().oracle_camera_update(ctypes.byref(self.c))

    def move(self, direction, speed):
        lib().oracle_camera_move(ctypes.byref(self.c), direction, speed)

    def mouse(self, x, y):
        lib().oracle_camera_mouse(ctypes.byref(self.c), x, y)

    def keyboard(self, keys, dt):
        lib().oracle_camera_keyboard(ctypes.byref(self.c), keys, dt)

    def state(self) -> np.ndarray:
        """CameraData (16), front (3), pitch, yaw as float32 (21)."""
        c = self.c
        return np.array(list(c.cam) + list(c.front) + [c.pitch, c.yaw], np.float32)


def ref_present(image0, image1, width, height):
    """The reference's Fullscreen.frag compiled for the host (oracle/_ref)."""
    L = ctypes.CDLL(os.path.join(REF_DIR, "libref_present.so"))
    u32 = ctypes.c_uint32
    L.ref_present.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, u32, u32, u32, u32, ctypes.c_void_p]
    L.ref_present.restype = None
    a = np.ascontiguousarray(image0)
    b = np.ascontiguousarray(image1)
    out = np.zeros((height, width, 4), np.float32)
    L.ref_present(_p(a), _p(b), int(a.dtype == np.float32), a.shape[1], a.shape[0], width, height, _p(out))
    return out


def ref_camera_ops(ops, args):
    """Camera.cpp operations from the default camera; (n, 21) states."""
    L = ctypes.CDLL(os.path.join(REF_DIR, "libref_camera.so"))
    L.ref_camera_ops.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_camera_ops.restype = None
    op = np.ascontiguousarray(ops, np.int32)
    ar = np.ascontiguousarray(args, np.float32).reshape(-1)
    out = np.zeros((len(op), 21), np.float32)
    L.ref_camera_ops(len(op), _p(op), _p(ar), _p(out))
    return out


# ---------------------------------------------------- legacy Whitted shader --
def whitted(frame, width, height):
    """Assets/Raytracer.comp restated (oracle/whitted_oracle.cpp): returns
    dict(rgba32f, rgba8, stats)."""
    f = np.ascontiguousarray(frame).reshape(())
    rgba = np.zeros((height, width, 4), np.float32)
    u8 = np.zeros((height, width, 4), np.uint8)
    st = OStats()
    lib().oracle_whitted(f.ctypes.data_as(ctypes.c_void_p), width, height, _p(rgba), _p(u8), ctypes.byref(st))
    return {"rgba32f": rgba, "rgba8": u8, "stats": {k: int(getattr(st, k)) for k in STATS_FIELDS}}


def ref_whitted(frame, width, height):
    """The reference's Raytracer.comp compiled for the host (oracle/_ref)."""
    L = ctypes.CDLL(os.path.join(REF_DIR, "libref_whitted.so"))
    L.ref_whitted_render.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_whitted_render.restype = None
    f = np.ascontiguousarray(frame).reshape(())
    rgba = np.zeros((height, width, 4), np.float32)
    u8 = np.zeros((height, width, 4), np.uint8)
    L.ref_whitted_render(f.ctypes.data_as(ctypes.c_void_p), width, height, _p(rgba), _p(u8))
    return rgba, u8
