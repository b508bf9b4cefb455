"""ctypes binding of the C ABI (include/tracer_abi.h) and a thin Python
mirror of the reference's per-frame interface.

The library must exist (``vktrace._build.build()`` makes it); there is no
fallback: a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import scene as S
from ._build import LIB_PATH

OK = 0
ERR_NO_SUITABLE_GPU = -1
ERR_NO_SUITABLE_SURFACE = -2
ERR_UNKNOWN = -3
ERR_INVALID_ARG = -4
ERR_OOM = -5
ERR_TIMEOUT = -6
ERR_TRAVERSAL_LIMIT = -7
ERR_STACK_OVERFLOW = -8
ERR_CUDA = -9
ERR_NO_SCENE = -10
ERR_BAD_BVH = -11

TIES_REFERENCE, TIES_STRICT = 0, 1
KERNEL_AUTO, KERNEL_PLAIN, KERNEL_WAVEFRONT = 0, 1, 2
AOV_RGBA8, AOV_RGBA32F, AOV_PRIMARY_HIT, AOV_STATS, AOV_LINEAR = 0, 1, 2, 3, 4
PRIM_TRIANGLE, PRIM_SPHERE = 0, 1

STATS_FIELDS = ["closest_rays", "shadow_rays", "node_fetches", "tri_tests", "sphere_tests", "plane_tests", "hits"]

EXPORTED_SYMBOLS = [
    "tracer_create", "tracer_destroy", "tracer_last_error", "tracer_status_string", "tracer_set_timeout",
    "tracer_upload_scene", "tracer_set_materials", "tracer_trace", "tracer_readback", "tracer_synchronize",
    "tracer_device_image", "tracer_build_bvh", "tracer_validate_bvh", "tracer_set_profiling",
    "tracer_last_timings", "tracer_trace_noalloc", "tracer_upload_scenes", "tracer_trace_batched",
    "tracer_readback_scene", "tracer_trace_adjoint", "tracer_present", "tracer_draw", "tracer_draw_reset",
    "tracer_camera_init", "tracer_camera_init_startup", "tracer_camera_update", "tracer_camera_move",
    "tracer_camera_cursor", "tracer_camera_keys", "tracer_camera_script", "tracer_trace_whitted",
    "tracer_last_rounds", "tracer_measure_l2_read", "tracer_set_traversal_limit", "tracer_set_edge_sampling",
    "tracer_set_adjoint_hit_log",
]
PRESENT_PINGPONG, PRESENT_ACCUMULATE = 0, 1
KEY_W, KEY_S, KEY_A, KEY_D, KEY_R, KEY_F = 1, 2, 4, 8, 16, 32
NOALLOC_MAX_PIXELS = 16384
NOALLOC_MAX_ROUNDS = 8192


class TracerError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("triangles", ctypes.c_void_p), ("num_triangles", ctypes.c_uint32),
        ("materials", ctypes.c_void_p), ("num_materials", ctypes.c_uint32),
        ("spheres", ctypes.c_void_p), ("num_spheres", ctypes.c_uint32),
        ("planes", ctypes.c_void_p), ("num_planes", ctypes.c_uint32),
        ("bvh", ctypes.c_int32), ("leaf_size", ctypes.c_uint32), ("sah_bins", ctypes.c_uint32),
        ("tri_nodes", ctypes.c_void_p), ("num_tri_nodes", ctypes.c_uint32), ("tri_prim_index", ctypes.c_void_p),
        ("sphere_nodes", ctypes.c_void_p), ("num_sphere_nodes", ctypes.c_uint32),
        ("sphere_prim_index", ctypes.c_void_p),
    ]


class TraceParams(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
        ("max_depth", ctypes.c_uint32), ("rr_start", ctypes.c_uint32), ("sky", ctypes.c_float * 3),
        ("tie_mode", ctypes.c_int32), ("kernel", ctypes.c_int32), ("block", ctypes.c_uint32),
        ("stack_depth", ctypes.c_uint32), ("wavefront", ctypes.c_uint32), ("aov_mask", ctypes.c_uint32),
        ("stats", ctypes.c_uint32), ("bvh_width", ctypes.c_uint32), ("tail_paths", ctypes.c_uint32),
    ]


class PresentParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("out_aov", ctypes.c_uint32),
                ("mode", ctypes.c_uint32)]


class CameraController(ctypes.Structure):
    _fields_ = [("data", ctypes.c_float * 16), ("front", ctypes.c_float * 3), ("pitch", ctypes.c_float),
                ("yaw", ctypes.c_float), ("last_mouse", ctypes.c_float * 2), ("light_locked", ctypes.c_uint32),
                ("light_pos", ctypes.c_float * 3)]


class InputFrame(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_float), ("keys", ctypes.c_uint32), ("toggle_light", ctypes.c_uint32),
                ("has_cursor", ctypes.c_uint32), ("cursor_x", ctypes.c_double), ("cursor_y", ctypes.c_double)]


class Timings(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_float), ("extend_ms", ctypes.c_float), ("shade_ms", ctypes.c_float),
                ("rounds", ctypes.c_uint32), ("launches", ctypes.c_uint32), ("finish_ms", ctypes.c_float)]


class RoundInfo(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint32), ("finish", ctypes.c_uint32), ("extend_ms", ctypes.c_float),
                ("shade_ms", ctypes.c_float)]


_lib = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Loads libtracer.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library not built: {p} (run vktrace._build.build())")
    lib = ctypes.CDLL(p)
    vp, u32, i32, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_size_t
    lib.tracer_create.argtypes = [ctypes.POINTER(vp), i32]
    lib.tracer_destroy.argtypes = [vp]
    lib.tracer_destroy.restype = None
    lib.tracer_last_error.argtypes = [vp]
    lib.tracer_last_error.restype = ctypes.c_char_p
    lib.tracer_status_string.argtypes = [i32]
    lib.tracer_status_string.restype = ctypes.c_char_p
    lib.tracer_set_timeout.argtypes = [vp, u32]
    lib.tracer_set_traversal_limit.argtypes = [vp, u32]
    lib.tracer_set_edge_sampling.argtypes = [vp, u32]
    lib.tracer_set_adjoint_hit_log.argtypes = [vp, ctypes.c_uint64]
    lib.tracer_upload_scene.argtypes = [vp, ctypes.POINTER(SceneDesc)]
    lib.tracer_set_materials.argtypes = [vp, vp, u32]
    lib.tracer_trace.argtypes = [vp, vp, ctypes.POINTER(TraceParams), vp]
    lib.tracer_readback.argtypes = [vp, i32, vp, sz]
    lib.tracer_synchronize.argtypes = [vp]
    lib.tracer_device_image.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(sz)]
    lib.tracer_build_bvh.argtypes = [i32, i32, vp, u32, u32, u32, vp, ctypes.POINTER(u32), vp, ctypes.POINTER(u32)]
    lib.tracer_validate_bvh.argtypes = [i32, vp, u32, vp, u32, vp, ctypes.POINTER(u32)]
    lib.tracer_set_profiling.argtypes = [vp, i32]
    lib.tracer_last_timings.argtypes = [vp, ctypes.POINTER(Timings)]
    lib.tracer_last_rounds.argtypes = [vp, ctypes.POINTER(RoundInfo), u32, ctypes.POINTER(u32)]
    lib.tracer_measure_l2_read.argtypes = [vp, sz, u32, ctypes.POINTER(ctypes.c_double)]
    lib.tracer_trace_noalloc.argtypes = [vp, vp, ctypes.POINTER(TraceParams), vp, vp, vp]
    lib.tracer_upload_scenes.argtypes = [vp, ctypes.POINTER(SceneDesc), u32]
    lib.tracer_trace_batched.argtypes = [vp, vp, ctypes.POINTER(TraceParams), u32, i32, vp]
    lib.tracer_readback_scene.argtypes = [vp, u32, i32, vp, sz]
    lib.tracer_trace_adjoint.argtypes = [vp, vp, ctypes.POINTER(TraceParams), vp, vp, vp, vp, vp, vp]
    lib.tracer_present.argtypes = [vp, vp, vp, u32, u32, i32, ctypes.POINTER(PresentParams), vp, sz, vp]
    lib.tracer_draw.argtypes = [vp, vp, ctypes.POINTER(TraceParams), ctypes.POINTER(PresentParams), vp, sz, vp]
    lib.tracer_draw_reset.argtypes = [vp]
    lib.tracer_trace_whitted.argtypes = [vp, vp, ctypes.POINTER(TraceParams), vp]
    pc = ctypes.POINTER(CameraController)
    for fn in ("tracer_camera_init", "tracer_camera_init_startup", "tracer_camera_update"):
        getattr(lib, fn).argtypes = [pc]
        getattr(lib, fn).restype = None
    lib.tracer_camera_move.argtypes = [pc, i32, ctypes.c_float]
    lib.tracer_camera_cursor.argtypes = [pc, ctypes.c_double, ctypes.c_double]
    lib.tracer_camera_cursor.restype = None
    lib.tracer_camera_keys.argtypes = [pc, u32, ctypes.c_float]
    lib.tracer_camera_keys.restype = None
    lib.tracer_camera_script.argtypes = [pc, ctypes.POINTER(InputFrame), u32, vp]
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    return None if a is None or a.size == 0 else a.ctypes.data_as(ctypes.c_void_p)


def build_bvh(kind: int, prims: np.ndarray, leaf_size: int = 0, sah_bins: int = 0):
    """Runs the library's host BVH builder; returns (nodes, prim_index, depth)."""
    lib = load_library()
    prims = np.ascontiguousarray(prims)
    ptype = PRIM_TRIANGLE if prims.dtype == S.TRIANGLE else PRIM_SPHERE
    n = len(prims)
    nodes = np.zeros(max(1, 2 * n), S.BVH_NODE)
    idx = np.zeros(n, np.uint32)
    nn, depth = ctypes.c_uint32(), ctypes.c_uint32()
    r = lib.tracer_build_bvh(kind, ptype, _ptr(prims), n, leaf_size, sah_bins, _ptr(nodes), ctypes.byref(nn),
                             _ptr(idx), ctypes.byref(depth))
    if r != OK:
        raise TracerError(r, lib.tracer_status_string(r).decode())
    return nodes[: nn.value].copy(), idx, depth.value


def validate_bvh(prims: np.ndarray, nodes: np.ndarray, idx: np.ndarray) -> int:
    lib = load_library()
    ptype = PRIM_TRIANGLE if prims.dtype == S.TRIANGLE else PRIM_SPHERE
    depth = ctypes.c_uint32()
    r = lib.tracer_validate_bvh(ptype, _ptr(prims), len(prims), _ptr(nodes), len(nodes), _ptr(idx),
                                ctypes.byref(depth))
    if r != OK:
        raise TracerError(r, lib.tracer_status_string(r).decode())
    return depth.value


class Tracer:
    """One tracer context on one CUDA device (tracer_create .. tracer_destroy)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        r = self.lib.tracer_create(ctypes.byref(h), device)
        if r != OK:
            raise TracerError(r, self.lib.tracer_status_string(r).decode())
        self.h = h
        self.width = self.height = 0
        self._scene_keep = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.tracer_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, r: int):
        if r != OK:
            raise TracerError(r, self.lib.tracer_last_error(self.h).decode())

    def set_timeout(self, ms: int):
        self._check(self.lib.tracer_set_timeout(self.h, ms))

    def set_traversal_limit(self, steps: int):
        """Cap on BVH traversal steps per ray (0 = automatic)."""
        self._check(self.lib.tracer_set_traversal_limit(self.h, steps))

    def set_edge_sampling(self, samples_per_edge: int):
        """Pieces per triangle edge of the camera gradient's boundary part (0 = off, the default)."""
        self._check(self.lib.tracer_set_edge_sampling(self.h, samples_per_edge))

    def set_adjoint_hit_log(self, max_bytes: int):
        """Device memory the wavefront adjoint may keep pass 1's hits in; 0 (the default) = none: pure
        path replay, pass 2 traces again."""
        self._check(self.lib.tracer_set_adjoint_hit_log(self.h, max_bytes))

    @staticmethod
    def _fill_desc(d: SceneDesc, sc: S.Scene, tri_bvh=None, sphere_bvh=None) -> list:
        """Fills a tracer_scene_desc; returns the arrays it points into (keep alive)."""
        arrs = [np.ascontiguousarray(a) for a in (sc.triangles, sc.materials, sc.spheres, sc.planes)]
        d.triangles, d.num_triangles = _ptr(arrs[0]), len(arrs[0])
        d.materials, d.num_materials = _ptr(arrs[1]), len(arrs[1])
        d.spheres, d.num_spheres = _ptr(arrs[2]), len(arrs[2])
        d.planes, d.num_planes = _ptr(arrs[3]), len(arrs[3])
        d.bvh, d.leaf_size, d.sah_bins = sc.bvh, sc.leaf_size, sc.sah_bins
        keep = list(arrs)
        if tri_bvh is not None:
            nodes, idx = np.ascontiguousarray(tri_bvh[0]), np.ascontiguousarray(tri_bvh[1], np.uint32)
            d.tri_nodes, d.num_tri_nodes, d.tri_prim_index = _ptr(nodes), len(nodes), _ptr(idx)
            keep += [nodes, idx]
        if sphere_bvh is not None:
            nodes, idx = np.ascontiguousarray(sphere_bvh[0]), np.ascontiguousarray(sphere_bvh[1], np.uint32)
            d.sphere_nodes, d.num_sphere_nodes, d.sphere_prim_index = _ptr(nodes), len(nodes), _ptr(idx)
            keep += [nodes, idx]
        return keep

    def upload_scene(self, sc: S.Scene, tri_bvh=None, sphere_bvh=None):
        d = SceneDesc()
        keep = self._fill_desc(d, sc, tri_bvh, sphere_bvh)
        self._check(self.lib.tracer_upload_scene(self.h, ctypes.byref(d)))
        del keep

    def upload_scenes(self, scenes: list):
        """tracer_upload_scenes: a batch packed into one device arena."""
        descs = (SceneDesc * len(scenes))()
        keep = [self._fill_desc(descs[i], sc) for i, sc in enumerate(scenes)]
        self._check(self.lib.tracer_upload_scenes(self.h, descs, len(scenes)))
        self.batch_sizes = [None] * len(scenes)
        del keep

    def trace_batched(self, frames: list, params: list, use_graph: bool = True, stream: int | None = None):
        n = len(frames)
        fr = np.zeros(n, S.FRAME)
        for i, f in enumerate(frames):
            fr[i] = np.asarray(f, S.FRAME).reshape(())
        prm = (TraceParams * n)(*params)
        self._check(self.lib.tracer_trace_batched(self.h, fr.ctypes.data_as(ctypes.c_void_p), prm, n,
                                                  1 if use_graph else 0,
                                                  ctypes.c_void_p(stream) if stream else None))
        self.batch_sizes = [(p.width, p.height) for p in params]

    def readback_scene(self, scene: int, aov: int, out: np.ndarray | None = None) -> np.ndarray:
        w, h = self.batch_sizes[scene]
        shape, dt = {AOV_RGBA8: ((h, w, 4), np.uint8), AOV_RGBA32F: ((h, w, 4), np.float32),
                     AOV_PRIMARY_HIT: ((h, w, 2), np.uint32), AOV_STATS: ((len(STATS_FIELDS),), np.uint64)}[aov]
        if out is None:
            out = np.empty(shape, dt)
        self._check(self.lib.tracer_readback_scene(self.h, scene, aov, out.ctypes.data_as(ctypes.c_void_p),
                                                   out.nbytes))
        return out

    def set_materials(self, mats: np.ndarray):
        mats = np.ascontiguousarray(mats, S.MATERIAL)
        self._check(self.lib.tracer_set_materials(self.h, _ptr(mats), len(mats)))

    @staticmethod
    def params(width, height, spp=4, max_depth=4, rr_start=0, sky=(0.0, 0.0, 0.0), tie_mode=TIES_STRICT,
               kernel=KERNEL_AUTO, block=0, stack_depth=0, wavefront=0, aovs=(AOV_RGBA8,), stats=False,
               bvh_width=0, tail_paths=0) -> TraceParams:
        p = TraceParams()
        p.width, p.height, p.spp, p.max_depth, p.rr_start = width, height, spp, max_depth, rr_start
        p.sky = (ctypes.c_float * 3)(*sky)
        p.tie_mode, p.kernel, p.block, p.stack_depth, p.wavefront = tie_mode, kernel, block, stack_depth, wavefront
        p.bvh_width = bvh_width
        p.tail_paths = tail_paths
        m = 0
        for a in aovs:
            m |= 1 << a
        p.aov_mask = m
        p.stats = 1 if stats else 0
        return p

    def trace(self, frame: np.ndarray, params: TraceParams, stream: int | None = None):
        f = np.ascontiguousarray(np.asarray(frame, S.FRAME).reshape(()))
        self._check(self.lib.tracer_trace(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
                                          ctypes.c_void_p(stream) if stream else None))
        self.width, self.height = params.width, params.height

    def trace_noalloc(self, frame: np.ndarray, params: TraceParams, rgba8_dev: int | None,
                      rgba32f_dev: int | None, stream: int | None = None):
        """tracer_trace_noalloc: writes into caller-owned device buffers
        (addresses as ints) and allocates nothing; asynchronous."""
        f = np.ascontiguousarray(np.asarray(frame, S.FRAME).reshape(()))
        self._check(self.lib.tracer_trace_noalloc(
            self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
            ctypes.c_void_p(rgba8_dev) if rgba8_dev else None, ctypes.c_void_p(rgba32f_dev) if rgba32f_dev else None,
            ctypes.c_void_p(stream) if stream else None))

    def synchronize(self):
        self._check(self.lib.tracer_synchronize(self.h))

    def readback(self, aov: int, out: np.ndarray | None = None) -> np.ndarray:
        w, h = self.width, self.height
        if aov == AOV_RGBA8:
            shape, dt = (h, w, 4), np.uint8
        elif aov == AOV_RGBA32F:
            shape, dt = (h, w, 4), np.float32
        elif aov == AOV_PRIMARY_HIT:
            shape, dt = (h, w, 2), np.uint32
        elif aov == AOV_STATS:
            shape, dt = (len(STATS_FIELDS),), np.uint64
        elif aov == AOV_LINEAR:
            shape, dt = (h, w, 4), np.float32
        else:
            raise ValueError(aov)
        if out is None:
            out = np.empty(shape, dt)
        self._check(self.lib.tracer_readback(self.h, aov, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def stats(self) -> dict:
        v = self.readback(AOV_STATS)
        return {k: int(x) for k, x in zip(STATS_FIELDS, v)}

    def trace_adjoint(self, frame: np.ndarray, params: TraceParams, dl_dimage, linear=None, num_materials=None,
                      outputs=None, stream: int | None = None):
        """tracer_trace_adjoint.  dl_dimage / linear: (h, w, 4) float32 numpy
        arrays (host) or device addresses (ints).  Returns host arrays
        (albedo (nm, 3), emission (nm, 3), campos (3,)), or, with outputs =
        (albedo_ptr, emission_ptr, campos_ptr) device addresses, writes there
        asynchronously and returns None."""
        f = np.ascontiguousarray(np.asarray(frame, S.FRAME).reshape(()))

        def ptr(x):
            if x is None:
                return None
            if isinstance(x, int):
                return ctypes.c_void_p(x)
            return np.ascontiguousarray(x, np.float32).ctypes.data_as(ctypes.c_void_p)

        keep = [np.ascontiguousarray(x, np.float32) for x in (dl_dimage, linear) if isinstance(x, np.ndarray)]
        dl = keep[0].ctypes.data_as(ctypes.c_void_p) if isinstance(dl_dimage, np.ndarray) else ptr(dl_dimage)
        ln = None
        if linear is not None:
            ln = keep[-1].ctypes.data_as(ctypes.c_void_p) if isinstance(linear, np.ndarray) else ptr(linear)
        st = ctypes.c_void_p(stream) if stream else None
        if outputs is not None:
            self._check(self.lib.tracer_trace_adjoint(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
                                                      dl, ln, ptr(outputs[0]), ptr(outputs[1]), ptr(outputs[2]), st))
            return None
        nm = num_materials
        ga = np.zeros((nm, 3), np.float32)
        ge = np.zeros((nm, 3), np.float32)
        gc = np.zeros(3, np.float32)
        self._check(self.lib.tracer_trace_adjoint(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params), dl,
                                                  ln, ga.ctypes.data_as(ctypes.c_void_p),
                                                  ge.ctypes.data_as(ctypes.c_void_p),
                                                  gc.ctypes.data_as(ctypes.c_void_p), st))
        return ga, ge, gc

    def set_profiling(self, on: bool):
        self._check(self.lib.tracer_set_profiling(self.h, 1 if on else 0))

    def timings(self) -> dict:
        t = Timings()
        self._check(self.lib.tracer_last_timings(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Timings._fields_}

    def measure_l2_read(self, nbytes: int = 16 << 20, passes: int = 64) -> float:
        """Read bandwidth (GB/s) of an L2-resident buffer, loads bypassing L1."""
        g = ctypes.c_double()
        self._check(self.lib.tracer_measure_l2_read(self.h, nbytes, passes, ctypes.byref(g)))
        return g.value

    def rounds(self) -> np.ndarray:
        """Per-round live paths and kernel times of the last profiled wavefront
        trace (structured array: paths, finish, extend_ms, shade_ms)."""
        n = ctypes.c_uint32()
        self._check(self.lib.tracer_last_rounds(self.h, None, 0, ctypes.byref(n)))
        buf = (RoundInfo * max(n.value, 1))()
        self._check(self.lib.tracer_last_rounds(self.h, buf, n.value, ctypes.byref(n)))
        dt = np.dtype([("paths", np.uint32), ("finish", np.uint32), ("extend_ms", np.float32),
                       ("shade_ms", np.float32)])
        return np.frombuffer(bytes(buf), dt, count=n.value).copy()

    def device_image(self, aov: int):
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(self.lib.tracer_device_image(self.h, aov, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def trace_whitted(self, frame: np.ndarray, params: TraceParams, stream: int | None = None):
        """tracer_trace_whitted: the legacy Raytracer.comp over its own scene."""
        f = np.ascontiguousarray(np.asarray(frame, S.FRAME).reshape(()))
        self._check(self.lib.tracer_trace_whitted(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
                                                  ctypes.c_void_p(stream) if stream else None))
        self.width, self.height = params.width, params.height

    # ------------------------------------------------------ present pass --
    @staticmethod
    def _present_out(width, height, out_aov):
        if out_aov == AOV_RGBA8:
            return np.zeros((height, width, 4), np.uint8)
        return np.zeros((height, width, 4), np.float32)

    def present(self, image0, image1, width: int, height: int, out_aov: int = AOV_RGBA8, out: int | None = None,
                stream: int | None = None):
        """tracer_present over two (h, w, 4) images (uint8 RGBA8 or float32
        RGBA32F numpy arrays, or device addresses with src=(w, h, aov) given
        as image0=(ptr, w, h, aov)).  Returns the framebuffer (row 0 = top), or
        None when out is a device address (asynchronous)."""
        if isinstance(image0, tuple):
            p0, sw, sh, aov = image0
            p1 = image1[0]
            a0, a1 = ctypes.c_void_p(p0), ctypes.c_void_p(p1)
            keep = ()
        else:
            i0, i1 = np.ascontiguousarray(image0), np.ascontiguousarray(image1)
            assert i0.shape == i1.shape and i0.dtype == i1.dtype
            sh, sw = i0.shape[:2]
            aov = AOV_RGBA8 if i0.dtype == np.uint8 else AOV_RGBA32F
            keep = (i0, i1)
            a0, a1 = _ptr(i0), _ptr(i1)
        pp = PresentParams(width, height, out_aov, PRESENT_PINGPONG)
        nbytes = width * height * (4 if out_aov == AOV_RGBA8 else 16)
        st = ctypes.c_void_p(stream) if stream else None
        if out is not None:
            self._check(self.lib.tracer_present(self.h, a0, a1, sw, sh, aov, ctypes.byref(pp), ctypes.c_void_p(out),
                                                nbytes, st))
            return None
        res = self._present_out(width, height, out_aov)
        self._check(self.lib.tracer_present(self.h, a0, a1, sw, sh, aov, ctypes.byref(pp), _ptr(res), nbytes, st))
        del keep
        return res

    def draw(self, frame: np.ndarray, params: TraceParams, width: int, height: int, mode: int = PRESENT_PINGPONG,
             out_aov: int = AOV_RGBA8, out: int | None = None, stream: int | None = None):
        """tracer_draw: trace + present into a width x height framebuffer."""
        f = np.ascontiguousarray(np.asarray(frame, S.FRAME).reshape(()))
        pp = PresentParams(width, height, out_aov, mode)
        nbytes = width * height * (4 if out_aov == AOV_RGBA8 else 16)
        st = ctypes.c_void_p(stream) if stream else None
        if out is not None:
            self._check(self.lib.tracer_draw(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
                                             ctypes.byref(pp), ctypes.c_void_p(out), nbytes, st))
            return None
        res = self._present_out(width, height, out_aov)
        self._check(self.lib.tracer_draw(self.h, f.ctypes.data_as(ctypes.c_void_p), ctypes.byref(params),
                                         ctypes.byref(pp), _ptr(res), nbytes, st))
        self.width, self.height = params.width, params.height
        return res

    def draw_reset(self):
        self._check(self.lib.tracer_draw_reset(self.h))


class Camera:
    """The camera controller of the C ABI (host only; needs the library but
    no GPU): Camera.cpp plus the main loop's input handling."""

    def __init__(self, startup: bool = False, lib: ctypes.CDLL | None = None):
        self.lib = lib or load_library()
        self.c = CameraController()
        (self.lib.tracer_camera_init_startup if startup else self.lib.tracer_camera_init)(ctypes.byref(self.c))

    def update(self):
        self.lib.tracer_camera_update(ctypes.byref(self.c))

    def move(self, direction: int, speed: float):
        r = self.lib.tracer_camera_move(ctypes.byref(self.c), direction, speed)
        if r != OK:
            raise TracerError(r, "bad direction")

    def cursor(self, x: float, y: float):
        self.lib.tracer_camera_cursor(ctypes.byref(self.c), x, y)

    def keys(self, keys: int, dt: float):
        self.lib.tracer_camera_keys(ctypes.byref(self.c), keys, dt)

    def state(self) -> np.ndarray:
        """CameraData (16), front (3), pitch, yaw as float32 (21)."""
        c = self.c
        return np.array(list(c.data) + list(c.front) + [c.pitch, c.yaw], np.float32)

    def camera(self) -> np.ndarray:
        return np.frombuffer(bytes(self.c.data), dtype=S.CAMERA).reshape(()).copy()

    def script(self, inputs, frames: np.ndarray | None = None) -> np.ndarray:
        """inputs: sequence of dicts (dt, keys, toggle_light, cursor=(x, y)
        or None).  Returns n FrameData records (aspect/seed from frames)."""
        n = len(inputs)
        arr = (InputFrame * n)()
        for i, d in enumerate(inputs):
            cur = d.get("cursor")
            arr[i] = InputFrame(d.get("dt", 0.0), d.get("keys", 0), int(d.get("toggle_light", False)),
                                int(cur is not None), cur[0] if cur else 0.0, cur[1] if cur else 0.0)
        out = np.zeros(n, S.FRAME) if frames is None else np.ascontiguousarray(np.array(frames, S.FRAME))
        r = self.lib.tracer_camera_script(ctypes.byref(self.c), arr, n, out.ctypes.data_as(ctypes.c_void_p))
        if r != OK:
            raise TracerError(r, "camera script")
        return out
