"""Scene and frame records (std430, byte-compatible with include/tracer_abi.h),
deterministic synthetic scene generators and the camera helper.

Record layouts follow the reference shader and host structs:
  Material  Assets/Tracer.comp:59-74      48 B
  Sphere    Assets/Tracer.comp:102-111    64 B
  Plane     Assets/Tracer.comp:118-125    64 B
  Triangle  Assets/Tracer.comp:127-132, Include/GraphicsDevice.h:13-18   48 B
  Camera    Include/Camera.h:5-12         64 B
  FrameData Include/GraphicsDevice.h:20-29   96 B
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MAT_DIFFUSE = 0
MAT_DIELECTRIC = 1

BVH_NONE, BVH_MEDIAN, BVH_SAH = 0, 1, 2

MATERIAL = np.dtype({
    "names": ["albedo", "_pad0", "emissive", "roughness", "metalness", "type", "_pad1"],
    "formats": [("<f4", 3), "<u4", ("<f4", 3), "<f4", "<f4", "<u4", ("<u4", 2)],
    "offsets": [0, 12, 16, 28, 32, 36, 40], "itemsize": 48})
SPHERE = np.dtype({"names": ["mat", "P", "r"], "formats": [MATERIAL, ("<f4", 3), "<f4"],
                   "offsets": [0, 48, 60], "itemsize": 64})
PLANE = np.dtype({"names": ["mat", "N", "len"], "formats": [MATERIAL, ("<f4", 3), "<f4"],
                  "offsets": [0, 48, 60], "itemsize": 64})
TRIANGLE = np.dtype({"names": ["v0", "material", "v1", "_pad1", "v2", "_pad2"],
                     "formats": [("<f4", 3), "<u4", ("<f4", 3), "<u4", ("<f4", 3), "<u4"],
                     "offsets": [0, 12, 16, 28, 32, 44], "itemsize": 48})
BVH_NODE = np.dtype({"names": ["bmin", "left_or_first", "bmax", "count"],
                     "formats": [("<f4", 3), "<i4", ("<f4", 3), "<i4"],
                     "offsets": [0, 12, 16, 28], "itemsize": 32})
CAMERA = np.dtype({"names": ["pos", "dir", "right", "up"], "formats": [("<f4", 3)] * 4,
                   "offsets": [0, 16, 32, 48], "itemsize": 64})
FRAME = np.dtype({"names": ["aspect_ratio", "seed", "light_pos", "camera"],
                  "formats": ["<f4", "<f4", ("<f4", 3), CAMERA],
                  "offsets": [0, 4, 16, 32], "itemsize": 96})


def material(albedo, emissive=(0.0, 0.0, 0.0), roughness=0.0, metalness=0.0, mtype=MAT_DIFFUSE):
    m = np.zeros((), MATERIAL)
    m["albedo"] = albedo
    m["emissive"] = emissive
    m["roughness"] = roughness
    m["metalness"] = metalness
    m["type"] = mtype
    return m


@dataclass
class Scene:
    """A scene as the C ABI takes it (host arrays, copied on upload)."""
    triangles: np.ndarray = field(default_factory=lambda: np.zeros(0, TRIANGLE))
    materials: np.ndarray = field(default_factory=lambda: np.zeros(0, MATERIAL))
    spheres: np.ndarray = field(default_factory=lambda: np.zeros(0, SPHERE))
    planes: np.ndarray = field(default_factory=lambda: np.zeros(0, PLANE))
    bvh: int = BVH_NONE
    leaf_size: int = 0
    sah_bins: int = 0

    @property
    def num_prims(self) -> int:
        return len(self.triangles) + len(self.spheres) + len(self.planes)


# ----------------------------------------------------------------- camera --
def camera_basis(pos, dir_, vfov_deg: float | None = None) -> np.ndarray:
    """CameraData from a position and view direction, with the basis of
    Source/Camera.cpp:60-63: right = normalize(cross((0,1,0), dir)),
    up = cross(dir, right).  With vfov_deg, right and up are scaled by
    tan(vfov/2) (the reference has no field of view; its ray direction is
    dir + right*tx + up*ty, Tracer.comp:570)."""
    d = np.asarray(dir_, np.float64)
    d = d / np.linalg.norm(d)
    right = np.cross(np.array([0.0, 1.0, 0.0]), d)
    right = right / np.linalg.norm(right)
    up = np.cross(d, right)
    if vfov_deg is not None:
        s = math.tan(math.radians(vfov_deg) / 2.0)
        right = right * s
        up = up * s
    cam = np.zeros((), CAMERA)
    cam["pos"] = pos
    cam["dir"] = d
    cam["right"] = right
    cam["up"] = up
    return cam


def look_at(pos, target, vfov_deg: float) -> np.ndarray:
    return camera_basis(pos, np.asarray(target, np.float64) - np.asarray(pos, np.float64), vfov_deg)


def frame(camera: np.ndarray, aspect: float, seed: float, light_pos=(0.0, 64.0, 0.0)) -> np.ndarray:
    f = np.zeros((), FRAME)
    f["aspect_ratio"] = aspect
    f["seed"] = seed
    f["light_pos"] = light_pos
    f["camera"] = camera
    return f


# ------------------------------------------------------ reference scene --
# The reference shader's constant scene (Assets/Tracer.comp:186-211) and the
# single triangle its host uploads (Source/GraphicsDevice.cpp:817).  The
# values must be these exact numbers: parity with the reference depends on
# them.  tests/golden/ holds the same records read out of the compiled
# reference shader, and tests check this table against them.
def _ref_materials():
    D, G = MAT_DIFFUSE, MAT_DIELECTRIC
    return {
        "matte_white": material((1.0, 1.0, 1.0), (0, 0, 0), 0.3, 0.7, D),
        "matte_red": material((0.75, 0.25, 0.25), (0, 0, 0), 0.4, 0.0, D),
        "matte_green": material((0.25, 0.75, 0.25), (0, 0, 0), 0.4, 0.0, D),
        "matte_blue": material((0.25, 0.25, 0.75), (0, 0, 0), 0.4, 0.0, D),
        "plastic": material((0.25, 0.25, 0.75), (0, 0, 0), 0.3, 0.6, D),
        "mirror": material((1.0, 0.5, 0.5), (0, 0, 0), 0.0, 1.0, D),
        "glass": material((1.0, 1.0, 1.0), (0, 0, 0), 0.42, 0.0, G),
        "light": material((1.0, 1.0, 1.0), (128.0, 128.0, 128.0), 0.6, 0.0, D),
    }


def reference_scene() -> Scene:
    m = _ref_materials()
    sph = np.zeros(4, SPHERE)
    for i, (mat, p, r) in enumerate([("glass", (42.0, 16.0, 12.0), 16.0), ("light", (0.0, 96.0, 0.0), 12.0),
                                     ("mirror", (-32.0, 24.0, 24.0), 24.0), ("plastic", (-24.0, 11.0, -48.0), 11.0)]):
        sph[i]["mat"] = m[mat]
        sph[i]["P"] = p
        sph[i]["r"] = r
    pl = np.zeros(5, PLANE)
    for i, (mat, n, d) in enumerate([("matte_white", (0.0, 1.0, 0.0), 0.0), ("matte_white", (0.0, -1.0, 0.0), 128.0),
                                     ("matte_red", (1.0, 0.0, 0.0), 64.0), ("matte_green", (0.0, 0.0, -1.0), 64.0),
                                     ("matte_blue", (-1.0, 0.0, 0.0), 64.0)]):
        pl[i]["mat"] = m[mat]
        pl[i]["N"] = n
        pl[i]["len"] = d
    tri = np.zeros(1, TRIANGLE)
    tri[0]["v0"] = (10.0, 10.0, 0.0)
    tri[0]["v1"] = (0.0, 20.0, 0.0)
    tri[0]["v2"] = (-10.0, 10.0, 0.0)
    tri[0]["material"] = 0
    mats = np.zeros(1, MATERIAL)
    mats[0] = m["mirror"]  # the material every triangle hit gets (Tracer.comp:386)
    return Scene(triangles=tri, materials=mats, spheres=sph, planes=pl, bvh=BVH_NONE)


REF_CAMERA_POS = (32.8509, 30.6991, -106.389)  # Source/Main.cpp:134
REF_CAMERA_PITCH = 4.44998                     # Source/Main.cpp:136
REF_CAMERA_YAW = -602.79                       # Source/Main.cpp:137
REF_ASPECT = 1024.0 / 768.0                    # swapchain extent, GraphicsDevice.cpp:1260; window Main.cpp:92
REF_RESOLUTION = 1024                          # Source/Main.cpp:112


def reference_camera() -> np.ndarray:
    """The reference's start-up camera (Source/Main.cpp:134-139) through
    Camera::update (Source/Camera.cpp:48-64): glm::radians in float, the C
    library's double cos/sin (the float argument is promoted), products in
    double rounded to float, then glm's float normalize/cross."""
    f = np.float32

    def dot(a, b):
        return f(f(f(a[0] * b[0]) + f(a[1] * b[1])) + f(a[2] * b[2]))

    def normalize(v):
        s = f(f(1.0) / f(np.sqrt(dot(v, v))))
        return [f(v[0] * s), f(v[1] * s), f(v[2] * s)]

    def cross(x, y):
        return [f(f(x[1] * y[2]) - f(y[1] * x[2])), f(f(x[2] * y[0]) - f(y[2] * x[0])),
                f(f(x[0] * y[1]) - f(y[0] * x[1]))]

    deg = f(0.01745329251994329576923690768489)
    pr = float(f(f(REF_CAMERA_PITCH) * deg))
    yr = float(f(f(REF_CAMERA_YAW) * deg))
    front = normalize([f(math.cos(pr) * math.cos(yr)), f(math.sin(pr)), f(math.cos(pr) * math.sin(yr))])
    pos = [f(v) for v in REF_CAMERA_POS]
    d = normalize([f(f(pos[i] + front[i]) - pos[i]) for i in range(3)])
    right = normalize(cross([f(0), f(1), f(0)], d))
    up = cross(d, right)
    cam = np.zeros((), CAMERA)
    cam["pos"] = pos
    cam["dir"] = d
    cam["right"] = right
    cam["up"] = up
    return cam


def reference_frame(seed: float = 0.5, camera: np.ndarray | None = None) -> np.ndarray:
    """FrameData as GraphicsDevice::Draw pushes it (GraphicsDevice.cpp:1258-1262),
    with the per-frame seed fixed instead of rand()/RAND_MAX."""
    return frame(reference_camera() if camera is None else camera, REF_ASPECT, seed, (0.0, 64.0, 0.0))


# ----------------------------------------------------- synthetic scenes --
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """Counter-based splitmix64: value i of a stream is mix(seed + (i+1)*gamma).
    Vectorised, identical on every platform (integer arithmetic only)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.count = 0

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            i = np.arange(self.count + 1, self.count + 1 + n, dtype=np.uint64)
            z = self.state + i * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        self.count += n
        return z

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """Top 24 bits x 2^-24 in [0, 1), scaled to [lo, hi) in float64."""
        u = (self.u64(n) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        """Approximately N(0, 1): Irwin-Hall sum of 12 uniforms minus 6 (exact
        arithmetic, so identical on every platform; variance 1, tails cut at 6)."""
        return self.uniform(12 * n).reshape(n, 12).sum(axis=1) - 6.0

    def integers(self, n: int, k: int) -> np.ndarray:
        return np.minimum((self.uniform(n) * k).astype(np.int64), k - 1)


def random_materials(rng: SplitMix64, n: int) -> np.ndarray:
    """n materials drawn uniformly from {Lambertian, metal, dielectric}:
    albedo U[0,1]^3, metal fuzz U[0,0.5], dielectric IOR 1.5, no emission.
    Mapped onto the reference Material: Lambertian = diffuse, metalness 0,
    roughness 0.5; metal = diffuse, metalness 1 - fuzz, roughness fuzz (the
    shader's jitter lobe scales with 1 - metalness, Tracer.comp:454);
    dielectric = type 1 with the IOR in roughness (Tracer.comp:532, :539)."""
    kind = rng.integers(n, 3)
    alb = rng.uniform(3 * n).reshape(n, 3)
    fuzz = rng.uniform(n, 0.0, 0.5)
    m = np.zeros(n, MATERIAL)
    m["albedo"] = alb
    lam, met, die = kind == 0, kind == 1, kind == 2
    m["type"][die] = MAT_DIELECTRIC
    m["roughness"][lam] = 0.5
    m["roughness"][met] = fuzz[met]
    m["metalness"][met] = 1.0 - fuzz[met]
    m["roughness"][die] = 1.5
    return m


def random_spheres(seed: int, n: int = 64, extent: float = 10.0, rmin: float = 0.2, rmax: float = 1.5) -> np.ndarray:
    rng = SplitMix64(seed)
    c = rng.uniform(3 * n, -extent, extent).reshape(n, 3)
    r = rng.uniform(n, rmin, rmax)
    mats = random_materials(rng, n)
    s = np.zeros(n, SPHERE)
    s["P"] = c
    s["r"] = r
    s["mat"] = mats
    return s


def triangle_soup(seed: int, n: int, extent: float = 50.0, sigma: float = 0.5, n_materials: int = 256):
    """n triangles with centroids U[-extent, extent]^3 and vertices offset from
    the centroid by N(0, sigma^2) per axis; materials assigned uniformly."""
    rng = SplitMix64(seed)
    c = rng.uniform(3 * n, -extent, extent).reshape(n, 1, 3)
    off = rng.normal(9 * n).reshape(n, 3, 3) * sigma
    v = (c + off).astype(np.float32)
    mid = rng.integers(n, n_materials)
    mats = random_materials(rng, n_materials)
    t = np.zeros(n, TRIANGLE)
    t["v0"] = v[:, 0]
    t["v1"] = v[:, 1]
    t["v2"] = v[:, 2]
    t["material"] = mid
    return t, mats
