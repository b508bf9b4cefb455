"""Synthetic workloads with the shapes of the benchmark configurations.

Each workload is a scene (deterministic, from its seed), a FrameData and the
trace parameters.  Data are synthetic stand-ins generated by vktrace.scene's
splitmix64 generator; no dataset is involved.

  ref  the reference's own frame: constant scene (Tracer.comp:186-211) plus
       the uploaded triangle, 1024^2, 4 spp, depth 4, RR every depth, linear
       scan, reference ties, start-up camera (Main.cpp:134-139)
  c0   512^2, 1 spp, depth 2, 64 spheres in [-10,10]^3, r in [0.2,1.5],
       median-split BVH leaf 2, camera (0,0,25) -> origin, vfov 40, seed 0
  c1   1920x1080, 16 spp, depth 8, RR from depth 3, 100k-triangle soup
       (centroids U[-50,50]^3, vertices + N(0,0.5^2)), 256 materials, SAH 16
       bins leaf 4, sky 1.0, seed 1
  c2   64 scenes, triangles log-uniform in [1k, 200k] with c1's geometry,
       resolutions from {128^2, 256^2, 512^2, 1024^2}, 4 spp, depth 6, seed 2
  c3   256^2, 4 spp, depth 4, 10k triangles scaled to [-10,10]^3, 64
       materials, sky 1.0, seed 3 (differentiable)
  c4   1024^2, 64 spp, depth 12, 1M triangles, 1024 materials, seed 4
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import scene as S


@dataclass
class Workload:
    name: str
    scene: S.Scene
    frame: np.ndarray
    width: int
    height: int
    spp: int
    max_depth: int
    rr_start: int
    sky: tuple = (0.0, 0.0, 0.0)
    tie_mode: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def pixels(self) -> int:
        return self.width * self.height


def ref() -> Workload:
    return Workload("ref-1024x1024-4spp-d4-linear", S.reference_scene(), S.reference_frame(0.5), 1024, 1024, 4, 4, 0,
                    tie_mode=0)


def c0(width: int = 512, height: int = 512) -> Workload:
    sc = S.Scene(spheres=S.random_spheres(0, 64), bvh=S.BVH_MEDIAN, leaf_size=2)
    fr = S.frame(S.look_at((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0), width / height, 0.0)
    return Workload("c0-spheres64-512x512-1spp-d2-median", sc, fr, width, height, 1, 2, 0)


C1_CAMERA = ((0.0, 0.0, 120.0), (0.0, 0.0, 0.0), 40.0)


def soup(seed: int, n: int, n_mat: int, extent: float = 50.0, sigma: float = 0.5) -> S.Scene:
    tris, mats = S.triangle_soup(seed, n, extent=extent, sigma=sigma, n_materials=n_mat)
    return S.Scene(triangles=tris, materials=mats, bvh=S.BVH_SAH, leaf_size=4, sah_bins=16)


def c1(width: int = 1920, height: int = 1080, spp: int = 16, n_tris: int = 100_000) -> Workload:
    sc = soup(1, n_tris, 256)
    fr = S.frame(S.look_at(*C1_CAMERA), width / height, 1.0)
    return Workload(f"c1-soup{n_tris // 1000}k-{width}x{height}-{spp}spp-d8-rr3-sah16", sc, fr, width, height, spp, 8,
                    3, sky=(1.0, 1.0, 1.0))


def c2_scene_sizes(seed: int = 2, n: int = 64):
    g = S.SplitMix64(seed)
    lo, hi = math.log(1_000), math.log(200_000)
    tris = np.round(np.exp(lo + (hi - lo) * g.uniform(n))).astype(np.int64)
    res = np.array([128, 256, 512, 1024])[g.integers(n, 4)]
    return tris, res


def c2(n_scenes: int = 64) -> list[Workload]:
    tris, res = c2_scene_sizes(2, n_scenes)
    out = []
    for i in range(n_scenes):
        sc = soup(1000 + i, int(tris[i]), 256)
        fr = S.frame(S.look_at(*C1_CAMERA), 1.0, float(i) / n_scenes)
        out.append(Workload(f"c2-scene{i}", sc, fr, int(res[i]), int(res[i]), 4, 6, 3, sky=(1.0, 1.0, 1.0)))
    return out


C3_CAMERA = ((0.0, 0.0, 25.0), (0.0, 0.0, 0.0), 40.0)


def c3(width: int = 256, n_tris: int = 10_000) -> Workload:
    sc = soup(3, n_tris, 64, extent=10.0, sigma=0.1)
    fr = S.frame(S.look_at(*C3_CAMERA), 1.0, 0.3)
    return Workload(f"c3-soup{n_tris // 1000}k-{width}^2-4spp-d4", sc, fr, width, width, 4, 4, 3, sky=(1.0, 1.0, 1.0))


def c4(width: int = 1024, spp: int = 64, n_tris: int = 1_000_000) -> Workload:
    sc = soup(4, n_tris, 1024)
    fr = S.frame(S.look_at(*C1_CAMERA), 1.0, 0.4)
    return Workload(f"c4-soup{n_tris // 1000}k-{width}^2-{spp}spp-d12", sc, fr, width, width, spp, 12, 3,
                    sky=(1.0, 1.0, 1.0))


WORKLOADS = {"ref": ref, "c0": c0, "c1": c1, "c3": c3, "c4": c4}
