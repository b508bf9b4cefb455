"""Host-side checks of the C ABI (no GPU): struct layouts against the
reference's std430 records and the numpy dtypes, exported symbols, and
status strings."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO
from vktrace import abi
from vktrace import scene as S

HEADER = os.path.join(REPO, "include", "tracer_abi.h")

LAYOUT_PROGRAM = r"""
#include <stdio.h>
#include <stddef.h>
#include "tracer_abi.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F))
#define S(T) printf(#T " %zu\n", sizeof(T))
int main(void) {
  S(tracer_camera); P(tracer_camera, pos); P(tracer_camera, dir); P(tracer_camera, right); P(tracer_camera, up);
  S(tracer_frame); P(tracer_frame, aspect_ratio); P(tracer_frame, seed); P(tracer_frame, light_pos);
  P(tracer_frame, camera);
  S(tracer_material); P(tracer_material, albedo); P(tracer_material, emissive); P(tracer_material, roughness);
  P(tracer_material, metalness); P(tracer_material, type);
  S(tracer_sphere); P(tracer_sphere, mat); P(tracer_sphere, P); P(tracer_sphere, r);
  S(tracer_plane); P(tracer_plane, mat); P(tracer_plane, N); P(tracer_plane, len);
  S(tracer_triangle); P(tracer_triangle, v0); P(tracer_triangle, material); P(tracer_triangle, v1);
  P(tracer_triangle, v2);
  S(tracer_bvh_node); P(tracer_bvh_node, bmin); P(tracer_bvh_node, left_or_first); P(tracer_bvh_node, bmax);
  P(tracer_bvh_node, count);
  S(tracer_stats); S(tracer_trace_params); S(tracer_scene_desc); S(tracer_timings);
  S(tracer_present_params); S(tracer_camera_controller); S(tracer_input_frame); S(tracer_round_info);
  P(tracer_camera_controller, front); P(tracer_camera_controller, light_pos); P(tracer_input_frame, cursor_x);
  return 0;
}
"""

# Reference std430 offsets (Assets/Tracer.comp:22-35, :59-74, :102-132, :151-166;
# Include/GraphicsDevice.h:13-29, Include/Camera.h:5-12)
EXPECTED = {
    "tracer_camera": 64, "tracer_camera.pos": 0, "tracer_camera.dir": 16, "tracer_camera.right": 32,
    "tracer_camera.up": 48,
    "tracer_frame": 96, "tracer_frame.aspect_ratio": 0, "tracer_frame.seed": 4, "tracer_frame.light_pos": 16,
    "tracer_frame.camera": 32,
    "tracer_material": 48, "tracer_material.albedo": 0, "tracer_material.emissive": 16,
    "tracer_material.roughness": 28, "tracer_material.metalness": 32, "tracer_material.type": 36,
    "tracer_sphere": 64, "tracer_sphere.mat": 0, "tracer_sphere.P": 48, "tracer_sphere.r": 60,
    "tracer_plane": 64, "tracer_plane.mat": 0, "tracer_plane.N": 48, "tracer_plane.len": 60,
    "tracer_triangle": 48, "tracer_triangle.v0": 0, "tracer_triangle.material": 12, "tracer_triangle.v1": 16,
    "tracer_triangle.v2": 32,
    "tracer_bvh_node": 32, "tracer_bvh_node.bmin": 0, "tracer_bvh_node.left_or_first": 12,
    "tracer_bvh_node.bmax": 16, "tracer_bvh_node.count": 28,
    "tracer_stats": 56,
}


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("layout")
    src = d / "layout.c"
    src.write_text(LAYOUT_PROGRAM)
    exe = d / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_std430_layouts(layout):
    for k, v in EXPECTED.items():
        assert layout[k] == v, k


def test_numpy_dtypes_match_header(layout):
    assert S.CAMERA.itemsize == layout["tracer_camera"]
    assert S.FRAME.itemsize == layout["tracer_frame"]
    assert S.MATERIAL.itemsize == layout["tracer_material"]
    assert S.SPHERE.itemsize == layout["tracer_sphere"]
    assert S.PLANE.itemsize == layout["tracer_plane"]
    assert S.TRIANGLE.itemsize == layout["tracer_triangle"]
    assert S.BVH_NODE.itemsize == layout["tracer_bvh_node"]
    for name, dt in [("tracer_material", S.MATERIAL), ("tracer_sphere", S.SPHERE), ("tracer_plane", S.PLANE),
                     ("tracer_triangle", S.TRIANGLE), ("tracer_bvh_node", S.BVH_NODE), ("tracer_camera", S.CAMERA),
                     ("tracer_frame", S.FRAME)]:
        for field, (fdt, off) in dt.fields.items():
            if field.startswith("_"):
                continue
            assert layout[f"{name}.{field}"] == off, (name, field)
    assert ctypes.sizeof(abi.TraceParams) == layout["tracer_trace_params"]
    assert ctypes.sizeof(abi.SceneDesc) == layout["tracer_scene_desc"]
    assert ctypes.sizeof(abi.Timings) == layout["tracer_timings"]
    assert ctypes.sizeof(abi.PresentParams) == layout["tracer_present_params"]
    assert ctypes.sizeof(abi.CameraController) == layout["tracer_camera_controller"]
    assert ctypes.sizeof(abi.InputFrame) == layout["tracer_input_frame"]
    assert ctypes.sizeof(abi.RoundInfo) == layout["tracer_round_info"]
    assert abi.CameraController.front.offset == layout["tracer_camera_controller.front"]
    assert abi.CameraController.light_pos.offset == layout["tracer_camera_controller.light_pos"]
    assert abi.InputFrame.cursor_x.offset == layout["tracer_input_frame.cursor_x"]


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|void|const char\*)\s+(tracer_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(tracer_lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(tracer_lib, n), n
    assert set(names) == set(abi.EXPORTED_SYMBOLS)


def test_status_strings(tracer_lib):
    for code in range(0, -12, -1):
        s = abi.load_library().tracer_status_string(code).decode()
        assert s and s != "unrecognised status"


def test_create_without_gpu_reports_no_suitable_gpu(tracer_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(abi.TracerError) as e:
        abi.Tracer(0)
    assert e.value.status == abi.ERR_NO_SUITABLE_GPU


def test_bvh_builder_errors(tracer_lib):
    tris, _ = S.triangle_soup(1, 10, extent=5.0)
    with pytest.raises(abi.TracerError):
        abi.build_bvh(7, tris)  # unknown kind
    nodes, idx, depth = abi.build_bvh(S.BVH_SAH, tris)
    bad = nodes.copy()
    bad[0]["left_or_first"] = len(nodes) + 5  # child index out of range
    with pytest.raises(abi.TracerError) as e:
        abi.validate_bvh(tris, bad, idx)
    assert e.value.status == abi.ERR_BAD_BVH
    dup = idx.copy()
    dup[1] = dup[0]  # a primitive referenced twice, another never
    with pytest.raises(abi.TracerError):
        abi.validate_bvh(tris, nodes, dup)
    shrunk = nodes.copy()
    shrunk[0]["bmax"] = shrunk[0]["bmin"]  # root box no longer contains its children
    with pytest.raises(abi.TracerError):
        abi.validate_bvh(tris, shrunk, idx)
    assert abi.validate_bvh(tris, nodes, idx) == depth
