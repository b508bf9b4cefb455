"""In-tree build of the CUDA library (libtracer.so) for sm_103a.

Compiles each translation unit with nvcc in parallel and links a shared
library into ``vk-renderer_gb300/_build/``.  No CMake; re-running only
rebuilds objects whose sources changed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtracer.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no multiply-add contraction, so the kernels round exactly as
# the expressions are written (the parity definition); explicit __fmaf_rn
# calls are unaffected.
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall"]

SOURCES = ["tracer_kernels.cu", "tracer_wavefront.cu", "tracer_adjoint.cu", "tracer_edges.cu", "tracer_present.cu",
           "tracer_whitted.cu",
           "tracer_abi.cu", "bvh_build.cpp", "bvh_wide.cpp", "bvh_cw8.cpp", "camera.cpp"]
HEADERS = ["tracer_device.cuh", "tracer_core.cuh", "tracer_traverse.cuh", "tracer_launch.h", "tracer_wavefront.h",
           "tracer_present.h", "tracer_cw8.cuh", "tracer_edges.h",
           "bvh_wide.h", "bvh_cw8.h"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "tracer_abi.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objs.append(obj)
        if not _stale(obj, [path] + hdrs + [os.path.abspath(__file__)]):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCC_FLAGS + (extra_flags or []) + ["-I", INCLUDE, "-I", CSRC, "-c", path, "-o", obj]
        else:
            cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-I", INCLUDE, "-c", path, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB_PATH):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB_PATH] + objs
        run(cmd)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
