"""The compressed 8-wide BVH builder, checked on the host (no GPU): node
invariants the device kernel relies on (every index it reads is in range)
and a host emulation of its traversal, whose closest hits must equal a
brute-force scan's (tests/cw8_host_check.cpp)."""
import os
import subprocess

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "vk-renderer_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cw8") / "cw8_host_check")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(REPO, "include"),
           "-I", CSRC, os.path.join(REPO, "tests", "cw8_host_check.cpp"), os.path.join(CSRC, "bvh_build.cpp"),
           os.path.join(CSRC, "bvh_cw8.cpp"), "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("n,extent,sigma,leaf,rays,seed", [
    (100_000, 50.0, 0.5, 4, 1500, 1),   # the c1 soup
    (10_000, 10.0, 0.1, 4, 3000, 3),    # the c3 soup
    (3000, 10.0, 2.0, 1, 2000, 5),      # overlapping triangles, one per leaf
    (5000, 5.0, 1.0, 6, 2000, 6),       # the largest leaf the 8-wide nodes hold
    (1, 1.0, 0.3, 4, 500, 7),           # a root leaf
    (7, 1.0, 0.3, 2, 500, 8),
    (2000, 20.0, 0.5, 8, 10, 9),        # leaves beyond the limit: refused
])
def test_cw8_builder(checker, n, extent, sigma, leaf, rays, seed):
    out = subprocess.run([checker, str(n), str(extent), str(sigma), str(leaf), str(rays), str(seed)],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    line = out.stdout.strip()
    if leaf > 6:
        assert line == "refused", line
    else:
        assert line.startswith("ok"), line
        hits = int(line.split("hits=")[1])
        assert hits > 0 or n < 10, line
