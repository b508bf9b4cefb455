import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "vk-renderer_gb300")
ORACLE = os.path.join(REPO, "oracle")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (PKG, ORACLE, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def tracer_lib():
    """Builds (if needed) and loads libtracer.so."""
    from vktrace import _build
    from vktrace.abi import load_library
    _build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu_tracer(tracer_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a GPU")
    from vktrace import Tracer
    t = Tracer(0)
    yield t
    t.close()


def fbits(a):
    """float32 bit patterns with every NaN mapped to one canonical NaN: the
    payload an operation returns for NaN operands depends on the operand
    order a compiler picks for commutative + and *, and carries no meaning."""
    import numpy as np
    a = np.ascontiguousarray(a, np.float32)
    return np.where(np.isnan(a), np.uint32(0x7FC00000), a.view(np.uint32))


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
