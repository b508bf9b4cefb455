"""The portable cos/sin that fixes the reference RNG's stream (no GPU)."""
import math
from decimal import Decimal, getcontext

import numpy as np
import pytest

from vktrace import scene as S


def _pi_machin(digits=60):
    getcontext().prec = digits + 10

    def atan_inv(n):
        x = Decimal(1) / n
        x2, s, t, k = x * x, Decimal(0), x, 0
        while True:
            term = t / (2 * k + 1)
            if abs(term) < Decimal(10) ** -(digits + 5):
                return s
            s += -term if k % 2 else term
            t *= x2
            k += 1

    return 16 * atan_inv(5) - 4 * atan_inv(239)


def _f32_nearest(d: Decimal) -> float:
    f = np.float32(float(d))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    return float(min(cands, key=lambda c: abs(Decimal(float(c)) - d)))


def test_reduction_constants_are_derived_from_pi():
    """C1, C2, C3 and 2/pi in rng_trig.h are the floats nearest to pi/2, to
    what remains of pi/2 after C1, and after C1 + C2 (pi by Machin's formula)."""
    import re
    import os
    from conftest import REPO
    text = open(os.path.join(REPO, "oracle", "rng_trig.h")).read()

    def const(name):
        m = re.search(name + r"\s+\(?(-?0x[0-9a-fp.+-]+)f\)?", text)
        return float.fromhex(m.group(1))

    pi = _pi_machin()
    half = pi / 2
    c1 = _f32_nearest(half)
    c2 = _f32_nearest(half - Decimal(c1))
    c3 = _f32_nearest(half - Decimal(c1) - Decimal(c2))
    assert const("ORACLE_TRIG_C1") == c1
    assert const("ORACLE_TRIG_C2") == c2
    assert const("ORACLE_TRIG_C3") == c3
    assert const("ORACLE_TRIG_TWO_OVER_PI") == _f32_nearest(2 / pi)
    for n in (2, 4, 6, 8, 10, 12):
        assert const(f"ORACLE_COS_C{n}") == _f32_nearest(Decimal((-1) ** (n // 2)) / math.factorial(n))
    for n in (3, 5, 7, 9, 11):
        assert const(f"ORACLE_SIN_S{n}") == _f32_nearest(Decimal((-1) ** ((n - 1) // 2)) / math.factorial(n))


@pytest.mark.parametrize("lo,hi", [(-4.0, 4.0), (-1e3, 1e3), (1e4, 3e5), (-1e6, -1e5)])
def test_accuracy_against_double(oracle_lib, lo, hi):
    g = S.SplitMix64(int(abs(lo)) + 7)
    xs = g.uniform(4000, lo, hi).astype(np.float32)
    L = oracle_lib.lib()
    c = np.array([L.oracle_cos(float(x)) for x in xs], np.float64)
    s = np.array([L.oracle_sin(float(x)) for x in xs], np.float64)
    ref_c = np.cos(xs.astype(np.float64))
    ref_s = np.sin(xs.astype(np.float64))
    ulp = np.spacing(np.float32(1.0)) / 2  # 2^-24: half-ulp at 1
    # absolute error a few float ulps of 1 (the RNG uses cos in [-1, 1])
    assert np.max(np.abs(c - ref_c)) < 8 * ulp
    assert np.max(np.abs(s - ref_s)) < 8 * ulp


def test_special_values(oracle_lib):
    L = oracle_lib.lib()
    assert math.isnan(L.oracle_cos(float("nan")))
    assert math.isnan(L.oracle_cos(float("inf")))
    assert math.isnan(L.oracle_sin(float("-inf")))
    assert L.oracle_cos(0.0) == 1.0
    assert L.oracle_sin(0.0) == 0.0


def test_rand_in_unit_interval(oracle_lib):
    r = oracle_lib.rand(0.25, 0.5, 3.0, 2000)
    assert (r >= 0).all() and (r < 1).all()
    # roughly uniform
    h, _ = np.histogram(r, bins=10, range=(0, 1))
    assert h.min() > 120
