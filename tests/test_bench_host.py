"""Host-side pieces of bench.py (no GPU): the parity summary that the bench
line carries for the benchmarked frame."""
import numpy as np


def test_bench_parity_summary_flags_mismatch():
    """The bench line's parity summary (its c1 check) counts an id mismatch
    that is not a tie, and reports the float image's RMSE (a planted
    difference on the CPU; no GPU involved)."""
    from bench import parity_summary
    h, w = 8, 6
    base = {"rgba32f": np.ones((h, w, 4), np.float32), "hit_id": np.arange(h * w, dtype=np.uint32).reshape(h, w),
            "hit_t": np.full((h, w), 5.0, np.float32)}
    other = {k: v.copy() for k, v in base.items()}
    other["hit_id"][2, 3] += 1
    other["hit_t"][4, 4] = 5.0 * (1 + 1e-4)
    other["rgba32f"][1, 2, 0] = 2.0
    r = parity_summary(base, other, (0, h, 1))
    assert r["id_mismatch"] == 0 and r["id_ties"] == 1  # same t: a tie
    assert abs(r["max_t_rel"] - 1e-4) < 1e-6
    assert r["rmse"] > 0 and r["column0_nan_equal"]
    other["hit_t"][2, 3] = 7.0
    assert parity_summary(base, other, (0, h, 2))["id_mismatch"] == 1
