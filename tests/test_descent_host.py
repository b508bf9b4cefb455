"""Gradient descent on albedos (vktrace.descent), host only: Adam updates,
the clamp, and checkpoint/resume giving bit-identical parameters."""
import numpy as np

from vktrace.descent import AlbedoDescent


def _grad(x, target):
    # gradient of a quadratic loss toward `target`, with materials 3 and 5
    # never receiving a gradient (as materials no ray hits)
    g = 2.0 * (x - target)
    g[[3, 5]] = 0.0
    return g


def _run(opt, target, steps):
    for _ in range(steps):
        opt.step(_grad(opt.x, target))
        opt.record(loss=float(np.sum((opt.x - target) ** 2)))
    return opt


def test_descent_converges_and_clamps():
    g = np.random.default_rng(0)
    start = g.uniform(0, 1, (8, 3))
    target = g.uniform(-0.2, 1.2, (8, 3))
    opt = _run(AlbedoDescent(start, lr=0.05), target, 300)
    want = np.clip(target, 1e-3, 1.0)
    moved = np.ones(8, bool)
    moved[[3, 5]] = False
    assert np.abs(opt.x[moved] - want[moved]).max() < 1e-2
    assert (opt.x >= 1e-3).all() and (opt.x <= 1.0).all()
    assert np.array_equal(opt.x[~moved], start[~moved])
    assert opt.seen.tolist() == moved.tolist()


def test_checkpoint_resume_is_bit_identical(tmp_path):
    g = np.random.default_rng(1)
    start = g.uniform(0, 1, (16, 3))
    target = g.uniform(0, 1, (16, 3))
    straight = _run(AlbedoDescent(start, lr=0.01), target, 10)
    path = str(tmp_path / "gd.npz")
    first = _run(AlbedoDescent(start, lr=0.01), target, 4)
    first.save(path)
    resumed = _run(AlbedoDescent.load(path), target, 6)
    assert resumed.t == straight.t == 10
    assert resumed.x.tobytes() == straight.x.tobytes()
    assert resumed.m.tobytes() == straight.m.tobytes() and resumed.v.tobytes() == straight.v.tobytes()
    assert resumed.albedo.dtype == np.float32
    assert resumed.log["loss"] == straight.log["loss"]
    assert resumed.seen.tolist() == straight.seen.tolist()
