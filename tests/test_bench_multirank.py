"""The bench's multi-GPU host logic on CPU: two gloo ranks (weak scaling,
replicas with their own frame seeds; the job's throughput is all ranks' rays
over the slowest rank's time)."""
import os
import socket
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.dist_setup()
    rays = 1000.0 * (rank + 1)       # different frames trace different numbers of rays
    seconds = 0.5 + 0.25 * rank      # rank 1 is the slowest
    value, t, total = bench.aggregate(w, rays, seconds, device="cpu")
    q.put((r, local, value, t, total, bench.rank_seed(0.5, r)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, l0, v0, t0, n0, s0), (r1, l1, v1, t1, n1, s1) = res
    assert (r0, r1) == (0, 1) and (l0, l1) == (0, 1)
    # both ranks agree: (1000 + 2000) rays over max(0.5, 0.75) s
    for v, t, n in ((v0, t0, n0), (v1, t1, n1)):
        assert t == pytest.approx(0.75) and n == pytest.approx(3000.0)
        assert v == pytest.approx(3000.0 / 0.75 / 1e6)
    assert s0 != s1  # every rank its own frame


def test_single_rank_aggregate_has_no_collective():
    sys.path.insert(0, REPO)
    import bench
    v, t, n = bench.aggregate(1, 2e6, 0.5)
    assert v == pytest.approx(4.0) and t == 0.5 and n == 2e6
