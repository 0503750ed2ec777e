"""The N > 1 path of bench.py on CPU: two gloo ranks. Under torchrun each
rank runs an independent replica of the workload (the step does not shard);
the timed region is bracketed by barriers, the job time is the slowest
rank's and the value is the cells all ranks updated over that time."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = bench.dist_env()
        bench.rank_barrier(w)
        times = bench.gather_max([0.10 * (rank + 1), 3.0 - rank], w)   # per-step ms, e2e seconds
        bench.rank_barrier(w)
        q.put((r, w, lr, times, bench.replica_rate(1000, 50, times[1], w)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, times, rate) in enumerate(out):
        assert (rank, world, local) == (r, 2, r)
        assert times == pytest.approx([0.2, 3.0])   # maxima over the ranks, the same on both
        assert rate == pytest.approx(2 * 1000 * 50 / 3.0 / 1e6)


def test_single_process_needs_no_process_group():
    import bench
    assert bench.gather_max([1.5, 2.5], 1) == [1.5, 2.5]
    bench.rank_barrier(1)
    assert bench.replica_rate(3_312_000, 200, 0.028, 1) == pytest.approx(3_312_000 * 200 / 0.028 / 1e6)
