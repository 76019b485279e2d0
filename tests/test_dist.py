"""The N > 1 host path of bench.py on CPU: two gloo ranks (replicas, no collective on the data
path) agree on the barrier, the max-over-ranks time and the whole-job particle count, a rank
other than 0 leaves the reference arm without work, and the ranks' shares of a scene batch and
of a job stream (computed by each rank alone) cover every scene and job exactly once."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        t_max = d.reduce(10.0 + rank, "max")          # per-rank timed region, ms
        n_sum = d.reduce(1000.0 * (rank + 1), "sum")  # particles per rank
        skipped = bench.reference_arm(None, d) if rank != 0 else None
        from vedo_gb300 import partition
        w = [float((q * 7919) % 997 + 1) for q in range(256)]
        scenes = d.gather(partition.pack_scenes(w, world)[rank])
        jobs = d.gather([q for q, r in enumerate(partition.dispatch_stream(w, world)) if r == rank])
        out.put((rank, t_max, n_sum, skipped, scenes, jobs))
    finally:
        d.close()


def test_two_gloo_ranks_reduce_like_the_bench():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, n_sum, skipped, scenes, jobs in res:
        assert t_max == 11.0                           # the slowest rank's time
        assert n_sum == 3000.0                         # whole-job particles
        assert skipped is None
        for share in (scenes, jobs):
            assert len(share) == world
            assert sorted(q for part in share for q in part) == list(range(256))
    assert res[0][4] == res[1][4] and res[0][5] == res[1][5]   # every rank saw the same placement
