"""Multi-rank host logic of bench.py on CPU: world size 2 over gloo.

The detection path shards by image with no collective on the data path
(replicas); the only cross-rank operations are the barrier around the timed
region and the max-over-ranks of the step time.  Each rank draws its own
batch (seeds offset by rank)."""
import os

import pytest


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    ws, r, local = bench.dist_init()
    assert dist.get_backend() == "gloo" or dist.get_backend() == "nccl"
    bench.barrier(ws)
    m = bench.max_over_ranks(float(10 * (rank + 1)), ws)
    # each rank's batch seed range is disjoint
    seed0 = bench.SEED0 + bench.N_IMAGES * r
    q.put((r, m, seed0))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import multiprocessing as mp
    import socket
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("CPU-only test")
    except ImportError:
        pytest.skip("torch missing")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [m for _, m, _ in res] == [20.0, 20.0]
    assert res[0][2] != res[1][2]
