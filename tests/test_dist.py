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


def test_reference_arm_line(monkeypatch, capsys):
    """bench.py --impl reference prints exactly one line, JSON with the
    contract's keys (a one-image sample here), and the cross-check of the
    reference's own CPU build against the port where that build exists."""
    import json
    import types
    import bench
    import oracle
    monkeypatch.setattr(bench, "REF_SAMPLE_IMAGES", 1)
    bench.run_reference(types.SimpleNamespace(steps=1, warmup=1), 1, 0)
    out = capsys.readouterr().out.strip().splitlines()
    assert len(out) == 1  # the reference classes' own prints are silenced
    line = json.loads(out[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Mpixel/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["sample"].startswith("first 1 images of the batch")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cc = line["reference_build_crosscheck"]
    if oracle.ref_sources_present():
        assert cc["reference_mpx_s"] > 0 and cc["port_mpx_s"] > 0 and cc["edgels"][0] == cc["edgels"][1]
