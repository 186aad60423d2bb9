"""The N-GPU bench runs independent replicas (no collective on the data
path); the only cross-rank step is the max of the timed durations.  Checked
here with two gloo ranks on the CPU, using bench.py's own helpers."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank          # rank 1 is the slowest
    m = bench.max_over_ranks(ms, world, device="cpu")
    v = bench.replica_throughput(160, world, m)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m, v))


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == pytest.approx(150.0)
        # 160 views per rank, 2 ranks, over the slowest 150 ms
        assert v == pytest.approx(2 * 160 / 0.150)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_throughput(10, 1, 1000.0) == pytest.approx(10.0)
