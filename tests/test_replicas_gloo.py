"""The multi-rank path of the benchmark line on CPU (world_size 2, gloo): the engine does not shard one
grid or one solve across GPUs ("replicas only"), so an N-GPU run is N independent replicas whose
figures combine as the slowest replica's - the job time is the largest rank time, a rate the smallest
rank rate times N (bench.replica_max / bench.replica_min, the reductions bench.py makes over NCCL)."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev = torch.device("cpu")
        ms = 10.0 + 2.5 * rank            # rank 1 is the slow one
        rate = 400.0 - 50.0 * rank
        got_ms = bench.replica_max(ms, world, dist, dev)
        got_rate = bench.replica_min(rate, world, dist, dev)
        q.put((rank, got_ms, got_rate, bench.replica_max(ms, 1, dist, dev)))
    finally:
        dist.destroy_process_group()


def test_replica_figures_combine_as_the_slowest_rank():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, got_ms, got_rate, alone in res:
        assert got_ms == 12.5          # the slowest rank's time, on every rank
        assert got_rate == 350.0       # the slowest rank's rate (bench multiplies it by N)
        assert alone == 10.0 + 2.5 * rank  # one rank: its own figure
