"""The multi-rank side of bench.py on CPU: two gloo ranks.

The path does not shard a network: `bench.py --gpus N` runs one replica per
rank with no data-path collective, and only the whole-job figures cross ranks
(the slowest rank's time, every rank's force evaluations).  Under torchrun the
reference arm runs on rank 0 alone.
"""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms, calls = bench.combine_ranks(dist, 100.0 + 50.0 * rank, 1000 + rank)
        ref = bench.run_reference(types.SimpleNamespace(warmup=3, steps=3, cpu_seconds=1.0), rank, world) \
            if rank != 0 else "rank 0 runs it"
        q.put((rank, ms, calls, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_max_time_and_total_calls():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, ms, calls, ref = q.get(timeout=120)
        out[rank] = (ms, calls, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        assert out[rank][0] == 150.0   # the slower rank's time
        assert out[rank][1] == 2001    # both ranks' force evaluations
    assert out[1][2] is None           # the reference arm does no work off rank 0


def test_single_process_combine_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(None, 12.5, 7) == (12.5, 7)
