"""The N > 1 logic of bench.py on CPU: two gloo ranks (replicas only, no data
exchange).  Timing reductions take the max over ranks (the slowest replica
sets the step time), throughput sums the rays of all ranks, and the
reference arm runs on rank 0 alone."""
import os
import socket
import sys
from argparse import Namespace
from pathlib import Path

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        mx = bench.allreduce_max(10.0 + rank, world)
        sm = bench.allreduce_sum(4096.0, world)
        ref = bench.run_reference(Namespace(warmup=1, steps=1), rank, world) if rank != 0 else "skipped"
        out.put((rank, mx, sm, ref))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_max_time_and_sum_rays():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]     # max over ranks
    assert [r[2] for r in res] == [8192.0, 8192.0]  # rays of both replicas
    assert res[1][3] is None                        # reference arm: only rank 0 works
