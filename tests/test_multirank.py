"""The multi-process path of bench.py on CPU (gloo, world size 2, 127.0.0.1): the job time
is the slowest rank's, the whole-job rate counts every replica's units, replicas draw
distinct batches of the same shape, and the reference arm runs on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import numpy as np
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(10.0 * (rank + 1))
        rate = bench.whole_job_rate(bench.N_MATS, world, 5, slowest * 1e-3)
        _, _, _, sizes = bench.make_batch(seed=rank)
        out = io.StringIO()

        class Args:
            gpus, steps, warmup = world, 1, 0
        with redirect_stdout(out):
            if rank != 0:
                bench.run_reference(Args)  # every rank but 0 returns without work
        q.put((rank, slowest, rate, sizes.tolist(), out.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, s0, r0, z0, _), (_, s1, r1, z1, out1) = res
    assert s0 == s1 == 20.0                      # slowest rank's time on every rank
    assert r0 == r1 == 2 * 8192 * 5 / 0.02       # whole-job perms/s
    assert z0 != z1 and len(z0) == len(z1) == 8192  # distinct replicas, same batch size
    assert min(z0) >= 8 and max(z0) <= 24
    assert out1 == ""                            # rank 1 of the reference arm prints nothing


def test_single_process_defaults():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 1, 2, 4.0) == 5.0
