"""The multi-GPU path of bench.py is independent replicas (streams shard
with no exchange step): two `gloo` ranks on the CPU check the pieces that
run under torchrun -- distinct seeds per rank (so replicas never produce the
same numbers), the slowest rank's time, the whole-job value, and the
reference arm printing on rank 0 only."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from mtgp_gb300.params import load_table
    from oracle.bind import Oracle
    seed = bench.replica_seed(rank)
    first = Oracle().gen(load_table("mtgp32_fast_11213")[0], seed=seed).fill(0, 64)
    ms = bench.max_over_ranks(1.0 + rank, world, device="cpu")
    value = bench.job_value(world, 1_000_000_000, ms)
    import io
    import contextlib
    buf = io.StringIO()

    class Args:
        pass
    with contextlib.redirect_stdout(buf):
        if rank != 0:          # the reference arm prints on rank 0 only
            a = Args()
            a.gpus, a.steps, a.warmup = world, 1, 1
            bench.run_reference(a)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, seed, first.tolist(), ms, value, buf.getvalue()))


def test_two_replicas_gloo(orc):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, s0, f0, ms0, v0, out0), (r1, s1, f1, ms1, v1, out1) = res
    assert s0 != s1 and f0 != f1
    assert ms0 == ms1 == 2.0
    assert v0 == v1 == pytest.approx(2 * 1e9 / 2e-3 / 1e9)
    assert out1 == ""
