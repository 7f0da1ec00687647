"""CPU tests of bench.py's replicas path with two gloo ranks: the timed value is the maximum over
ranks, and the reference arm runs on rank 0 alone (the other ranks return without work)."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, values, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    try:
        dist.init_process_group("gloo", rank=rank, world_size=2)
        got = bench.max_over_ranks(dist, values[rank], torch.device("cpu"))
        env = bench.dist_env()
        # the reference arm on a rank other than 0: no work, exit status 0
        ref = bench.run_reference(None) if rank == 1 else None
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, got, env, ref))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, repr(e), None, None))


def test_max_over_two_gloo_ranks():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    values = [1.25, 3.5]
    procs = [ctx.Process(target=_rank, args=(r, port, values, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in range(2):
            r, got, env, ref = q.get(timeout=120)
            out[r] = (got, env, ref)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    assert out[0][0] == 3.5 and out[1][0] == 3.5, out
    assert out[0][1] == (2, 0, 0) and out[1][1] == (2, 1, 1)
    assert out[1][2] == 0


def test_single_process_value_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(None, 1.5, None) == 1.5
