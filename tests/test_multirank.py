"""The replicas-only multi-GPU path of bench.py on CPU: two gloo ranks
(127.0.0.1) meet in barriers and take the max over ranks of their timings;
the reference arm's non-zero ranks exit without work."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
    import bench
    r, w, dist = bench.dist_setup(backend="gloo")
    bench.barrier(dist)
    m = bench.max_over_ranks(dist, 10.0 * (r + 1))
    # the reference arm: only rank 0 times the CPU restatement
    import argparse
    args = argparse.Namespace(steps=1, warmup=3)
    rc = bench.run_reference(args, r, w, dist) if r != 0 else 0
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, m, rc))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 20.0, 0), (1, 2, 20.0, 0)]
