"""The multi-GPU path of the benchmark is replicas (each rank advances its own
scene, no collective on the data path): its host logic with two gloo ranks on
the CPU.  The whole-job value is every rank's particle-substeps over the
slowest rank's time, and the reference arm runs on rank 0 alone."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        value, t_max = bench.replica_throughput(torch, times[rank], 1000.0, world, device="cpu")
        ref = bench.run_reference(bench_args()) if rank != 0 else "rank 0"
        out.put((rank, value, t_max, ref))
    finally:
        dist.destroy_process_group()


def bench_args():
    import argparse

    return argparse.Namespace(steps=1, warmup=0, workload="small", gpus=2)


def test_two_replicas_report_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.5, 2.0]  # seconds: rank 1 is the slower
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t_max, ref in results:
        assert t_max == 2.0
        assert value == pytest.approx(2 * 1000.0 / 2.0)  # both ranks' units over the slowest time
        if rank != 0:
            assert ref is None  # the reference arm does no work off rank 0
