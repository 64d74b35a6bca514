"""The N > 1 path of bench.py on CPU: two gloo ranks stand in for two GPUs.

With N GPUs bench.py runs N independent replicas of the CCSD iteration (no collective on
the data path). The job's step time is the slowest replica's, taken with one MAX
all-reduce. Its rate is N x the flop of one iteration per step. Only rank 0 prints,
and the reference arm runs on rank 0 alone.
"""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.replica_time(10.0 + 5.0 * rank, world, torch.device("cpu"))
    rate = bench.job_tflops(2.0e12, ms, world)

    class Args:  # the reference arm's arguments; rank 1 must return without work
        steps, warmup, gpus = 1, 3, world

    buf = io.StringIO()
    with redirect_stdout(buf):
        if rank != 0:
            bench.reference_arm(Args, rank)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"ms": ms, "rate": rate, "printed": buf.getvalue()}, f)


def test_replicas_max_time_and_job_rate(tmp_path):
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    for r in res:
        assert r["ms"] == pytest.approx(15.0)             # the slowest replica
        assert r["rate"] == pytest.approx(2 * 2.0e12 / 15e-3 / 1e12)
    assert res[1]["printed"] == ""                        # non-zero ranks print nothing
