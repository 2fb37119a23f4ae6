"""The multi-GPU path of bench.py is replicas only: every rank advances its
own seeded domain, the timed region ends at the slowest rank (max over
ranks) and the job rate counts every rank's steps.  Exercised here with two
gloo ranks on the CPU (no GPU, no data-path collective)."""
import json
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import argparse

    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank                      # this rank's timed region
        ms_max = bench.max_over_ranks(ms, world, device="cpu")
        rate = bench.job_rate(world, 10, ms_max)
        args = argparse.Namespace(n=8, log_var=2.0, corr=2.0, seed=2026, kwh=1000.0)
        case = bench.make_workload(args, rank)   # this rank's replica
        res = {"ms_max": ms_max, "rate": rate, "k_sum": float(np.sum(case.permeab_rock))}
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
        json.dump(res, fh)


def test_replicas_max_over_ranks_and_job_rate(tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r = [json.load(open(tmp_path / f"rank{q}.json")) for q in range(world)]
    assert r[0]["ms_max"] == r[1]["ms_max"] == 15.0          # the slowest rank's time on every rank
    assert r[0]["rate"] == pytest.approx(world * 10 / 0.015)  # whole-job steps per second
    assert r[0]["k_sum"] != r[1]["k_sum"]                     # independent seeded replicas
