"""Replica (N > 1) path of bench.py on CPU: two gloo ranks on 127.0.0.1.

Each rank reports its own timed region; the job's time is the slowest
rank's and the job's fits are the sum over ranks (no data-path collective).
The reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev_s, e2e_s, value, e2e_val = bench.replica_totals(1.0 + rank, 2.0 + 0.5 * rank, 3, 8,
                                                            dist, "cpu")
        out[rank] = (dev_s, e2e_s, value, e2e_val)
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_max_time_and_sum_fits():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        dev_s, e2e_s, value, e2e_val = out[r]
        assert dev_s == 2.0 and e2e_s == 2.5
        assert value == pytest.approx(3 * 8 * 2 / (2.0 / 3600.0))
        assert e2e_val == pytest.approx(3 * 8 * 2 / (2.5 / 3600.0))


def test_single_replica_without_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_totals(4.0, 5.0, 2, 8) == (4.0, 5.0, 16 / (4.0 / 3600.0),
                                                   16 / (5.0 / 3600.0))


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    from coherit_gb300.configs import WORKLOADS

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(None, WORKLOADS["c2"]) is None
