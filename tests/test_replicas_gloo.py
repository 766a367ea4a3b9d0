"""The multi-rank host path of bench.py on CPU: two gloo ranks run as
independent replicas joined only by a barrier and a max over ranks of the
timed duration; the whole-job value counts the steps of every rank against the
slowest rank's time, and the reference arm runs on rank 0 alone."""
import json
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank))
    import bench
    reps = bench.Replicas(2, backend="gloo")
    reps.barrier()
    local_ms = 100.0 if rank == 0 else 250.0          # rank 1 is the slow one
    value, ms = reps.throughput(10, local_ms)
    out[rank] = (value, ms, reps.max(float(rank)))
    reps.close()


def test_two_gloo_replicas_take_max_time():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        value, ms, mx = res[r]
        assert ms == 250.0 and mx == 1.0
        assert abs(value - 2 * 10 / 0.25) < 1e-9          # 2 ranks x 10 steps over the slowest 250 ms


def test_reference_arm_rank1_does_no_work(capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench

    class A:
        warmup, steps, workload = 1, 1, "hydro2d-128"
    assert bench.run_reference(A, bench.WORKLOADS["hydro2d-128"], 2, 1) == 0
    assert capsys.readouterr().out == ""


def test_single_rank_replicas_are_local():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    reps = bench.Replicas(1)
    value, ms = reps.throughput(5, 50.0)
    assert ms == 50.0 and abs(value - 100.0) < 1e-12
    reps.close()
