"""The multi-GPU path of bench.py is replicas: each rank transforms its own
batch, with no collective on the data path; the only exchange is the max of
the step time over ranks.  These tests run that logic as two gloo ranks on the
CPU (the same helpers bench.py calls under torchrun with NCCL)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
        ms = bench.max_over_ranks(local_ms, dist, "cpu")
        rate = bench.whole_job_rate(8, world, ms * 1e-3)
        import numpy as np

        first = float(np.random.default_rng(bench.replica_seed(rank)).normal())
        out[rank] = (ms, rate, first)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    ms0, rate0, x0 = out[0]
    ms1, rate1, x1 = out[1]
    assert ms0 == ms1 == 15.0
    assert rate0 == rate1 == pytest.approx(2 * 8 / 0.015)
    assert x0 != x1  # distinct inputs per replica (weak scaling)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(16, 1, 0.5) == 32.0


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU reference path, no GPU) prints one
    JSON line with the metric, the reference marker, a cpu_baseline and an e2e
    entry without copies (a small band-limit keeps it to seconds)."""
    import json
    import subprocess

    out = subprocess.run([sys.executable, os.path.join(HERE, "..", "bench.py"), "--impl", "reference",
                          "--L", "64", "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=300, check=True).stdout.strip().splitlines()
    d = json.loads(out[-1])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "maps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["L"] == 64
