"""The replicas-only multi-GPU path of bench.py, host side, as two gloo processes on the CPU:
every rank gets its own seeded replica (distinct initial fields and noise seeds), the slowest
rank's time counts (all-reduce MAX), and the whole-job throughput scales with the world size.
No GPU and no data-path collective: ranks only exchange their timings."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = dict(bench.workload(bench.parse_args(["--size", "64"])))
        field = bench.initial_field(w, rank)
        seconds = 1.0 + rank  # rank 1 is the slow one
        total, launch = bench.max_over_ranks(tdist, [seconds, 0.1 * (rank + 1)], "cpu")
        value = bench.job_throughput(world, steps=4, inner=10, sites=field.size, seconds=total)
        out[rank] = (float(field[0, 0]), total, launch, value)
    finally:
        tdist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    (f0, t0, l0, v0), (f1, t1, l1, v1) = out[0], out[1]
    assert f0 != f1                       # independent replicas
    assert t0 == t1 == 2.0 and l0 == l1 == pytest.approx(0.2)   # max over ranks, everywhere
    assert v0 == v1 == pytest.approx(2 * 4 * 10 * 64 * 64 / 2.0 / 1e9)


def test_single_process_path_has_no_collective():
    assert bench.max_over_ranks(None, [3.0, 1.0], "cpu") == [3.0, 1.0]
    assert bench.job_throughput(1, 2, 5, 100, 1.0) == pytest.approx(1e-6)
