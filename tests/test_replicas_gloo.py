"""Several-GPU runs are independent replicas (no data-path collective); the
host logic that combines them runs here as two gloo ranks on the CPU:
max-over-ranks timing, the whole-job rate, and distinct per-rank workloads."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    from natrix_gb300 import replicas
    from natrix_gb300 import workloads as wl

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "timed" (r + 1) ms for the solver and 10 - r ms end to end
        ms, ms_e2e = replicas.max_over_ranks([rank + 1.0, 10.0 - rank])
        spec = wl.LARGE_2048
        obst = wl.workload_obstacles(replicas.replica_seed(rank), spec)
        forcing = wl.step_forcing(replicas.replica_seed(rank), 0, spec)
        out.put((rank, ms, ms_e2e, obst.tobytes(), forcing.tobytes()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(world):
        r, ms, ms_e2e, obst, forcing = q.get(timeout=120)
        got[r] = (ms, ms_e2e, obst, forcing)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's times
    for r in range(world):
        assert got[r][0] == 2.0 and got[r][1] == 10.0
    # each replica runs its own seeded workload
    assert got[0][2] != got[1][2] and got[0][3] != got[1][3]


def test_whole_job_rate():
    from natrix_gb300 import replicas

    cells, steps = 2048 * 2048, 500
    assert replicas.whole_job_rate(cells * steps, 1, 0.2) == pytest.approx(cells * steps / 0.2)
    assert replicas.whole_job_rate(cells * steps, 4, 0.2) == pytest.approx(4 * cells * steps / 0.2)
    # without a process group the values come back unchanged
    assert replicas.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    assert np.isclose(replicas.replica_seed(3), 3)
