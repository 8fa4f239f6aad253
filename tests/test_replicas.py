"""The multi-GPU path of the benchmark is weak-scaling replicas (no exchange
step in the chemistry): every rank integrates its own grid and the only
collective is the max-reduction of the timings. Checked here with two gloo
ranks on the CPU: the reduction gives every rank the slowest rank's time,
the whole-job rate counts every rank's cells, and the ranks' grids differ."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from reprobus_gb300 import inputs
    from reprobus_gb300.replicas import max_over_ranks, replica_seed, whole_job_rate
    ms = 100.0 + 25.0 * rank  # rank 1 is the slower one
    slowest = max_over_ranks(ms)
    case = inputs.make_case("grid", seed=replica_seed(1234, rank), nlon=4, nlat=3, nivbas=94)
    rate = whole_job_rate(case.ncells, world, 3, 3 * slowest * 1e-3)
    out.put((rank, slowest, rate, float(case.qj1[..., 7].sum())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest_and_count_all_cells():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, rate0, ox0), (r1, s1, rate1, ox1) = res
    assert s0 == s1 == 125.0
    cells = 4 * 3 * 94
    assert rate0 == rate1 == pytest.approx(cells * 2 / 0.125)
    assert ox0 != ox1  # each rank integrates its own grid


def test_single_process_needs_no_group():
    from reprobus_gb300.replicas import max_over_ranks
    assert max_over_ranks(3.5) == 3.5
