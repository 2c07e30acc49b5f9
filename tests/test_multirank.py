"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), each with its own seeded
replica batch (weak scaling, no data-path collective), combined by bench.job_rate into the
whole-job throughput (units summed over ranks, time of the slowest rank)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    reps = bench.build_workload(rank, n_rep=4)
    units = float(sum(s.npt for s in reps))
    seconds = 1.0 + rank                      # rank 1 is the slower one
    rate, slowest = bench.job_rate(units, seconds)
    out.put((rank, units, rate, slowest, [s.npt for s in reps], float(reps[0].coor[0, 0])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_job_rate_and_per_rank_batches():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, u0, rate0, t0, n0, x0), (r1, u1, rate1, t1, n1, x1) = res
    assert (r0, r1) == (0, 1)
    assert rate0 == rate1 == pytest.approx((u0 + u1) / 2.0)
    assert t0 == t1 == 2.0
    # each rank has its own seeded replicas (independent units, no exchange)
    assert n0 != n1 or x0 != x1


def test_single_process_job_rate():
    import bench
    assert bench.job_rate(10.0, 2.0) == (5.0, 2.0)
    a = bench.build_workload(0, n_rep=3)
    b = bench.build_workload(0, n_rep=3)
    assert [s.npt for s in a] == [s.npt for s in b]
    assert np.array_equal(a[0].coor, b[0].coor)
