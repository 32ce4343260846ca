"""The multi-GPU path is replicas only: each rank solves its own instance set
(the workload seeded with 20261203 + rank) and the ranks exchange nothing but
the timing and the counts.  Two gloo ranks on the CPU run bench.py's
rendezvous and reductions: the instance sets are disjoint, the time is the
maximum over ranks and the counts add up."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup(world)
    try:
        params, prof = bench.workload(16, 20261203 + r)
        bench.barrier(w)
        t = bench.reduce_max(10.0 + r, w)
        c = bench.reduce_sum(3 + r, w)
        out.put((r, w, local, t, c, [d["alpha"] for d in params], float(prof[0][1, 2])))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_solve_disjoint_instances_and_reduce_timing():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 11.0 for r in res)          # max over ranks
    assert all(r[4] == 7.0 for r in res)           # sum over ranks
    a0, a1 = np.array(res[0][5]), np.array(res[1][5])
    assert a0.shape == a1.shape and len(a0) == 16 and not np.array_equal(a0, a1)   # disjoint draws
