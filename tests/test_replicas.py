"""bench.py's multi-GPU path on CPU: world_size 2 over gloo.

With N GPUs every rank steps its own replica of the vesicle workload (its own
seed) with no exchange, and the job is timed by its slowest rank. The
whole-job value counts the vertices of every rank's set, which differ from
rank to rank. The ranks' hosts run the same reduction helpers bench.py uses
under torchrun, here on CPU tensors."""
from __future__ import annotations

import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    from umcp_gb300 import workloads as W

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        specs = W.vesicle_specs(16, bench.replica_seed(r))
        nv = sum(10 * 4 ** s.level + 2 for s in specs)  # vertices of a level-L icosphere
        seconds = 1.0 + 0.5 * r  # rank 1 is the slower one
        t = bench.over_ranks(seconds, "max", "cpu")
        nv_job = int(bench.over_ranks(nv, "sum", "cpu"))
        q.put((r, w, local, [(s.level, s.radius) for s in specs], nv, t, nv_job))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_time_by_slowest_rank_and_count_every_rank():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, specs0, nv0, t0, job0), (r1, w1, l1, specs1, nv1, t1, job1) = got
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert specs0 != specs1, "each rank steps its own replica set"
    assert t0 == t1 == 1.5, "both ranks see the slowest rank's time"
    assert job0 == job1 == nv0 + nv1, "the whole-job count adds every rank's vertices"
    # the rank-0 set is the single-GPU workload
    sys.path.insert(0, str(ROOT))
    import bench
    from umcp_gb300 import workloads as W

    assert specs0 == [(s.level, s.radius) for s in W.vesicle_specs(16, bench.WORKLOAD["seed"])]
