"""The N > 1 path of bench.py ("replicas only": every rank runs an independent copy of
the operator workload and the job reports the slowest rank's step time) with two
gloo ranks on the CPU. Each rank applies the oracle operator to its own replica and
the aggregation must match what a single process computes for the same ranks."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench

SETTINGS = {"BOX NX": 2, "BOX NY": 2, "BOX NZ": 2, "BOX DIMX": 2, "BOX DIMY": 2, "BOX DIMZ": 2,
            "BOX BOUNDARY FLAG": 1, "POLYNOMIAL DEGREE": 3, "LAMBDA": 1.0, "MESH JITTER": 0.1}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    o = Oracle(SETTINGS)
    q = np.random.default_rng(rank).uniform(-1, 1, o.Ngather)
    y = o.operator(q)
    ms = 10.0 + 5.0 * rank                  # rank 1 is the slow one
    job_ms = bench.max_over_ranks(ms, dist)
    value = bench.job_throughput(o.Nlocal, world, job_ms)
    out[rank] = (job_ms, value, float(np.linalg.norm(y)), o.Nlocal)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_two_gloo_replicas_aggregate_like_the_bench():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    (ms0, v0, n0, nl), (ms1, v1, n1, _) = out[0], out[1]
    assert ms0 == ms1 == 15.0                # max over ranks
    assert v0 == v1 == pytest.approx(2 * nl / 15e-3 / 1e9)
    assert n0 > 0 and n1 > 0 and n0 != n1    # independent replicas (different inputs)
