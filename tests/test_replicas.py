"""World-size-2 gloo test of the replicas-only multi-rank path (CPU).

Each rank advances its own seeded replica with the FP64 oracle (the GPU library runs the same
way on its GPU) and the ranks aggregate throughput as total steps / slowest rank.  Replicas are
independent: rank 1's fields differ from rank 0's and equal a single-process run of its seed.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from drd_application_gb300 import abi
    from drd_application_gb300.replicas import replica_seed, replica_throughput
    from drd_application_gb300.workloads import make_case
    from oracle.oracle import Oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    case = make_case("c2", seed=replica_seed(rank), nr=24, nz=12)
    orc = Oracle(case.params)
    st = case.copy_state()
    t = 0.0
    for s in range(2):
        orc.step(st, case.coefs, s == 0, t)
        t += case.params.dt
    secs = 1.0 + rank  # rank 1 is the slowest
    thr, mx = replica_throughput(2, secs, dist)
    dist.barrier()
    out[rank] = (thr, mx, float(st[abi.F_PH].sum()))
    dist.destroy_process_group()


def test_two_rank_replicas_gloo(oracle_build):
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    (thr0, mx0, m0), (thr1, mx1, m1) = out[0], out[1]
    assert thr0 == pytest.approx(4 / 2.0) and thr1 == thr0  # 4 steps in total over max 2 s
    assert mx0 == mx1 == 2.0
    assert m0 != m1  # independent replicas

    # rank 1's replica equals a one-process run of its seed
    from drd_application_gb300 import abi
    from drd_application_gb300.replicas import replica_seed
    from drd_application_gb300.workloads import make_case
    from oracle.oracle import Oracle

    case = make_case("c2", seed=replica_seed(1), nr=24, nz=12)
    orc = Oracle(case.params)
    st = case.copy_state()
    t = 0.0
    for s in range(2):
        orc.step(st, case.coefs, s == 0, t)
        t += case.params.dt
    assert np.isclose(float(st[abi.F_PH].sum()), m1, rtol=0, atol=1e-12)


def test_single_process_throughput():
    from drd_application_gb300.replicas import replica_throughput

    assert replica_throughput(10, 2.0) == (5.0, 2.0)
