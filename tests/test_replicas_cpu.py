"""The N > 1 path of bench.py is replicas only: each rank runs its own sigma
and the ranks exchange nothing but the slowest time.  World size 2 on the
gloo backend (CPU), rendezvous on 127.0.0.1."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    local = 1.0 + rank  # rank 1 is the slower replica
    t = bench.max_over_ranks(local, ws)
    v = bench.replica_gdets(1_000_000_000, 2, ws, t)
    e = bench.dist_env()
    q.put((rank, t, v, e))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v, e in out:
        assert t == 2.0                 # max over ranks
        assert v == pytest.approx(2.0)  # 2 ranks x 2 steps x 1e9 dets / 2 s
        assert e == (2, rank, rank)


def test_reference_arm_other_ranks_exit_quietly(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, L, N, seed, cpu_seconds = 1, 1, 10, 5, 3, 0.1
    assert bench.reference_arm(A, 2, 1) is None
    assert capsys.readouterr().out == ""
