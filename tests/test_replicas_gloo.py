"""Replica aggregation across ranks (the multi-GPU path of the bench) with
two gloo ranks on CPU: the slowest rank's time, the sum of throughputs."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    from dtcf_gb300 import replicas
    w = replicas.world()
    replicas.barrier()
    t = replicas.max_over_ranks(1.0 + rank)          # rank 1 is the slow one
    s = replicas.sum_over_ranks(10.0 * (rank + 1))
    v = replicas.replica_throughput(12.0, 2.0 + 2.0 * rank)
    q.put((rank, w, t, s, v))
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_time_and_throughput():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, w, t, s, v in out:
        assert w == (2, rank, rank)
        assert t == 2.0 and s == 30.0
        assert v == pytest.approx(24.0 / 4.0)


def test_single_process_is_identity():
    from dtcf_gb300 import replicas
    if dist.is_available() and dist.is_initialized():
        pytest.skip("a process group is active")
    assert replicas.max_over_ranks(3.5) == 3.5 and replicas.sum_over_ranks(2.0) == 2.0
    assert replicas.replica_throughput(8.0, 2.0) == 4.0
