"""N > 1: independent replicas, one per GPU (the path has no exchange step).
The host logic -- disjoint seeds per rank, the max-over-ranks timing and the
whole-job rate -- is checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from zest_gb300.replicas import max_over_ranks, replica_seed0, whole_job_rate
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_seconds = [0.25, 0.75][rank]
    slowest = max_over_ranks(local_seconds, dist, "cpu")
    s0 = replica_seed0(rank, 64)
    dist.barrier()
    q.put((rank, slowest, list(range(s0, s0 + 64)), whole_job_rate(64, world, slowest)))
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=120) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [r[1] for r in res] == [0.75, 0.75]  # every rank sees the slowest rank's time
    assert not set(res[0][2]) & set(res[1][2])  # the ranks' batches are disjoint
    assert res[0][3] == res[1][3] == pytest.approx(2 * 64 / 0.75)
    assert all(p.exitcode == 0 for p in procs)


def test_single_process_has_no_collective():
    sys.path.insert(0, ROOT)
    from zest_gb300.replicas import max_over_ranks, replica_seed0, whole_job_rate
    assert max_over_ranks(0.5) == 0.5
    assert replica_seed0(0, 64) == 1
    assert whole_job_rate(64, 1, 0.5) == 128
