"""bench.py with N > 1 replicas (-m "not gpu"): two gloo ranks on the CPU
check the timing reduction the GPU run uses -- barriers around the timed
region, the slowest rank's time, the whole-job rate over all ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as tmp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import bench
    dist = bench.dist_setup(world)
    bench.barrier(dist)
    t = bench.max_over_ranks(0.5 + rank, dist)   # rank r "took" 0.5 + r seconds
    rate = bench.aggregate_rate(1000.0, world, t)
    bench.barrier(dist)
    out[rank] = (t, rate)
    dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_rank():
    world = 2
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        t, rate = out[r]
        assert t == 1.5
        assert rate == pytest.approx(1000.0 * world / 1.5)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.dist_setup(1) is None
    assert bench.max_over_ranks(2.5, None) == 2.5
    assert bench.aggregate_rate(100.0, 1, 2.0) == 50.0


def test_self_started_replicas_get_one_rank_each():
    """bench.py --gpus N without a launcher starts N workers itself: each
    gets its own RANK / LOCAL_RANK (its GPU), the same WORLD_SIZE and a
    127.0.0.1 rendezvous."""
    sys.path.insert(0, REPO)
    import bench
    envs = [bench.replica_env(r, 4, 29500, base={"PATH": "/bin"}) for r in range(4)]
    assert [e["RANK"] for e in envs] == ["0", "1", "2", "3"]
    assert [e["LOCAL_RANK"] for e in envs] == ["0", "1", "2", "3"]
    assert {e["WORLD_SIZE"] for e in envs} == {"4"}
    assert {e["MASTER_ADDR"] for e in envs} == {"127.0.0.1"}
    assert {e["MASTER_PORT"] for e in envs} == {"29500"}
    assert all(e["PATH"] == "/bin" for e in envs)
