"""bench.py's N > 1 path on CPU with two gloo ranks: replicas only (one
simulation per rank, distinct seeds), the maximum time over ranks, and the
whole-job aggregate."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, init_method="tcp://127.0.0.1:%d" % port)
    r, w, local = bench.dist_env()
    ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    ms_max = bench.reduce_max_ms(ms, w, "cpu")
    out.put((r, w, local, ms_max, bench.aggregate_value(64, 5, w, ms_max)))
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 20.0 for r in res)  # both ranks see the slower rank's 20 ms
    assert all(abs(r[4] - 64 ** 3 * 5 * 2 / 0.020) < 1e-6 * r[4] for r in res)


def seed_worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world, init_method="tcp://127.0.0.1:%d" % port)
    import torch
    seeds = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(seeds, torch.tensor([bench.replica_seed(1, rank)], dtype=torch.int64))
    out.put((rank, [int(t.item()) for t in seeds]))
    dist.destroy_process_group()


def test_replicas_get_distinct_seeds():
    """Each rank's replica is an independent simulation: the seeds the ranks derive
    (gathered over two gloo ranks) differ, and the aggregate is linear in the ranks."""
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=seed_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seeds = res[0][1]
    assert res[1][1] == seeds and len(set(seeds)) == 2
    assert len({bench.replica_seed(1, r) for r in range(8)}) == 8
    assert bench.aggregate_value(512, 20, 8, 40.0) == 8 * bench.aggregate_value(512, 20, 1, 40.0)
