"""Multi-rank benchmark path on CPU: two gloo ranks, 127.0.0.1 rendezvous.

The substep shards only as independent replicas (no data-path collective):
each rank simulates its own cloth and the job's throughput is the total work
divided by the slowest rank's time (bench.replica_throughput).  A rank whose
peer never joins must fail with a timeout instead of hanging."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys
    from datetime import timedelta

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=30))
    ms_mine = 10.0 * (rank + 1)           # rank 1 is the slow one
    value, ms = bench.replica_throughput(1000, ms_mine, world, device="cpu")
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        value, ms = res[rank]
        assert ms == 20.0                   # max over ranks
        assert value == pytest.approx(2 * 1000 / 0.020)


def _lonely(rank, port, q):
    from datetime import timedelta

    import torch.distributed as dist

    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=2,
                                timeout=timedelta(seconds=3))
        q.put("joined")
    except Exception as e:  # noqa: BLE001 - any rendezvous failure is the expected outcome
        q.put(type(e).__name__)


def test_missing_peer_times_out():
    """Rank 0 of a 2-rank job whose peer never starts gets an error on the host,
    not a hang (failure injected on the host: the second rank is never launched)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_lonely, args=(0, _free_port(), q))
    p.start()
    p.join(timeout=60)
    assert not p.is_alive()
    assert q.get(timeout=5) != "joined"


def _shard_worker(rank, world, port, out):
    import sys
    from datetime import timedelta

    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge

    pkg = ge.load_package()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=30))
    insts = pkg.batched_scene(512, seed=0)
    mine = pkg.shard_instances(insts, rank, world)
    counts = [None] * world
    dist.all_gather_object(counts, mine)  # host-side check only: the data path exchanges nothing
    out[rank] = counts
    dist.barrier()
    dist.destroy_process_group()


def test_batched_instances_shard_across_two_ranks():
    """The 512 batched cloths split across 2 gloo ranks: every instance on
    exactly one rank, and the ranks' loads (V + constraints) within 1 % of each
    other (greedy, largest first)."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_shard_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    shards = res[0]
    assert shards == res[1]
    allidx = sorted(shards[0] + shards[1])
    assert allidx == list(range(512))
    insts = pkg.batched_scene(512, seed=0)
    w = [i.x.shape[0] + 3 * i.faces.shape[0] for i in insts]
    loads = [sum(w[i] for i in s) for s in shards]
    assert abs(loads[0] - loads[1]) <= 0.01 * max(loads)
