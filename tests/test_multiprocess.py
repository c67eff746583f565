"""Multi-rank host logic on CPU (gloo, world size 2): each rank derives its
share of the ensemble without communicating, the shares partition the
instances, and the timing reduction takes the maximum over ranks -- the
pieces bench.py uses under torchrun."""
import os
import socket

import numpy as np
import pytest

from gpusmoldyn_gb300 import sharding

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, counts, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = sharding.my_instances(counts, world, rank)
    load = torch.tensor([float(sum(counts[k] for k in mine))], dtype=torch.float64)
    gathered = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, load)
    t = torch.tensor([float(rank + 1) * 1.5], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, mine, [g.item() for g in gathered], t.item()))
    dist.barrier()
    dist.destroy_process_group()


def test_sharding_partitions_and_balances():
    g = np.random.Generator(np.random.Philox(4))
    counts = [int(c) for c in np.exp(g.uniform(np.log(1e3), np.log(1e6), 256))]
    parts = sharding.balance(counts, 8)
    flat = sorted(k for p in parts for k in p)
    assert flat == list(range(256))
    loads = [sum(counts[k] for k in p) for p in parts]
    assert max(loads) / (sum(counts) / 8) < 1.05
    assert sharding.balance(counts, 1) == [list(range(256))]


def test_two_gloo_ranks_agree_without_communication():
    counts = [5, 100, 7, 60, 3, 3, 40, 90]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, counts, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shares = [r[1] for r in res]
    assert sorted(shares[0] + shares[1]) == list(range(len(counts)))
    assert not set(shares[0]) & set(shares[1])
    # both ranks saw the same per-rank loads and the same max
    assert res[0][2] == res[1][2]
    assert res[0][3] == res[1][3] == 3.0
