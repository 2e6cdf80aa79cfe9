"""Multi-process host logic on CPU (gloo, world size 2): the instance
partition used by the batched workload under torchrun, and the reductions of
the step time (max over ranks) and of the work (sum over ranks)."""
from __future__ import annotations

import importlib.util
import os
import socket

import pytest

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pressio-demoapps_gb300")


def _multi():
    spec = importlib.util.spec_from_file_location("pda_multi", os.path.join(PKG, "multi.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_shard_by_cost_is_a_balanced_partition():
    m = _multi()
    import numpy as np
    rng = np.random.default_rng(512)
    costs = list((rng.choice(np.arange(64, 513, 32), size=512) ** 2).astype(float))
    for world in (1, 2, 4, 8):
        shards = m.shard_by_cost(costs, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(512))
        loads = [sum(costs[i] for i in s) for s in shards]
        assert max(loads) - min(loads) <= max(costs)
        assert shards == m.shard_by_cost(costs, world)  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = _multi()
    costs = [float(c) for c in (64, 96, 512, 128, 480, 64, 256, 320)]
    mine = m.shard_by_cost(costs, world)[rank]
    work = sum(costs[i] for i in mine)
    t = m.max_over_ranks(1.0 + rank)
    total = m.sum_over_ranks(work)
    q.put((rank, mine, t, total))
    dist.destroy_process_group()


def test_two_ranks_gloo_reductions():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (r0, s0, t0, w0), (r1, s1, t1, w1) = out
    assert sorted(s0 + s1) == list(range(8)) and not set(s0) & set(s1)
    assert t0 == t1 == 2.0
    assert w0 == w1 == float(64 + 96 + 512 + 128 + 480 + 64 + 256 + 320)
