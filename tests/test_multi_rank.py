"""Multi-process host logic on CPU (gloo, world size 2): the instance
partition used by the batched workload under torchrun, the reductions of
the step time (max over ranks) and of the work (sum over ranks), and the
reassembly of a sharded batch's per-instance states in global order."""
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


def _host_step(i, n):
    """A deterministic stand-in for advancing instance i (3 n^2 dofs) one step."""
    import numpy as np
    u = np.arange(3 * n * n, dtype=np.float64) * 1e-3 + i
    return 0.75 * u + 0.25 * np.sin(u)


def _batch_worker(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = _multi()
    rng = np.random.default_rng(512)
    ns = rng.choice(np.arange(64, 513, 32), size=24) // 16  # small meshes, the batch's size mix
    mine = m.shard_by_cost([float(n) ** 2 for n in ns], world)[rank]
    states = [_host_step(i, int(ns[i])) for i in mine]
    allst = m.gather_instances(mine, states, len(ns))
    cells = m.sum_over_ranks(sum(int(ns[i]) ** 2 for i in mine))
    q.put((rank, mine, [float(a.sum()) for a in allst], [a.size for a in allst], cells))
    dist.destroy_process_group()


def test_two_ranks_sharded_batch_reassembly():
    """Each gloo rank advances its cost-balanced share of a 24-instance batch
    (a host stand-in for the device step) and the per-instance states come
    back in global instance order on every rank, equal to advancing all
    instances in one process; the summed cell count is the batch's."""
    import numpy as np
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    rng = np.random.default_rng(512)
    ns = rng.choice(np.arange(64, 513, 32), size=24) // 16
    ref = [_host_step(i, int(ns[i])) for i in range(len(ns))]
    (_, s0, sums0, sizes0, c0), (_, s1, sums1, sizes1, c1) = out
    assert sorted(s0 + s1) == list(range(len(ns))) and s0 and s1
    for sums, sizes in ((sums0, sizes0), (sums1, sizes1)):
        assert sizes == [a.size for a in ref]
        assert sums == [float(a.sum()) for a in ref]
    assert c0 == c1 == float(sum(int(n) ** 2 for n in ns))


def test_gather_instances_rejects_double_or_missing_owners():
    m = _multi()
    import numpy as np
    with pytest.raises(ValueError):
        m.gather_instances([0, 0], [np.zeros(1), np.zeros(1)], 2)
    with pytest.raises(ValueError):
        m.gather_instances([0], [np.zeros(1)], 2)
    assert [a[0] for a in m.gather_instances([1, 0], [np.ones(1), np.zeros(1)], 2)] == [0.0, 1.0]
