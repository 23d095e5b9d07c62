"""Sharding one ensemble over ranks (rapt_gb300.shard) on the host, no GPU:
the cost-balanced contiguous partition, and with two gloo ranks the gather of
per-shard final states to rank 0, the sum of counters and bench.py's timing
reductions (max over ranks, sums) -- the calls bench.py's own arm makes under
torchrun. The advance of each shard is replaced
by a deterministic host function of the state, which is all the sharding logic
can see of it."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from rapt_gb300 import shard
from rapt_gb300 import workloads as W


def _costs(n=4096):
    w = W.gc_bench(n)
    B = 3.07e-5 * (W.Re / np.linalg.norm(w["pos"], axis=1)) ** 3
    return w, shard.cost_estimate(1, w["pos"], w["v"], w["mass"], w["charge"], B, 1.0)


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_is_contiguous_and_balanced(world):
    _, c = _costs()
    parts = shard.partition(c, world)
    assert parts[0][0] == 0 and parts[-1][1] == len(c)
    assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
    assert all(stop > start for start, stop in parts)
    loads = np.array([c[a:b].sum() for a, b in parts])
    # each shard within one tracer's cost of the even share
    assert np.all(np.abs(loads - c.sum() / world) <= c.max() + 1e-9 * c.sum()), (loads, c.sum() / world)


def test_partition_edge_cases():
    assert shard.partition([], 4) == [(0, 0)]
    assert shard.partition([1.0, 1.0], 1) == [(0, 2)]
    p = shard.partition([0.0] * 5, 5)  # zero cost: one tracer each
    assert p == [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5)]
    p = shard.partition([1.0] * 3 + [100.0], 2)  # one expensive tracer alone
    assert p == [(0, 3), (3, 4)]


def test_cost_model_orders_modes():
    """A particle costs per gyro-period, a guiding centre per transit: the
    cyclotron frequency of a keV proton at 5 Re is far above its transit rate."""
    pos = np.array([[5 * W.Re, 0, 0]] * 2)
    v = np.array([4e5, 4e5])
    c = shard.cost_estimate([0, 1], pos, v, W.m_pr, W.e, 2.5e-7, 10.0)
    assert c[0] > c[1] > 0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _fake_advance(st):
    return {"x": st["x"] * 2.0 + 1.0, "status": np.zeros(len(st["x"]), np.int32),
            "naccept": (np.abs(st["x"][:, 0]).astype(np.int64) % 97) + 1}


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, c = _costs(1000)
        a, b = shard.shard(c, rank, world)
        mine = {"x": w["pos"][a:b] / W.Re}
        out = _fake_advance(mine)
        tot = shard.sum_counters(dist, {"accepted": int(out["naccept"].sum()), "tracers": b - a})
        g = shard.gather(dist, out)
        # bench.py's timing reductions: the slowest rank's time, the summed work
        red = (bench.allmax(dist, 1.0 + rank), bench.allsum(dist, float(b - a)))
        bench.barrier(dist)
        if rank == 0:
            q.put(("ok", g, tot, red))
        else:
            q.put(("rank", g is None, tot, red))
    except Exception as e:  # report instead of hanging the parent
        q.put(("err", repr(e), None, None))
    finally:
        dist.destroy_process_group()


def test_gather_and_counters_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert not any(r[0] == "err" for r in res), res
    ok = [r for r in res if r[0] == "ok"][0]
    other = [r for r in res if r[0] == "rank"][0]
    assert other[1] is True  # only rank 0 receives the gather
    w, _ = _costs(1000)
    ref = _fake_advance({"x": w["pos"] / W.Re})
    g = ok[1]
    assert np.array_equal(g["x"], ref["x"]) and np.array_equal(g["naccept"], ref["naccept"])
    assert ok[2] == other[2] == {"accepted": int(ref["naccept"].sum()), "tracers": 1000}
    assert ok[3] == other[3] == (2.0, 1000.0)
