"""Serving on several GPUs is independent replicas behind a dispatcher: the
assignment must be deterministic and balanced, every request served exactly once,
and the replicas' statistics merged on every rank.  The multi-rank path runs here
as two gloo processes on the CPU, with a stand-in for the per-rank serving loop."""
import os
import socket
from dataclasses import dataclass

import numpy as np
import pytest

from twoscalesplit_gb300 import dispatch


@dataclass
class _Scene:
    n_low: int


@dataclass
class _Req:
    scene: _Scene
    horizon: int
    arrival_s: float


def _trace(n, seed):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(0.2, n))
    counts = np.exp(rng.uniform(np.log(1000), np.log(500000), n)).astype(int)
    hs = rng.integers(200, 5001, n)
    return [_Req(_Scene(int(c)), int(h), float(a)) for c, h, a in zip(counts, hs, t)]


def _fake_serve(reqs):
    # per-request completion after its own work at 1e9 particle-steps/s
    stats = [{"arrival_s": r.arrival_s, "done_s": r.arrival_s + r.scene.n_low * r.horizon / 1e9, "status": 0,
              "n_low": r.scene.n_low} for r in reqs]
    summary = {"makespan_s": max([s["done_s"] for s in stats], default=0.0), "steps": sum(r.horizon for r in reqs),
               "scene_steps": sum(r.horizon for r in reqs),
               "low_particle_steps": float(sum(r.scene.n_low * r.horizon for r in reqs)), "served": len(reqs),
               "max_active": 1, "mean_active": 1.0}
    return stats, summary


def test_assignment_is_deterministic_and_balanced():
    reqs = _trace(400, 1)
    arr = [r.arrival_s for r in reqs]
    w = [dispatch.request_work(r.scene.n_low, r.horizon) for r in reqs]
    for n in (1, 2, 4, 8):
        a = dispatch.assign(arr, w, n)
        assert np.array_equal(a, dispatch.assign(arr, w, n))
        loads = np.bincount(a, weights=w, minlength=n)
        assert loads.min() > 0.8 * loads.max()  # greedy balance within the largest request
        assert set(a.tolist()) == set(range(n))
    # everything arriving at once still spreads over the replicas
    a = dispatch.assign([0.0] * 64, [1.0] * 64, 4)
    assert np.bincount(a).tolist() == [16, 16, 16, 16]


def test_merge_rejects_duplicates_and_gaps():
    with pytest.raises(ValueError):
        dispatch.merge_stats([([0, 1], [{}, {}]), ([1], [{}])], 2)
    with pytest.raises(ValueError):
        dispatch.merge_stats([([0], [{}])], 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        reqs = _trace(120, 7)
        stats, summary = dispatch.serve_replicated(reqs, _fake_serve, rank, world)
        q.put((rank, [s["arrival_s"] for s in stats], summary))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_serve_every_request_once():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    reqs = _trace(120, 7)
    for rank, arrivals, summary in out:
        assert arrivals == [r.arrival_s for r in reqs]  # merged in trace order, on every rank
        assert summary["served"] == 120
        assert summary["scene_steps"] == sum(r.horizon for r in reqs)
    assert out[0][2] == out[1][2]
