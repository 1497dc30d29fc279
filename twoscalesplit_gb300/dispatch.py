"""Serving on several GPUs: independent replicas behind a dispatcher.

Scenes are independent, so a request stream shards by request with no exchange in
the data path: every rank runs its own pool and serving loop (tss_server_run) on
the requests the dispatcher gives it, and the per-request statistics are gathered
on rank 0 at the end.  The dispatcher is deterministic, so every rank computes the
same assignment from the same trace without communicating.  No counterpart in the
reference (one scene per process, TwoScale2D/WCSPHSolver.cu:2728).
"""
import heapq

import numpy as np


def request_work(n_low, horizon):
    """Expected cost of a request: low-res particle-steps (the step time of a pool is
    proportional to the particles it holds)."""
    return float(n_low) * float(horizon)


def assign(arrivals, works, n_replicas):
    """Replica of each request: in arrival order, the replica with the least work
    assigned so far (ties: lowest rank) -- greedy balancing of the total work, the
    same on every rank."""
    if n_replicas < 1:
        raise ValueError("n_replicas must be >= 1")
    arrivals = np.asarray(arrivals, dtype=np.float64)
    works = np.asarray(works, dtype=np.float64)
    load = [(0.0, r) for r in range(n_replicas)]
    heapq.heapify(load)
    out = np.empty(len(arrivals), dtype=np.int64)
    for k in np.argsort(arrivals, kind="stable"):
        w, r = heapq.heappop(load)
        out[k] = r
        heapq.heappush(load, (w + works[k], r))
    return out


def merge_stats(parts, n):
    """Per-request statistics in trace order from the ranks' (indices, stats) parts;
    every request must appear exactly once."""
    merged = [None] * n
    for idx, stats in parts:
        for k, s in zip(idx, stats):
            if merged[k] is not None:
                raise ValueError(f"request {k} served twice")
            merged[k] = s
    missing = [k for k in range(n) if merged[k] is None]
    if missing:
        raise ValueError(f"requests not served: {missing[:8]}")
    return merged


def merge_summaries(summaries):
    """Run summary of all replicas: makespan the slowest replica's, counts summed."""
    out = {"makespan_s": max(s["makespan_s"] for s in summaries),
           "steps": sum(s["steps"] for s in summaries),
           "scene_steps": sum(s["scene_steps"] for s in summaries),
           "low_particle_steps": sum(s["low_particle_steps"] for s in summaries),
           "served": sum(s["served"] for s in summaries),
           "max_active": max(s["max_active"] for s in summaries)}
    steps = [s["steps"] for s in summaries]
    out["mean_active"] = (sum(s["mean_active"] * s["steps"] for s in summaries) / sum(steps)) if sum(steps) else 0.0
    return out


def gather(obj, group=None):
    """All ranks' `obj` on every rank (torch.distributed, any backend that carries
    objects; a single process returns [obj])."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, obj, group=group)
    return out


def serve_replicated(requests, serve_fn, rank, world, group=None):
    """Run this rank's share of `requests` with serve_fn(list of requests) ->
    (stats, summary) and return the merged (stats, summary) on every rank."""
    arrivals = [r.arrival_s for r in requests]
    works = [request_work(r.scene.n_low, r.horizon) for r in requests]
    who = assign(arrivals, works, world)
    mine = [k for k in range(len(requests)) if who[k] == rank]
    stats, summary = serve_fn([requests[k] for k in mine])
    parts = gather((mine, stats, summary), group)
    merged = merge_stats([(p[0], p[1]) for p in parts], len(requests))
    return merged, merge_summaries([p[2] for p in parts])
