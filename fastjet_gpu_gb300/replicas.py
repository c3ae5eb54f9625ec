"""Several GPUs: events are independent, so a batch is split across ranks (one
process per GPU) with no exchange during clustering; results meet on one rank.

``balance`` assigns events to ranks greedily by estimated cost (N^2 for an
event of N particles: its merge steps times the active pseudojets each step
scans), largest first onto the least-loaded rank.  ``cluster_sharded`` runs
one rank's share and gathers every rank's jets on ``dst`` with
torch.distributed (NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations

import heapq

import numpy as np


def balance(sizes, world):
    """Event indices per rank: greedy longest-processing-time on N^2 costs.
    Every rank's list is sorted (the order of the input batch)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    cost = sizes.astype(np.float64) ** 2
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for e in np.argsort(-cost, kind="stable"):
        load, r = heapq.heappop(heap)
        out[r].append(int(e))
        heapq.heappush(heap, (load + float(cost[e]), r))
    return [np.sort(np.array(ix, dtype=np.int64)) for ix in out]


def subset(particles, offsets, idx):
    """The CSR sub-batch of events `idx` (particles, offsets)."""
    offsets = np.asarray(offsets, dtype=np.int64)
    sizes = offsets[idx + 1] - offsets[idx]
    sub_off = np.zeros(idx.size + 1, np.int64)
    sub_off[1:] = np.cumsum(sizes)
    parts = np.concatenate([particles[offsets[e]:offsets[e + 1]] for e in idx]) if idx.size else \
        np.zeros((0, 4), np.float64)
    return parts, sub_off


def cluster_sharded(particles, offsets, algo, radius, cluster_fn=None, ctx=None, group=None, dst=0):
    """Cluster this rank's share of a host batch and gather all jets on `dst`.

    Every rank passes the whole batch (particles float64 [total, 4], offsets
    int64 [n_events + 1]).  `cluster_fn(particles, offsets, algo, radius)`
    returns (jets [total, 4], n_jets [n_events]) for a CSR sub-batch; by
    default `ctx.cluster_batch` on this rank's GPU.  Returns, on `dst`, a list
    with each event's jets ([n_jets, 4], promotion order) in batch order, and
    None on the other ranks.
    """
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    offsets = np.asarray(offsets, dtype=np.int64)
    sizes = np.diff(offsets)
    idx = balance(sizes, world)[rank]
    if cluster_fn is None:
        if ctx is None:
            raise ValueError("cluster_sharded needs ctx (a Context on this rank's GPU) or cluster_fn")

        def cluster_fn(p, o, a, r):
            res = ctx.cluster_batch(p, o, a, r)
            return res["jets"], res["n_jets"]
    p, o = subset(particles, offsets, idx)
    jets, n_jets = cluster_fn(p, o, algo, radius)
    mine = {int(e): np.asarray(jets[o[k]:o[k] + n_jets[k]]).copy() for k, e in enumerate(idx)}
    gathered = [None] * world if rank == dst else None
    dist.gather_object(mine, gathered, dst=dst, group=group)
    if rank != dst:
        return None
    merged = {}
    for part in gathered:
        merged.update(part)
    return [merged[e] for e in range(sizes.size)]
