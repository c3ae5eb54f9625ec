"""Several GPUs = independent ranks over disjoint event sets (no exchange while
clustering).  The host logic is tested here with world_size 2 on gloo, on the
CPU: the per-rank clustering is the oracle (the checker stands in for the GPU
of each rank), so the test checks the split and the gather, not the kernels."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from fastjet_gpu_gb300 import events as E
from fastjet_gpu_gb300 import replicas as R


def test_balance_assigns_every_event_once_and_evenly():
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(50), np.log(2000), 4096)).astype(int)
    for world in (1, 2, 3, 8):
        parts = R.balance(sizes, world)
        allx = np.concatenate(parts)
        assert np.array_equal(np.sort(allx), np.arange(sizes.size))
        loads = np.array([float((sizes[p].astype(float) ** 2).sum()) for p in parts])
        # greedy LPT: no rank exceeds the mean by more than the largest single cost
        assert loads.max() - loads.mean() <= (sizes.astype(float) ** 2).max()
        assert all(np.all(np.diff(p) > 0) for p in parts)


def _oracle_cluster(p, o, algo, radius):
    import oracle
    _, jets, _, _, n_jets, _ = oracle.cluster_batch(p, o, algo, radius, threads=1, want_history=False)
    return jets, n_jets


def _worker(rank, world, port, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        b = E.mixed_batch(40, 20, 400, seed=77)
        out = R.cluster_sharded(b.particles, b.offsets, -1, 0.4, cluster_fn=_oracle_cluster)
        if rank == 0:
            q.put([j.tolist() for j in out])
        else:
            q.put(out)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_gather_gloo_world2():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = [g for g in got if g is not None]
    assert len(res) == 1  # only rank 0 holds the gathered result
    b = E.mixed_batch(40, 20, 400, seed=77)
    jets, n_jets = _oracle_cluster(b.particles, b.offsets, -1, 0.4)
    for e in range(b.n_events):
        o = b.offsets[e]
        assert np.array_equal(np.array(res[0][e]).reshape(-1, 4), jets[o:o + n_jets[e]]), e
