"""The request server (continuous batching) on a GB300.

Each result must be identical -- merge history, jets, labels, constituents --
to the same event clustered alone, whatever else is in flight, whatever the
order of arrival and completion, and under back-pressure from a small arena.
"""
import numpy as np
import pytest

from fastjet_gpu_gb300 import events as E

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    c = F.Context(0)
    yield c
    c.close()


def _alone(ctx, ev, algo, radius):
    return ctx.cluster_batch(ev, np.array([0, ev.shape[0]]), algo, radius, history=True, owner=True)


def _same(ctx, got, ev, algo, radius, tag):
    ref = _alone(ctx, ev, algo, radius)
    nj = int(ref["n_jets"][0])
    assert got["status"] == 0, tag
    assert got["n_jets"] == nj, tag
    assert np.array_equal(got["jets"], ref["jets"][:nj]), tag
    assert np.array_equal(got["jet_label"], ref["jet_label"][:nj]), tag
    if "history" in got:
        assert np.array_equal(got["history"], ref["history"]), tag
        assert np.array_equal(got["owner"], ref["owner"]), tag


def _drive(srv, events, algo, radius, per_poll=7, seed=0):
    """Submit in bursts with polls in between; return results by event index."""
    rng = np.random.default_rng(seed)
    tickets, results = {}, {}
    i = 0
    while i < len(events) or srv.pending:
        for _ in range(int(rng.integers(1, per_poll + 1))):
            if i < len(events):
                tickets[srv.submit(events[i], int(algo[i]), float(radius[i]))] = i
                i += 1
        for r in srv.poll(64, timeout_us=int(rng.integers(0, 300))):
            results[tickets[r["ticket"]]] = r
    return results


def test_server_results_equal_alone_in_the_mix(ctx):
    import fastjet_gpu_gb300 as F
    batch, algo, radius = E.serving_mix(240, seed=11, hi=9000)
    events = [batch.event(e) for e in range(batch.n_events)] + [np.zeros((0, 4))]
    algo = np.append(algo, -1)
    radius = np.append(radius, 0.4)
    srv = F.Server(ctx, arena_particles=1 << 20, history=True)
    try:
        res = _drive(srv, events, algo, radius)
    finally:
        srv.close()
    assert sorted(res) == list(range(len(events)))
    for e, ev in enumerate(events):
        if ev.shape[0] == 0:
            assert res[e]["n_jets"] == 0
            continue
        _same(ctx, res[e], ev, int(algo[e]), float(radius[e]), f"event {e} n={ev.shape[0]}")


def test_server_back_pressure(ctx):
    """An arena of 12k particles, 6 slots, 2 streams, micro-batches of 3:
    requests wait for space, launch as others finish, results unchanged."""
    import fastjet_gpu_gb300 as F
    batch, algo, radius = E.serving_mix(60, seed=12, hi=6000)
    events = [batch.event(e) for e in range(batch.n_events)]
    srv = F.Server(ctx, arena_particles=12000, max_inflight=6, streams=2, max_batch=3, history=True)
    try:
        res = _drive(srv, events, algo, radius, per_poll=20, seed=3)
    finally:
        srv.close()
    for e, ev in enumerate(events):
        _same(ctx, res[e], ev, int(algo[e]), float(radius[e]), f"event {e}")


def test_server_rejects_bad_requests(ctx):
    import fastjet_gpu_gb300 as F
    srv = F.Server(ctx, arena_particles=5000)
    try:
        ev = E.single_event(100, 2, seed=1)
        with pytest.raises(F.FjgError) as ei:
            srv.submit(E.single_event(6000, 2, seed=2), -1, 0.4)
        assert ei.value.status == 4
        bad = ev.copy()
        bad[3, 2] = np.nan
        for args in ((bad, -1, 0.4), (ev, 2, 0.4), (ev, -1, -0.4), (ev, -1, float("nan"))):
            with pytest.raises(F.FjgError) as ei:
                srv.submit(*args)
            assert ei.value.status == 1
        t = srv.submit(ev, -1, 0.4)
        got = []
        while len(got) < 1:
            got += srv.poll(4, timeout_us=100000)
        assert got[0]["ticket"] == t
        _same(ctx, got[0], ev, -1, 0.4, "after rejections")
    finally:
        srv.close()


def test_server_replay_open_loop(ctx):
    import fastjet_gpu_gb300 as F
    batch, algo, radius = E.serving_mix(400, seed=13, hi=5000)
    rng = np.random.default_rng(5)
    arrival = np.cumsum(rng.exponential(1e6 / 20000.0, batch.n_events))
    srv = F.Server(ctx)
    try:
        lat, wall = srv.replay(batch.particles, batch.offsets, algo, radius, arrival)
        assert srv.pending == 0
        # continuous batching: at least one launch, at most one per request
        assert 1 <= srv.launches <= batch.n_events
    finally:
        srv.close()
    assert lat.shape == (batch.n_events,) and np.all(lat > 0)
    assert wall >= arrival[-1]


def test_server_poisoned_request_fails_alone(ctx):
    """With the momenta checked on the GPU (device_check), a request with a
    NaN or infinite component reaches the kernels: it completes with FJG_EINVAL
    and no jets, while the requests launched in the same micro-batches -- small
    and tiled alike -- complete as if it were not there, and the server keeps
    serving.  The fault is injected on the host (bad input); nothing faults."""
    import fastjet_gpu_gb300 as F
    batch, algo, radius = E.serving_mix(40, seed=14, hi=7000)
    events = [batch.event(e).copy() for e in range(batch.n_events)]
    sizes = np.array([ev.shape[0] for ev in events])
    small = int(np.flatnonzero(sizes <= 2048)[0])
    large = int(np.flatnonzero(sizes > 4096)[0])
    events[small][1, 0] = np.nan
    events[large][-1, 3] = np.inf
    srv = F.Server(ctx, history=True, device_check=True, max_batch=64)
    try:
        res = _drive(srv, events, algo, radius, per_poll=40, seed=4)
        again = _drive(srv, [batch.event(0)], algo[:1], radius[:1])
    finally:
        srv.close()
    for e, ev in enumerate(events):
        if e in (small, large):
            assert res[e]["status"] == 1 and res[e]["n_jets"] == 0, e
            continue
        _same(ctx, res[e], ev, int(algo[e]), float(radius[e]), f"event {e}")
    _same(ctx, again[0], batch.event(0), int(algo[0]), float(radius[0]), "after the poisoned requests")
