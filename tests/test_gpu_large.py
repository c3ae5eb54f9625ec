"""Events above 4096 particles (the tiled kernel) vs the CPU oracle (needs a GB300).

Events up to 20k particles, and three at the pile-up workload's sizes (31k,
45k and 60k particles, the oracle on one host thread per event), are checked
against the portable-kinematics oracle bit for bit (merge history with
distances, jets, constituents).  The reference's own grid backend is checked
on 10k-22k-particle events in test_gpu_parity (jets and merge histories).  The
whole 64-event workload and a 100k-particle event are checked through
size-independent properties: momentum conservation per jet from the
constituent map, a complete history, and identical results alone, in a batch
and run twice.
"""
import numpy as np
import pytest

import gpu_util as U
from fastjet_gpu_gb300 import events as E

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    return F.Context(0)


def _pileup(n, seed, axes=4):
    return E.single_event(n, axes, seed=seed, soft_mean=0.6, soft_eta=4.0)


def _one(ctx, ev, algo, radius):
    return ctx.cluster_batch(ev, np.array([0, ev.shape[0]]), algo, radius, history=True, owner=True)


def _check(ctx, ev, algo, radius, tag):
    res = _one(ctx, ev, algo, radius)
    U.compare_event(ev, algo, radius, res["jets"], res["n_jets"][0], res["history"], res["owner"],
                    res["jet_label"], ctx=tag)
    return res


@pytest.mark.parametrize("algo,radius", [(-1, 0.4), (1, 0.6), (0, 0.8), (-1, 0.1), (1, 1.5)])
def test_large_events_bit_exact(ctx, algo, radius):
    for n, seed in ((4097, 1), (5500, 2), (8000, 3)):
        _check(ctx, _pileup(n, seed), algo, radius, f"n={n} algo={algo} R={radius}")


def test_large_event_20k_bit_exact(ctx):
    ev = _pileup(20000, 11, axes=6)
    _check(ctx, ev, -1, 0.4, "20k anti-kt R=0.4")


def test_large_geometry_edges(ctx):
    """Narrow and wide rapidity ranges, rapidities beyond the tiled range,
    a single azimuth tile row, and the tile-count cap."""
    rng = np.random.default_rng(7)
    n = 5000
    pt = rng.exponential(1.0, n) + 0.1
    phi = rng.uniform(-np.pi, np.pi, n)
    narrow = E._massless(pt, rng.uniform(-0.05, 0.05, n), phi)
    far = E._massless(pt, np.concatenate([rng.uniform(-4, 4, n - 40), rng.uniform(16, 30, 20),
                                          rng.uniform(-30, -16, 20)]), phi)
    strip = E._massless(pt, rng.uniform(-4, 4, n), rng.uniform(0.3, 0.35, n))
    cases = [(narrow, -1, 0.4), (far, 1, 0.6), (strip, 0, 0.8), (_pileup(6000, 9), -1, 0.02),
             (_pileup(4500, 10), -1, 3.5)]
    for ci, (ev, algo, radius) in enumerate(cases):
        _check(ctx, ev, algo, radius, f"case {ci}")


def test_large_degenerate(ctx):
    """Repeated particles (one slot is the neighbour of hundreds of others:
    more targets than one pass lists), exact dR ties, zero-pT particles."""
    base = _pileup(4300, 12)
    dup = np.concatenate([base, np.repeat(base[:3], 200, axis=0)])
    zero = base.copy()
    zero[::50, :2] = 0.0
    for algo in (1, 0, -1):
        _check(ctx, dup, algo, 0.4, f"dup algo {algo}")
        _check(ctx, zero, algo, 0.5, f"zero-pt algo {algo}")


def test_mixed_small_and_large_batch(ctx):
    evs = [_pileup(n, 20 + k) for k, n in enumerate((120, 2048, 4097, 5000, 700, 3100, 1, 4096))]
    b = E._batch_from(evs)
    algo = np.array([-1, 1, 0, -1, 1, 0, -1, 1], np.int32)
    radius = np.array([0.4, 0.6, 0.8, 0.4, 1.0, 0.3, 0.4, 0.5])
    res = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True, owner=True)
    for e in range(b.n_events):
        o0, o1 = b.offsets[e], b.offsets[e + 1]
        U.compare_event(b.event(e), int(algo[e]), float(radius[e]), res["jets"][o0:o1], res["n_jets"][e],
                        res["history"][o0:o1], res["owner"][o0:o1], res["jet_label"][o0:o1], ctx=f"event {e}")


def test_plain_and_pseudojet_paths_large(ctx):
    import torch
    import fastjet_gpu_gb300 as F
    ev = _pileup(6000, 30)
    ref = _one(ctx, ev, -1, 0.4)
    one = ctx.cluster_event(torch.from_numpy(ev).cuda(), -1, 0.4, history=True)
    nj = int(one["n_jets"][0])
    assert nj == ref["n_jets"][0]
    assert np.array_equal(one["jets"][:nj].cpu().numpy(), ref["jets"][:nj])
    assert np.array_equal(F.history_records(one["history"][:ev.shape[0]]), ref["history"])
    rec = np.zeros(ev.shape[0], F.PSEUDOJET)
    rec["index"] = np.arange(ev.shape[0])
    rec["px"], rec["py"], rec["pz"], rec["E"] = ev.T
    ctx.cluster_pseudojets(rec, ev.shape[0], F.Algorithm.AntiKt, 0.4)
    assert np.array_equal(np.flatnonzero(rec["isJet"]), np.sort(ref["jet_label"][:nj]))


def _properties(ev, res, e_off=0, n_jets=None, tag=""):
    n = ev.shape[0]
    nj = int(n_jets)
    h = res["history"][e_off:e_off + n]
    assert (h["b"] == -1).sum() == nj, tag
    own = res["owner"][e_off:e_off + n]
    assert own.min() >= 0 and own.max() < nj, tag
    sums = np.zeros((nj, 4))
    np.add.at(sums, own, ev)
    jets = res["jets"][e_off:e_off + nj]
    scale = np.abs(ev).sum(axis=0).max()
    assert np.abs(sums - jets).max() <= 1e-12 * scale, tag


def test_pileup_workload_properties(ctx):
    """A slice of the 10k-60k pile-up workload, anti-kt R=0.4 and kt R=0.6:
    every jet is the sum of its constituents, the history is complete, and
    batch results are identical to the same events run alone and run twice."""
    b = E.pileup_batch(4, 10000, 60000, seed=4)
    for algo, radius in ((-1, 0.4), (1, 0.6)):
        r1 = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True, owner=True)
        r2 = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True, owner=True)
        U.same_results(r1, r2, b.offsets)
        for e in range(b.n_events):
            _properties(b.event(e), r1, b.offsets[e], r1["n_jets"][e], f"event {e} algo {algo}")
        alone = _one(ctx, b.event(1), algo, radius)
        o0, o1 = b.offsets[1], b.offsets[2]
        assert np.array_equal(alone["history"], r1["history"][o0:o1])


def test_very_large_event_properties(ctx):
    """One 100k-particle event (beyond the 10k-60k workload): complete history,
    every jet the sum of its constituents, identical when run twice."""
    ev = _pileup(100000, 40, axes=6)
    r1 = _one(ctx, ev, -1, 0.4)
    r2 = _one(ctx, ev, -1, 0.4)
    U.same_results(r1, r2, [0, ev.shape[0]])
    _properties(ev, r1, 0, r1["n_jets"][0], "100k")


def test_workload_size_events_match_oracle(ctx):
    """Pile-up-like events at the workload's sizes (31k, 45k and 60k
    particles), anti-kt R=0.4 and kt R=0.6: merge history, jets, labels and
    constituents identical bit for bit to the oracle (portable kinematics),
    which clusters the three events on three host threads."""
    import oracle
    evs = E.portable_pileup([31000, 45000, 60000], seed=41)
    b = E._batch_from(evs)
    for algo, radius in ((-1, 0.4), (1, 0.6)):
        res = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True, owner=True)
        hist, jets, lab, own, nj, _ = oracle.cluster_batch(b.particles, b.offsets, algo, radius, threads=3,
                                                           portable=True)
        assert np.array_equal(res["n_jets"], nj)
        assert np.array_equal(res["history"]["a"], hist["a"]) and np.array_equal(res["history"]["b"], hist["b"])
        assert np.array_equal(res["history"]["d"], hist["d"])
        assert np.array_equal(res["owner"], own)
        for e in range(b.n_events):
            o = b.offsets[e]
            assert np.array_equal(res["jets"][o:o + nj[e]], jets[o:o + nj[e]]), (algo, e)
            assert np.array_equal(res["jet_label"][o:o + nj[e]], lab[o:o + nj[e]]), (algo, e)


def test_tile_count_cap_event_matches_oracle(ctx):
    """A 40k-particle pile-up-like event at anti-kt R=0.1 would want ~1,240
    tiles of side 0.2 (32 particles a tile); the tiled kernel keeps at most
    1024 (its tile ranges and summaries live in shared memory) and halves the
    rapidity rows instead.  Merge history, jets and constituents identical bit
    for bit to the oracle (portable kinematics)."""
    import oracle
    b = E._batch_from([E.portable_event(40000, 4, seed=77)])
    res = ctx.cluster_batch(b.particles, b.offsets, -1, 0.1, history=True, owner=True)
    hist, jets, lab, own, nj, _ = oracle.cluster_batch(b.particles, b.offsets, -1, 0.1, threads=1, portable=True)
    assert np.array_equal(res["n_jets"], nj)
    assert np.array_equal(res["history"]["a"], hist["a"]) and np.array_equal(res["history"]["b"], hist["b"])
    assert np.array_equal(res["history"]["d"], hist["d"])
    assert np.array_equal(res["owner"], own)
    assert np.array_equal(res["jets"][:nj[0]], jets[:nj[0]])
    assert np.array_equal(res["jet_label"][:nj[0]], lab[:nj[0]])
