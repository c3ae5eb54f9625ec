"""GPU clustering vs the reference goldens and the CPU oracle (needs a GB300)."""
import collections

import numpy as np
import pytest

import golden_util as G
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


def _batch(evs):
    b = E._batch_from(evs)
    return b.particles, b.offsets


def test_reference_goldens_bit_exact(ctx):
    """Every reference golden case (552, plus 8 of pile-up-like events of
    10k-22k particles from the reference's grid backend): identical jet sets,
    bit for bit."""
    by = collections.defaultdict(list)
    for case in G.cases():
        by[(case[0], case[1], case[2])].append(case)
    n = 0
    for (name, algo, radius), cs in sorted(by.items()):
        evs = G.golden_events(name)
        p4, off = _batch(evs)
        res = ctx.cluster_batch(p4, off, G.ALGO_CODE[algo], float(radius))
        for _, _, _, ev, nj, dg in cs:
            got = res["n_jets"][ev]
            assert got == nj, (name, algo, radius, ev)
            jets = res["jets"][off[ev]:off[ev] + got]
            assert G.jets_digest(jets) == dg, (name, algo, radius, ev)
            n += 1
    assert n == 552 + 8


def test_reference_merge_histories(ctx):
    """The GPU's merge sequence is the reference's own (tri_matrix and grid,
    recorded by their step printfs; tests/golden/ref_history.json), step by
    step up to the order inside ties and near ties (golden_util.
    near_tie_mismatch), for every recorded case: the fixtures, the synthetic
    events and the 10k-22k-particle events; and the distances agree within
    the kinematics tolerance."""
    import oracle
    cases = G.history_cases()
    groups = collections.defaultdict(list)
    for key in cases:
        name, backend, algo, radius = key.split(".", 3)
        groups[(name, algo, radius)].append(key)
    checked = 0
    for (name, algo, radius), keys in sorted(groups.items()):
        evs = G.golden_events(name)
        p4, off = _batch(evs)
        res = ctx.cluster_batch(p4, off, G.ALGO_CODE[algo], float(radius), history=True)
        h = res["history"]
        ohist = oracle.cluster_batch(p4, off, G.ALGO_CODE[algo], float(radius), threads=16, portable=True)[0]
        for key in keys:
            ra, rb, rd = G.reference_history(key, ohist)
            for e in range(len(evs)):
                s0, s1 = off[e], off[e + 1]
                k, _ = G.near_tie_mismatch(h["a"][s0:s1], h["b"][s0:s1], h["d"][s0:s1], ra[s0:s1], rb[s0:s1],
                                           rd[s0:s1])
                assert k < 0, f"{key} event {e}: GPU merge sequence differs from the reference at step {k}"
            np.testing.assert_allclose(h["d"], rd, rtol=U.D_RTOL, atol=0, err_msg=key)
            checked += 1
    assert checked == len(cases)


@pytest.mark.parametrize("algo", [1, 0, -1])
@pytest.mark.parametrize("radius", [0.4, 0.8, 1.0])
def test_history_matches_oracle(ctx, algo, radius):
    b = E.mixed_batch(40, 2, 2048, seed=21 + algo)
    res = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True, owner=True)
    for e in range(b.n_events):
        o0, o1 = b.offsets[e], b.offsets[e + 1]
        args = (b.event(e), algo, radius, res["jets"][o0:o1], res["n_jets"][e], res["history"][o0:o1],
                res["owner"][o0:o1], res["jet_label"][o0:o1])
        U.compare_event(*args, ctx=f"event {e} n={o1 - o0}")
        U.compare_event(*args, ctx=f"libm: event {e} n={o1 - o0}", portable=False)


def test_bucket_boundaries_and_tiny(ctx):
    sizes = [0, 1, 2, 3, 31, 32, 33, 255, 256, 257, 511, 512, 513, 1023, 1024, 1025, 2047, 2048, 2049, 4095, 4096]
    evs = [E.single_event(n, 2, seed=n) if n else np.zeros((0, 4)) for n in sizes]
    p4, off = _batch(evs)
    for algo in (1, 0, -1):
        res = ctx.cluster_batch(p4, off, algo, 0.6, history=True, owner=True)
        for e, n in enumerate(sizes):
            o0, o1 = off[e], off[e + 1]
            U.compare_event(evs[e], algo, 0.6, res["jets"][o0:o1], res["n_jets"][e], res["history"][o0:o1],
                            res["owner"][o0:o1], ctx=f"n={n} algo={algo}")


def test_mixed_algorithms_and_radii_per_event(ctx):
    b, algo, radius = E.serving_mix(60, seed=8, hi=2000)
    res = ctx.cluster_batch(b.particles, b.offsets, algo, radius, history=True)
    for e in range(b.n_events):
        o0, o1 = b.offsets[e], b.offsets[e + 1]
        U.compare_event(b.event(e), int(algo[e]), float(radius[e]), res["jets"][o0:o1], res["n_jets"][e],
                        res["history"][o0:o1], ctx=f"event {e}")


def _symmetric_ladder(k=12):
    """A particle at rapidity 0 between mirrored particles at +-rap_i (phi = 0):
    dR2 to the left and right neighbours tie exactly, whatever the libm."""
    rows = [[1.0, 0.0, 0.0, 1.0]]
    for i in range(1, k + 1):
        s = 0.05 * i ** 1.3
        e = float(np.sqrt(1.0 + s * s))
        rows.append([1.0, 0.0, s, e])
        rows.append([1.0, 0.0, -s, e])
    return np.array(rows)


def test_degenerate_inputs(ctx):
    """Exact ties and special branches.  Against the portable-kinematics oracle
    every case must match bit for bit; against the libm oracle only the cases
    whose tie resolution does not hinge on the last bit of log/atan2."""
    zero_pt = np.array([[0.0, 0.0, 5.0, 5.0], [0.0, 0.0, -3.0, 3.0], [1.0, 0.5, 0.2, 1.2], [0.9, 0.6, 0.1, 1.1],
                        [0.0, 0.0, 0.0, 0.0], [0.0, 0.0, 2.0, 7.0]])
    # widely separated particles: every step promotes (C/A: all at d = 1, lowest label first)
    ring = np.array([[np.cos(t), np.sin(t), 0.0, 1.0] for t in np.linspace(0, 6, 40)])
    dup = np.repeat(E.single_event(20, 1, seed=5), 2, axis=0)  # exact duplicates: dR2 == 0 ties
    massive = E.single_event(300, 3, seed=6)
    massive[:, 3] *= 1.3  # E > |p|
    ladder = _symmetric_ladder()
    # (event, radii robust against libm differences, radii checked only bit-exactly)
    cases = [(zero_pt, (0.05, 0.7), ()), (ring, (0.05,), (0.7, 1.0)), (dup, (0.05, 0.7), ()),
             (massive, (0.05, 0.7), ()), (ladder, (0.3, 1.0), ())]
    for algo in (1, 0, -1):
        for ci, (ev, radii, exact_only) in enumerate(cases):
            for radius in radii + exact_only:
                res = ctx.cluster_batch(ev, np.array([0, ev.shape[0]]), algo, radius, history=True, owner=True)
                args = (ev, algo, radius, res["jets"], res["n_jets"][0], res["history"], res["owner"])
                U.compare_event(*args, ctx=f"case {ci} algo {algo} R {radius}")
                if radius in radii:
                    U.compare_event(*args, ctx=f"libm: case {ci} algo {algo} R {radius}", portable=False)


def test_batch_invariance_and_determinism(ctx):
    b = E.mixed_batch(64, 50, 2000, seed=31)
    r1 = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True)
    r2 = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True)
    U.same_results(r1, r2, b.offsets)
    for e in (0, 7, 63):
        ev = b.event(e)
        alone = ctx.cluster_batch(ev, np.array([0, ev.shape[0]]), -1, 0.4, history=True)
        o0, o1 = b.offsets[e], b.offsets[e + 1]
        assert np.array_equal(alone["jets"][:alone["n_jets"][0]], r1["jets"][o0:o0 + r1["n_jets"][e]])
        assert np.array_equal(alone["history"], r1["history"][o0:o1])


def test_plain_path_matches_batch(ctx):
    import torch
    b = E.mixed_batch(6, 50, 2000, seed=41)
    r = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True)
    for e in range(b.n_events):
        ev = torch.from_numpy(b.event(e)).cuda()
        one = ctx.cluster_event(ev, -1, 0.4, history=True)
        nj = int(one["n_jets"][0])
        o0 = b.offsets[e]
        assert nj == r["n_jets"][e]
        assert np.array_equal(one["jets"][:nj].cpu().numpy(), r["jets"][o0:o0 + nj])


def test_pseudojet_records_in_place(ctx):
    """cluster.h:6 contract on PseudoJet records: jets flagged isJet at their label slot."""
    import fastjet_gpu_gb300 as F
    import oracle
    ev = G.inputs("808_cms")[0]
    rec = np.zeros(ev.shape[0], F.PSEUDOJET)
    rec["index"] = np.arange(ev.shape[0])
    rec["px"], rec["py"], rec["pz"], rec["E"] = ev.T
    ctx.cluster_pseudojets(rec, ev.shape[0], F.Algorithm.AntiKt, 0.4)
    ref = oracle.cluster(ev, -1, 0.4)
    assert rec["isJet"].sum() == len(ref.jets)
    assert np.array_equal(np.flatnonzero(rec["isJet"]), np.sort(ref.jet_label))
    got = np.stack([rec["px"], rec["py"], rec["pz"], rec["E"]], axis=1)[rec["isJet"]]
    assert sorted(map(tuple, got.tolist())) == sorted(map(tuple, ref.jets.tolist()))
    assert np.array_equal(rec["index"], np.arange(ev.shape[0]))


def test_too_big_is_reported(ctx):
    """Events above the largest supported size (2**24 particles) are refused
    on the host before anything is read or launched."""
    import ctypes
    import torch
    import fastjet_gpu_gb300 as F
    small = torch.zeros((8, 4), dtype=torch.float64, device="cuda")
    jets = torch.zeros((8, 4), dtype=torch.float64, device="cuda")
    lab = torch.zeros(8, dtype=torch.int32, device="cuda")
    nj = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = F.lib().fjg_cluster_event(ctx._h, ctypes.c_void_p(small.data_ptr()), F.MAX_EVENT_PARTICLES + 1, -1, 0.4,
                                   ctypes.c_void_p(jets.data_ptr()), ctypes.c_void_p(lab.data_ptr()),
                                   ctypes.c_void_p(nj.data_ptr()), None, None)
    assert st == 4
    ev = E.single_event(100, 2, seed=1)
    ctx.cluster_batch(ev, np.array([0, 100]), -1, 0.4)  # the context stays usable


def test_host_entry_preallocated_outputs(ctx):
    """cluster_batch(out=...) fills the caller's (page-locked) arrays with the
    same results, and rejects arrays of the wrong dtype or length."""
    import torch
    b = E.mixed_batch(30, 50, 1500, seed=51)
    ref = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True)
    total = int(b.offsets[-1])
    out = {"jets": torch.empty((total, 4), dtype=torch.float64).pin_memory().numpy(),
           "jet_label": torch.empty(total, dtype=torch.int32).pin_memory().numpy(),
           "n_jets": torch.empty(b.n_events, dtype=torch.int32).pin_memory().numpy()}
    got = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True, out=out)
    assert np.array_equal(got["n_jets"], ref["n_jets"])
    assert np.array_equal(got["history"], ref["history"])
    for e in range(b.n_events):  # rows past an event's jet count are not written
        o, nj = b.offsets[e], ref["n_jets"][e]
        assert np.array_equal(got["jets"][o:o + nj], ref["jets"][o:o + nj]), e
        assert np.array_equal(got["jet_label"][o:o + nj], ref["jet_label"][o:o + nj]), e
    assert got["jets"].ctypes.data == out["jets"].ctypes.data
    with pytest.raises(ValueError):
        ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, out={"jets": np.zeros((total, 4), np.float32)})
    with pytest.raises(ValueError):
        ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, out={"n_jets": np.zeros(b.n_events - 1, np.int32)})


def test_non_finite_momenta_are_refused(ctx):
    """An event with a NaN or infinite momentum component is refused on the
    device (no jets, FJG_EINVAL); the other events of the batch are clustered
    as usual.  The same for the one-event path."""
    import torch
    import fastjet_gpu_gb300 as F
    b = E.mixed_batch(12, 20, 600, seed=61)
    clean = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True)
    bad_p = b.particles.copy()
    bad_p[b.offsets[3] + 1, 2] = np.nan
    bad_p[b.offsets[7], 3] = np.inf
    with pytest.raises(F.FjgError):
        ctx.cluster_batch(bad_p, b.offsets, -1, 0.4)
    p4 = torch.from_numpy(bad_p).cuda()
    off = torch.from_numpy(b.offsets).cuda()
    out = ctx.cluster_batch_device(p4, off, -1, 0.4, history=True)
    torch.cuda.synchronize()
    with pytest.raises(F.FjgError):
        ctx.check()
    nj = out["n_jets"].cpu().numpy()
    jets = out["jets"].cpu().numpy()
    assert nj[3] == 0 and nj[7] == 0
    for e in range(b.n_events):
        if e in (3, 7):
            continue
        o = b.offsets[e]
        assert nj[e] == clean["n_jets"][e]
        assert np.array_equal(jets[o:o + nj[e]], clean["jets"][o:o + nj[e]])
    one = torch.from_numpy(bad_p[b.offsets[3]:b.offsets[4]].copy()).cuda()
    with pytest.raises(F.FjgError):
        ctx.cluster_event(one, -1, 0.4)
    ctx.cluster_batch(b.particles, b.offsets, -1, 0.4)  # the context stays usable


def test_zero_radius(ctx):
    """R = 0, which the reference driver accepts (main.cc:159): 1/R^2 is
    infinite, so every particle is promoted, in order of weight, by the batch,
    one-event and PseudoJet paths, small and tiled kernels alike."""
    import torch
    evs = [E.single_event(n, 2, seed=90 + n) for n in (1, 2, 37, 700)] + [E.portable_event(5000, 3, seed=91)]
    p4, off = _batch(evs)
    for algo in (1, 0, -1):
        res = ctx.cluster_batch(p4, off, algo, 0.0, history=True, owner=True)
        for e, ev in enumerate(evs):
            o0, o1 = off[e], off[e + 1]
            assert res["n_jets"][e] == ev.shape[0]
            assert np.all(res["history"][o0:o1]["b"] == -1)
            U.compare_event(ev, algo, 0.0, res["jets"][o0:o1], res["n_jets"][e], res["history"][o0:o1],
                            res["owner"][o0:o1], ctx=f"R=0 n={ev.shape[0]} algo={algo}")
    one = ctx.cluster_event(torch.from_numpy(evs[3]).cuda(), -1, 0.0, history=True)
    assert int(one["n_jets"][0]) == evs[3].shape[0]


def test_bad_per_event_arguments_are_refused(ctx):
    """Per-event algorithm codes outside {kt, C/A, anti-kt} and radii that are
    negative or not finite are refused on the device (no jets, FJG_EINVAL);
    the other events are clustered as usual; scalar ones on the host."""
    import fastjet_gpu_gb300 as F
    b = E.mixed_batch(8, 20, 600, seed=62)
    algo = np.full(b.n_events, -1, np.int32)
    radius = np.full(b.n_events, 0.4)
    clean = ctx.cluster_batch(b.particles, b.offsets, algo, radius)
    algo[1] = 5
    radius[4] = -0.4
    radius[6] = np.nan
    with pytest.raises(F.FjgError):
        ctx.cluster_batch(b.particles, b.offsets, algo, radius)
    import torch
    out = ctx.cluster_batch_device(torch.from_numpy(b.particles).cuda(), torch.from_numpy(b.offsets).cuda(),
                                   torch.from_numpy(algo).cuda(), torch.from_numpy(radius).cuda())
    torch.cuda.synchronize()
    with pytest.raises(F.FjgError):
        ctx.check()
    nj = out["n_jets"].cpu().numpy()
    assert nj[1] == 0 and nj[4] == 0 and nj[6] == 0
    for e in (0, 2, 3, 5, 7):
        assert nj[e] == clean["n_jets"][e]
    for bad_r in (-1.0, float("nan"), float("inf")):
        with pytest.raises(F.FjgError):
            ctx.cluster_batch(b.particles, b.offsets, -1, bad_r)
    ctx.cluster_batch(b.particles, b.offsets, -1, 0.4)  # the context stays usable
