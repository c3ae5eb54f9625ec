"""Kernel shapes, launch tuning and CUDA-graph capture (needs a GB300).

Every compiled kernel shape and build (a request for more CTAs per SM than the
plain build fits runs the register-capped build of the shapes that have one),
every CTA-per-SM count and every tile side must
give results identical to the oracle's; a captured graph must give the same
results as the direct call, also after its input buffers are refilled with a
different batch.
"""
import numpy as np
import pytest

import gpu_util as U
from fastjet_gpu_gb300 import events as E

pytestmark = pytest.mark.gpu

SHAPES = {0: [(64, 4), (128, 2)], 1: [(64, 8), (128, 4), (256, 2)], 2: [(128, 8), (256, 4)],
          3: [(256, 8), (512, 4)], 4: [(512, 8), (256, 16)]}


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    c = F.Context(0)
    yield c
    c.close()


def _with_shape(base, b, shape, ctas=0):
    t = {k: (list(v) if isinstance(v, list) else v) for k, v in base.items()}
    t["threads"][b], t["slots_per_thread"][b] = shape
    t["ctas_per_sm"][b] = ctas
    return t


def _bucket_batch(b, n_events=10, seed=0):
    cap = 256 << b
    lo = 2 if b == 0 else cap // 2 + 1
    rng = np.random.default_rng(100 + b + seed)
    sizes = list(rng.integers(lo, cap + 1, n_events - 1)) + [cap]
    return E._batch_from([E.single_event(int(n), 3, seed=int(s)) for n, s in zip(sizes, rng.integers(0, 2**31, n_events))])


def _check_batch(ctx, batch, algo, radius, tag):
    res = ctx.cluster_batch(batch.particles, batch.offsets, algo, radius, history=True, owner=True)
    for e in range(batch.n_events):
        o0, o1 = batch.offsets[e], batch.offsets[e + 1]
        U.compare_event(batch.event(e), algo, radius, res["jets"][o0:o1], res["n_jets"][e], res["history"][o0:o1],
                        res["owner"][o0:o1], res["jet_label"][o0:o1], ctx=f"{tag} event {e}")
    return res


@pytest.mark.parametrize("b", [0, 1, 2, 3, 4])
def test_every_kernel_shape_bit_exact(ctx, b):
    base = ctx.tuning
    try:
        for shape in SHAPES[b]:
            for ctas in (0, 1, 64):  # 64: as many as any build fits
                ctx.tuning = _with_shape(base, b, shape, ctas)
                got = ctx.tuning
                assert (got["threads"][b], got["slots_per_thread"][b]) == shape
                for algo, radius in ((-1, 0.4), (1, 0.6), (0, 1.0)):
                    _check_batch(ctx, _bucket_batch(b), algo, radius, f"bucket {b} shape {shape} ctas {ctas}")
    finally:
        ctx.tuning = base


def test_tile_side_does_not_change_results(ctx):
    base = ctx.tuning
    evs = [E.single_event(n, 4, seed=s, soft_mean=0.6, soft_eta=4.0) for n, s in ((4500, 1), (6200, 2))]
    b = E._batch_from(evs)
    ref = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True, owner=True)
    try:
        for factor in (1.5, 2.0, 3.7):
            t = dict(base)
            t["tile_factor"] = factor
            t["large_ctas_per_sm"] = 1
            ctx.tuning = t
            got = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4, history=True, owner=True)
            U.same_results(got, ref, b.offsets)
    finally:
        ctx.tuning = base


def test_set_tuning_rejects_bad_shapes(ctx):
    import fastjet_gpu_gb300 as F
    base = ctx.tuning
    for bad in (_with_shape(base, 0, (64, 8)), _with_shape(base, 2, (96, 8)), dict(base, tile_factor=0.5),
                dict(base, large_ctas_per_sm=0)):
        with pytest.raises(F.FjgError) as ei:
            ctx.tuning = bad
        assert ei.value.status == 1
    assert ctx.tuning == base


def test_graph_matches_direct_and_refills(ctx):
    import torch
    b1 = E._batch_from([E.single_event(int(n), 3, seed=int(n)) for n in (40, 300, 700, 1500, 2048, 3600, 5000, 90)])
    total = int(b1.offsets[-1])
    p4 = torch.from_numpy(b1.particles).cuda()
    off = torch.from_numpy(b1.offsets).cuda()
    g = ctx.capture_batch(p4, off, -1, 0.4, total=total, history=True, owner=True)
    try:
        for batch in (b1, None):
            if batch is None:
                # a different partition of at most the same number of particles
                sizes = [5100, 4000, 1000, 600, 400, 200, 100, 33]
                batch = E._batch_from([E.single_event(n, 2, seed=7 + n) for n in sizes])
                assert batch.offsets[-1] <= total
                p4[: batch.offsets[-1]].copy_(torch.from_numpy(batch.particles))
                off.copy_(torch.from_numpy(batch.offsets))
            g.launch()
            g.check()
            ref = ctx.cluster_batch(batch.particles, batch.offsets, -1, 0.4, history=True, owner=True)
            nt = int(batch.offsets[-1])
            assert np.array_equal(g.out["n_jets"].cpu().numpy()[: batch.n_events], ref["n_jets"])
            from fastjet_gpu_gb300 import history_records
            h = history_records(g.out["history"][:nt])
            assert np.array_equal(h, ref["history"])
            assert np.array_equal(g.out["owner"][:nt].cpu().numpy(), ref["owner"])
            jets = g.out["jets"].cpu().numpy()
            for e in range(batch.n_events):
                o0 = batch.offsets[e]
                nj = ref["n_jets"][e]
                assert np.array_equal(jets[o0:o0 + nj], ref["jets"][o0:o0 + nj])
    finally:
        g.close()


def test_autotune_picks_compiled_shapes(ctx):
    import fastjet_gpu_gb300 as F
    c = F.Context(0)
    try:
        t = c.autotune(-1, 0.4)
        for b in range(5):
            assert (t["threads"][b], t["slots_per_thread"][b]) in SHAPES[b]
            assert t["events_per_s"][b] > 0
        assert t["tile_factor"] in (1.0, 1.5, 2.0)
        batch = E.mixed_batch(64, 50, 2000, seed=77)
        a = c.cluster_batch(batch.particles, batch.offsets, -1, 0.4, history=True)
        r = ctx.cluster_batch(batch.particles, batch.offsets, -1, 0.4, history=True)
        for k in ("n_jets", "history"):
            assert np.array_equal(a[k], r[k])
        for e in range(batch.n_events):  # rows past an event's jets are not written
            o0, nj = batch.offsets[e], r["n_jets"][e]
            assert np.array_equal(a["jets"][o0:o0 + nj], r["jets"][o0:o0 + nj])
    finally:
        c.close()


def test_phase_counters_absent_from_product_build():
    """The per-step phase counters are compiled only into the separate
    -DFJG_PHASE_CLOCKS build (python -m fastjet_gpu_gb300.phases); the product
    library reports FJG_EINVAL for them and clusters as usual."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    from fastjet_gpu_gb300 import events as E
    ctx = F.Context(0)
    with pytest.raises(F.FjgError) as ei:
        ctx.phase_clocks()
    assert ei.value.status == 1 and "FJG_PHASE_CLOCKS" in str(ei.value)
    b = E.mixed_batch(8, 50, 300, seed=9)
    res = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4)
    assert int(res["n_jets"].sum()) > 0
    ctx.close()
