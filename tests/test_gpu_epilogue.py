"""Device epilogue (inclusive-jet filter and pT sort) and event combination (needs a GB300).

Compared with the reference driver's host post-processing (main.cc:309-327),
restated here in numpy: keep jets with px*px + py*py >= ptmin^2, order by
decreasing pt^2; equal pt^2 by increasing jet label (the reference's std::sort
leaves that order unspecified).
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


def _expected(jets, labels, ptmin, sort):
    pt2 = jets[:, 0] * jets[:, 0] + jets[:, 1] * jets[:, 1]
    keep = ~(pt2 < ptmin * ptmin)
    j, l, p = jets[keep], labels[keep], pt2[keep]
    if sort:
        order = np.lexsort((l, -p))
        j, l = j[order], l[order]
    return j, l


def _run(ctx, batch, algo, radius, ptmin, sort):
    import torch
    p4 = torch.from_numpy(batch.particles).cuda()
    off = torch.from_numpy(batch.offsets).cuda()
    out = ctx.cluster_batch_device(p4, off, algo, radius)
    sel = ctx.select_jets(out, off, ptmin, sort)
    jets, labels, nj = out["jets"].cpu().numpy(), out["jet_label"].cpu().numpy(), out["n_jets"].cpu().numpy()
    sj, sl, sn = sel["jets"].cpu().numpy(), sel["jet_label"].cpu().numpy(), sel["n_jets"].cpu().numpy()
    for e in range(batch.n_events):
        o = batch.offsets[e]
        ej, el = _expected(jets[o:o + nj[e]], labels[o:o + nj[e]], ptmin, sort)
        assert sn[e] == len(ej), (e, ptmin, sort)
        got_l = sl[o:o + sn[e]]
        bad = np.flatnonzero(got_l != el)
        assert bad.size == 0, (e, ptmin, sort, nj[e], bad[:5], got_l[bad[:5]], el[bad[:5]])
        assert np.array_equal(sj[o:o + sn[e]], ej), (e, ptmin, sort)


@pytest.mark.parametrize("ptmin,sort", [(0.0, False), (0.0, True), (1.0, True), (5.0, False), (1e9, True)])
def test_select_matches_driver_postprocessing(ctx, ptmin, sort):
    b = E.mixed_batch(200, 1, 4000, seed=91)
    _run(ctx, b, -1, 0.4, ptmin, sort)


def test_select_many_jets_and_ties(ctx):
    """Events with more jets than the shared-memory sort holds (anti-kt with a
    tiny R keeps almost every particle a jet), and exact pT ties."""
    big = E.single_event(6000, 2, seed=3)
    ties = np.repeat(E.single_event(300, 2, seed=4), 3, axis=0)  # equal-pt jets with R tiny
    b = E._batch_from([big, ties, E.single_event(50, 1, seed=5)])
    _run(ctx, b, -1, 0.01, 0.0, True)
    _run(ctx, b, -1, 0.01, 0.3, True)


def test_combine_events(ctx):
    import torch
    b = E.mixed_batch(23, 1, 300, seed=92)
    off = torch.from_numpy(b.offsets).cuda()
    for k in (1, 2, 5, 23, 40, 0):
        got = ctx.combine_events(off, k).cpu().numpy()
        kk = b.n_events if k in (0,) or k > b.n_events else k
        exp = b.offsets[np.minimum(np.arange(0, b.n_events + kk, kk), b.n_events)]
        exp = np.unique(exp) if k == 0 or k > b.n_events else exp
        assert np.array_equal(got, exp), k
    # clustering the combined batch equals clustering the concatenation
    c = ctx.combine_events(off, 4)
    p4 = torch.from_numpy(b.particles).cuda()
    res = ctx.cluster_batch_device(p4, c, -1, 0.4, history=True)
    cn = c.cpu().numpy()
    for e in range(cn.size - 1):
        ev = b.particles[cn[e]:cn[e + 1]]
        alone = ctx.cluster_batch(ev, np.array([0, ev.shape[0]]), -1, 0.4, history=True)
        h = res["history"].cpu().numpy().view(np.dtype([("a", "<i4"), ("b", "<i4"), ("d", "<f8")])).reshape(-1)
        assert np.array_equal(h[cn[e]:cn[e + 1]], alone["history"])
