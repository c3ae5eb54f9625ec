"""Shared helpers for the GPU parity tests."""
import numpy as np

import oracle

D_RTOL = 1e-8  # history distances: see compare_event


def compare_event(p4, algo, radius, jets, n_jets, history=None, owner=None, jet_label=None, ctx="", portable=True):
    """Compare one event's GPU results with the CPU oracle.

    portable=True (default): the oracle runs with the library's integer
    kinematics (oracle.KIN_PORTABLE), i.e. the same FP64 values as the
    kernels, so everything must be identical bit for bit, distances included
    -- even for ties that hinge on the last bit of a log or atan2.
    portable=False: the oracle's libm kinematics (the form pinned to the
    reference outputs), compared as follows.

    Merge history: identical labels step by step (the merge decisions).  The
    recorded distances agree within 1e-8 relative: CUDA's and the host libm's
    log/atan2 may differ in the last place of a rapidity or azimuth, and for
    nearly coincident pseudojets dR2 = drap^2 + dphi^2 amplifies that
    cancellation error (observed: 2.6e-12 at dR2 ~ 1e-8).  Jet momenta:
    bit-identical (same merge tree; an E-scheme sum of two pseudojets does not
    depend on their order), in the same promotion order.
    """
    method = oracle.NN_INCREMENTAL | (oracle.KIN_PORTABLE if portable else 0)
    ref = oracle.cluster(p4, algo, radius, method)
    assert n_jets == len(ref.jets), f"{ctx}: n_jets {n_jets} vs {len(ref.jets)}"
    if history is not None:
        h = history
        assert np.array_equal(h["a"], ref.history["a"]) and np.array_equal(h["b"], ref.history["b"]), \
            f"{ctx}: merge history differs at step {int(np.flatnonzero((h['a'] != ref.history['a']) | (h['b'] != ref.history['b']))[0])}"
        if portable:
            assert np.array_equal(h["d"], ref.history["d"]), f"{ctx}: distances differ"
        else:
            np.testing.assert_allclose(h["d"], ref.history["d"], rtol=D_RTOL, atol=0, err_msg=ctx)
    assert np.array_equal(jets[:n_jets], ref.jets), f"{ctx}: jets differ"
    if jet_label is not None:
        assert np.array_equal(jet_label[:n_jets], ref.jet_label), f"{ctx}: jet labels differ"
    if owner is not None:
        assert np.array_equal(owner, ref.owner), f"{ctx}: constituents differ"
    return ref


def same_results(r1, r2, offsets, keys=("n_jets", "history", "owner")):
    """Two runs agree on every defined output: the whole of `keys` (those
    present), and the first n_jets[e] rows of jets and jet_label per event
    (rows past n_jets[e] are unspecified)."""
    for k in keys:
        if k in r1 or k in r2:
            assert np.array_equal(r1[k], r2[k]), k
    for e in range(len(offsets) - 1):
        o, nj = int(offsets[e]), int(r1["n_jets"][e])
        for k in ("jets", "jet_label"):
            assert np.array_equal(r1[k][o:o + nj], r2[k][o:o + nj]), (k, e)
