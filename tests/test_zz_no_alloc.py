"""The allocation-free entry point fjg_cluster_batch_noalloc agrees with fjg_cluster_batch.

fjg_cluster_batch_noalloc serves callers that cannot allocate device memory
when they cluster (real-time code that forbids allocation after start-up,
applications whose memory belongs to another allocator): they pass every
buffer, and the kernels' bookkeeping sits in a static device array.  This test
calls it twice in a row through the C ABI -- the second call must not see
stale counters from the first -- and compares each result with the regular
batch entry point: identical jets, labels, counts and merge histories (bits of
the distances included), for small events and for an event above 4096
particles placed last in its batch.
It lives in its own file, collected last, and also passes alone.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_noalloc(F, torch, batch, algo, radius):
    L = F.lib()
    L.fjg_cluster_batch_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                            ctypes.POINTER(F._Outputs), ctypes.c_void_p]
    dev = torch.device("cuda", 0)
    total = int(batch.offsets[-1])
    ne = batch.n_events
    p4 = torch.from_numpy(batch.particles).to(dev)
    off = torch.from_numpy(batch.offsets).to(dev)
    jets = torch.full((total, 4), float("nan"), dtype=torch.float64, device=dev)
    lab = torch.full((total,), -7, dtype=torch.int32, device=dev)
    nj = torch.full((ne,), -7, dtype=torch.int32, device=dev)
    hist = torch.zeros((total, 2), dtype=torch.float64, device=dev)
    a_t = torch.from_numpy(np.asarray(algo, dtype=np.int32)).to(dev) if not np.isscalar(algo) else None
    r_t = torch.from_numpy(np.asarray(radius, dtype=np.float64)).to(dev) if not np.isscalar(radius) else None
    out = F._Outputs(jets.data_ptr(), lab.data_ptr(), nj.data_ptr(), hist.data_ptr(), None)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()
    st = L.fjg_cluster_batch_noalloc(ctypes.c_void_p(p4.data_ptr()), ctypes.c_void_p(off.data_ptr()), ne, total,
                                     ctypes.c_void_p(a_t.data_ptr()) if a_t is not None else None,
                                     int(algo) if a_t is None else 0,
                                     ctypes.c_void_p(r_t.data_ptr()) if r_t is not None else None,
                                     float(radius) if r_t is None else 0.0, ctypes.byref(out),
                                     ctypes.c_void_p(stream))
    assert st == 0, L.fjg_last_error(None)
    return {"jets": jets.cpu().numpy(), "jet_label": lab.cpu().numpy(), "n_jets": nj.cpu().numpy(),
            "history": hist.cpu().numpy().view(F.STEP).reshape(-1)}


def test_noalloc_matches_batch_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    from fastjet_gpu_gb300 import events as E

    first = E.mixed_batch(120, 20, 2048, seed=71)
    second, algo2, radius2 = E.serving_mix(60, seed=72, lo=2, hi=2048)
    # small events and, last, one above 4096 particles: the tiled kernel's
    # region of the static workspace ends at the batch's last particle
    third = E._batch_from([E.single_event(n, 2, seed=73 + n) for n in (300, 1500, 60)] +
                          [E.portable_event(6100, 3, seed=74)])
    assert max(b.offsets[-1] for b in (first, second, third)) <= 131072
    ctx = F.Context(0)
    cases = ((first, -1, 0.4), (second, algo2, radius2), (third, 1, 0.6), (third, 1, 0.6))
    for batch, algo, radius in cases:
        got = _run_noalloc(F, torch, batch, algo, radius)
        ref = ctx.cluster_batch(batch.particles, batch.offsets, algo, radius, history=True)
        assert np.array_equal(got["n_jets"], ref["n_jets"])
        for e in range(batch.n_events):
            o0, o1 = batch.offsets[e], batch.offsets[e + 1]
            k = ref["n_jets"][e]
            assert np.array_equal(got["jets"][o0:o0 + k], ref["jets"][o0:o0 + k]), e
            assert np.array_equal(got["jet_label"][o0:o0 + k], ref["jet_label"][o0:o0 + k]), e
            # the same kernels on the same inputs: the histories are identical bit for bit
            h, r = got["history"][o0:o1], ref["history"][o0:o1]
            assert np.array_equal(h["a"], r["a"]) and np.array_equal(h["b"], r["b"]), e
            assert np.array_equal(h["d"].view(np.int64), r["d"].view(np.int64)), e
    ctx.close()


def test_noalloc_refuses_ranges_outside_its_scratch():
    """An event whose particle range reaches past FJG_NOALLOC_MAX_PARTICLES
    (offsets that disagree with `total`) is refused on the device before any
    of its momenta are read (FJG_EINVAL, no jets); the other events of the
    call are clustered, and the next call is unaffected."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    from fastjet_gpu_gb300 import events as E

    b = E._batch_from([E.single_event(n, 2, seed=80 + n) for n in (200, 900)])
    L = F.lib()
    dev = torch.device("cuda", 0)
    total = int(b.offsets[-1])
    p4 = torch.from_numpy(b.particles).to(dev)
    # a third event claims [total, 131072 + 64): outside the static scratch
    off = torch.tensor(list(b.offsets) + [131072 + 64], dtype=torch.int64, device=dev)
    jets = torch.zeros((total, 4), dtype=torch.float64, device=dev)
    lab = torch.zeros(total, dtype=torch.int32, device=dev)
    nj = torch.full((3,), -7, dtype=torch.int32, device=dev)
    out = F._Outputs(jets.data_ptr(), lab.data_ptr(), nj.data_ptr(), None, None)
    f = L.fjg_cluster_batch_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(F._Outputs), ctypes.c_void_p]
    torch.cuda.synchronize()
    st = f(ctypes.c_void_p(p4.data_ptr()), ctypes.c_void_p(off.data_ptr()), 3, total, None, -1, None, 0.4,
           ctypes.byref(out), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert st == 1, L.fjg_last_error(None)
    ctx = F.Context(0)
    ref = ctx.cluster_batch(b.particles, b.offsets, -1, 0.4)
    got = nj.cpu().numpy()
    assert got[2] == 0 and np.array_equal(got[:2], ref["n_jets"])
    good = _run_noalloc(F, torch, b, -1, 0.4)
    assert np.array_equal(good["n_jets"], ref["n_jets"])
    ctx.close()
