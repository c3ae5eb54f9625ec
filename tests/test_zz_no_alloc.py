"""The allocation-free entry point fjg_cluster_batch_noalloc agrees with fjg_cluster_batch.

fjg_cluster_batch_noalloc serves callers that cannot allocate device memory
when they cluster (real-time code that forbids allocation after start-up,
applications whose memory belongs to another allocator): they pass every
buffer, and the kernels' bookkeeping sits in a static device array.  This test
calls it twice in a row through the C ABI -- the second call must not see
stale counters from the first -- and compares each result with the regular
batch entry point: identical jets, labels, counts and merge histories.
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
    assert first.offsets[-1] <= 131072 and second.offsets[-1] <= 131072
    ctx = F.Context(0)
    for batch, algo, radius in ((first, -1, 0.4), (second, algo2, radius2)):
        got = _run_noalloc(F, torch, batch, algo, radius)
        ref = ctx.cluster_batch(batch.particles, batch.offsets, algo, radius, history=True)
        assert np.array_equal(got["n_jets"], ref["n_jets"])
        for e in range(batch.n_events):
            o0, o1 = batch.offsets[e], batch.offsets[e + 1]
            k = ref["n_jets"][e]
            assert np.array_equal(got["jets"][o0:o0 + k], ref["jets"][o0:o0 + k]), e
            assert np.array_equal(got["jet_label"][o0:o0 + k], ref["jet_label"][o0:o0 + k]), e
            h, r = got["history"][o0:o1], ref["history"][o0:o1]
            assert np.array_equal(h["a"], r["a"]) and np.array_equal(h["b"], r["b"]), e
            np.testing.assert_allclose(h["d"], r["d"], rtol=1e-8, atol=0)
    ctx.close()
