"""GB300-native sequential-recombination jet clustering (kt, Cambridge/Aachen, anti-kt).

Python host mirror of the library's C ABI (include/fastjet_gb300.h), loaded
from the in-tree build fastjet_gpu_gb300/_lib/libfastjet_gb300.so.  There is no
CPU fallback: every call runs the CUDA kernels, and importing the bindings
raises if the library has not been built.

Reference interface mirrored (fwyzard/fastjet_gpu):
  * ``Algorithm``            -- cluster.h:4 ``enum class Algorithm {Kt=1, CambridgeAachen=0, AntiKt=-1}``
  * ``PSEUDOJET``            -- PseudoJet.h:4-11, the 40-byte I/O record
  * ``cluster(records, size, algo, r)`` -- cluster.h:6, in-place clustering of
    PseudoJet records (numpy structured array on the host, or a CUDA tensor of
    raw records on the device)
  * ``Context.cluster_batch`` / ``cluster_batch_device`` -- many events per call
"""
from __future__ import annotations

import ctypes
import enum
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# FJG_LIB selects another build of the library (e.g. the phase-counter build
# in _lib_phases/, see fastjet_gpu_gb300.phases)
LIB_PATH = os.environ.get("FJG_LIB") or os.path.join(_HERE, "_lib", "libfastjet_gb300.so")


class Algorithm(enum.IntEnum):
    Kt = 1
    CambridgeAachen = 0
    AntiKt = -1


KT, CAM, ANTIKT = 1, 0, -1

PSEUDOJET = np.dtype({"names": ["index", "isJet", "px", "py", "pz", "E"],
                      "formats": ["<i4", "?", "<f8", "<f8", "<f8", "<f8"],
                      "offsets": [0, 4, 8, 16, 24, 32], "itemsize": 40})
STEP = np.dtype([("a", "<i4"), ("b", "<i4"), ("d", "<f8")])

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "event too large",
          5: "timed out", 6: "try again", 7: "kernel error"}


class FjgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class _Outputs(ctypes.Structure):
    _fields_ = [("jets", ctypes.c_void_p), ("jet_label", ctypes.c_void_p), ("n_jets", ctypes.c_void_p),
                ("history", ctypes.c_void_p), ("owner", ctypes.c_void_p)]


class _Tuning(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32 * 5), ("slots_per_thread", ctypes.c_int32 * 5),
                ("ctas_per_sm", ctypes.c_int32 * 5), ("events_per_s", ctypes.c_double * 5),
                ("large_ctas_per_sm", ctypes.c_int32), ("tile_factor", ctypes.c_double)]

    def to_dict(self):
        return {"threads": list(self.threads), "slots_per_thread": list(self.slots_per_thread),
                "ctas_per_sm": list(self.ctas_per_sm), "events_per_s": list(self.events_per_s),
                "large_ctas_per_sm": self.large_ctas_per_sm, "tile_factor": self.tile_factor}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        for k in ("threads", "slots_per_thread", "ctas_per_sm"):
            getattr(t, k)[:] = [int(x) for x in d[k]]
        t.events_per_s[:] = [float(x) for x in d.get("events_per_s", [0.0] * 5)]
        t.large_ctas_per_sm = int(d["large_ctas_per_sm"])
        t.tile_factor = float(d["tile_factor"])
        return t


FJG_TUNE_SKIP_LARGE = 1
MAX_EVENT_PARTICLES = 1 << 24  # FJG_MAX_EVENT_PARTICLES: larger events are refused (FJG_ETOOBIG)
FJG_SERVE_HISTORY = 1
FJG_SERVE_DEVICE_CHECK = 2


class _ServerConfig(ctypes.Structure):
    _fields_ = [("arena_particles", ctypes.c_int64), ("max_inflight", ctypes.c_int32), ("streams", ctypes.c_int32),
                ("max_batch", ctypes.c_int32), ("oversubscribe", ctypes.c_int32), ("flags", ctypes.c_int32)]


class _Served(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("status", ctypes.c_int32), ("n_particles", ctypes.c_int32),
                ("n_jets", ctypes.c_int32), ("jets", ctypes.POINTER(ctypes.c_double)),
                ("jet_label", ctypes.POINTER(ctypes.c_int32)), ("history", ctypes.c_void_p),
                ("owner", ctypes.POINTER(ctypes.c_int32)), ("latency_us", ctypes.c_double)]

_lib = None


def lib():
    """The loaded C library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m fastjet_gpu_gb300.build` first")
        L = ctypes.CDLL(LIB_PATH)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.fjg_ctx_create.argtypes = [I, ctypes.POINTER(P)]
        L.fjg_ctx_destroy.argtypes = [P]
        L.fjg_ctx_destroy.restype = None
        L.fjg_ctx_stream.argtypes = [P]
        L.fjg_ctx_stream.restype = P
        L.fjg_ctx_check.argtypes = [P]
        L.fjg_last_error.argtypes = [P]
        L.fjg_last_error.restype = ctypes.c_char_p
        L.fjg_phase_clocks.argtypes = [P, P, I, I]
        L.fjg_status_string.argtypes = [I]
        L.fjg_status_string.restype = ctypes.c_char_p
        L.fjg_cluster_batch.argtypes = [P, P, P, I, ctypes.c_int64, P, I, P, D, ctypes.POINTER(_Outputs), P]
        L.fjg_cluster_batch_host.argtypes = [P, P, P, I, P, I, P, D, ctypes.POINTER(_Outputs)]
        L.fjg_cluster_event.argtypes = [P, P, I, I, D, P, P, P, P, P]
        L.fjg_cluster_pseudojets.argtypes = [P, P, I, I, D, P]
        L.fjg_kinematics.argtypes = [P, P, I, I, P, P, P, P]
        L.fjg_graph_capture_batch.argtypes = [P, P, P, I, ctypes.c_int64, P, I, P, D, ctypes.POINTER(_Outputs),
                                              ctypes.POINTER(P)]
        L.fjg_graph_launch.argtypes = [P, P]
        L.fjg_graph_check.argtypes = [P]
        L.fjg_graph_destroy.argtypes = [P]
        L.fjg_graph_destroy.restype = None
        L.fjg_get_tuning.argtypes = [P, ctypes.POINTER(_Tuning)]
        L.fjg_set_tuning.argtypes = [P, ctypes.POINTER(_Tuning)]
        L.fjg_autotune.argtypes = [P, I, D, I, ctypes.POINTER(_Tuning)]
        L.fjg_select_jets.argtypes = [P, P, P, P, P, I, ctypes.c_int64, D, I, P, P, P, P]
        L.fjg_combine_events.argtypes = [P, P, I, I, P, ctypes.POINTER(I), P]
        L.fjg_server_create.argtypes = [P, ctypes.POINTER(_ServerConfig), ctypes.POINTER(P)]
        L.fjg_server_destroy.argtypes = [P]
        L.fjg_server_destroy.restype = None
        L.fjg_server_submit.argtypes = [P, P, I, I, D, ctypes.POINTER(ctypes.c_uint64)]
        L.fjg_server_poll.argtypes = [P, ctypes.POINTER(_Served), I, ctypes.POINTER(I), ctypes.c_int64]
        L.fjg_server_release.argtypes = [P, ctypes.c_uint64]
        L.fjg_server_pending.argtypes = [P]
        L.fjg_server_launches.argtypes = [P]
        L.fjg_server_launches.restype = ctypes.c_int64
        L.fjg_server_replay.argtypes = [P, P, P, I, P, P, P, P, ctypes.POINTER(D)]
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.fjg_parse_events.argtypes = [P, ctypes.c_size_t, I, P, ctypes.c_int64, P, ctypes.c_int64, i64p, i64p, i64p]
        _lib = L
    return _lib


def parse_events(text, threads=0):
    """Read the reference driver's event text (bytes or str) into CSR arrays
    with the native multi-threaded reader (fjg_parse_events: same rules and
    values as events.read_events).  Returns (particles float64 [total, 4],
    offsets int64 [n_events + 1]); ValueError names the rejected line.  Host
    only: no GPU needed."""
    buf = text.encode() if isinstance(text, str) else bytes(text)
    cap = buf.count(b"\n") + 1  # particles <= lines, events + 1 <= lines + 1
    parts = np.empty((cap, 4), np.float64)
    offs = np.empty(cap + 1, np.int64)
    npart, nev, bad = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    st = lib().fjg_parse_events(buf, len(buf), int(threads), _np_ptr(parts), cap, _np_ptr(offs), cap + 1,
                                ctypes.byref(npart), ctypes.byref(nev), ctypes.byref(bad))
    if st == 1 and bad.value > 0:
        raise ValueError(lib().fjg_last_error(None).decode())
    if st:
        raise FjgError(st, lib().fjg_last_error(None).decode())
    return parts[:npart.value].copy(), offs[:nev.value + 1].copy()


def _np_ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _t_ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


_CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy


def _torch_stream(stream, device):
    """The stream a device-tensor call runs on: the given handle, or torch's
    current stream, so that torch's copies, reads and frees of the tensors
    are ordered with the library's kernels."""
    if stream:
        return stream
    import torch
    h = torch.cuda.current_stream(device).cuda_stream
    # torch's default stream has handle 0, which the C API reads as "the
    # context's stream": pass the explicit legacy-default-stream handle instead
    return h if h else _CUDA_STREAM_LEGACY


class Context:
    """A library context on one CUDA device (stream, scratch, side streams).

    Calls on torch CUDA tensors run on torch's current stream unless a stream
    handle is given; the synchronous ones (``cluster_event``,
    ``cluster_pseudojets``, ``kinematics``) run on the context's stream after
    it has waited for torch's current stream.
    """

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        st = lib().fjg_ctx_create(int(device), ctypes.byref(self._h))
        if st:
            raise FjgError(st, lib().fjg_last_error(None).decode())
        self.device = device

    def close(self):
        if self._h:
            lib().fjg_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            raise FjgError(st, lib().fjg_last_error(self._h).decode())

    @property
    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return lib().fjg_ctx_stream(self._h)

    def check(self):
        self._check(lib().fjg_ctx_check(self._h))

    PHASES = ("s1_argmin", "s2_merge", "s3_new_jet", "tail_resolve", "kin_warp0", "kin_warp1", "kin_warp2",
              "rescan_s2", "steps", "events", "exact_argmin", "exact_closer",
              "t_rebuild", "t_s1_argmin", "t_s2_merge_detect", "t_s3_lists_targets_window", "t_s3_overflow",
              "t_s3c_summaries", "t_kin_rapidity", "t_detect_s2", "t_steps", "t_events", "exact_key", "exact_nn",
              "t_targets", "t_target_steps", "t_list_update", "t_targets_warp1", "t_window_thread0",
              "t_resolve_new_jet", "t_summary_new_jet_tile", "t_summaries_warp1")

    def phase_clocks(self, reset=False):
        """Per-step phase counters of the clustering kernels (only in the
        -DFJG_PHASE_CLOCKS build, see fastjet_gpu_gb300.phases): a dict of
        summed clock cycles per phase, steps and events (t_*: tiled kernel)."""
        buf = (ctypes.c_ulonglong * 32)()
        self._check(lib().fjg_phase_clocks(self._h, buf, 32, 1 if reset else 0))
        return {k: int(buf[i]) for i, k in enumerate(self.PHASES) if k}

    def _after_torch(self, device):
        """Make the context's stream wait for torch's current stream."""
        import torch
        torch.cuda.ExternalStream(self.stream, device=device).wait_stream(torch.cuda.current_stream(device))

    # ------------------------------------------------------------ host memory
    def cluster_batch(self, particles, offsets, algo, radius, history=False, owner=False, out=None):
        """Cluster a CSR batch held in host memory; returns numpy arrays.

        particles float64 [total, 4]; offsets int64 [n_events + 1]; algo and
        radius are scalars or per-event arrays.  Returns a dict with ``jets``
        [total, 4], ``jet_label`` [total], ``n_jets`` [n_events] and, when
        requested, ``history`` (STEP records) and ``owner``.  ``out`` may pass
        preallocated output arrays under those keys (C-contiguous, of those
        dtypes and at least those lengths; page-locked memory makes the copies
        back direct), which are filled and returned as views.
        """
        p4 = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 4)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        ne = off.size - 1
        total = int(off[-1]) if ne >= 0 else 0
        a_arr = None if np.isscalar(algo) else np.ascontiguousarray(algo, dtype=np.int32)
        r_arr = None if np.isscalar(radius) else np.ascontiguousarray(radius, dtype=np.float64)
        want = {"jets": ((max(total, 1), 4), np.float64), "jet_label": ((max(total, 1),), np.int32),
                "n_jets": ((max(ne, 1),), np.int32)}
        if history:
            want["history"] = ((max(total, 1),), STEP)
        if owner:
            want["owner"] = ((max(total, 1),), np.int32)
        res = {}
        for k, (shape, dt) in want.items():
            a = None if out is None else out.get(k)
            if a is None:
                res[k] = np.zeros(shape, dt)
                continue
            if (not isinstance(a, np.ndarray) or a.dtype != np.dtype(dt) or not a.flags.c_contiguous
                    or a.shape[1:] != shape[1:] or a.shape[0] < shape[0]):
                raise ValueError(f"out[{k!r}] must be a C-contiguous {np.dtype(dt)} array of shape {shape} or longer")
            res[k] = a
        out = _Outputs(_np_ptr(res["jets"]).value, _np_ptr(res["jet_label"]).value, _np_ptr(res["n_jets"]).value,
                       _np_ptr(res["history"]).value if history else None,
                       _np_ptr(res["owner"]).value if owner else None)
        st = lib().fjg_cluster_batch_host(self._h, _np_ptr(p4), _np_ptr(off), ne, _np_ptr(a_arr),
                                          int(algo) if a_arr is None else 0, _np_ptr(r_arr),
                                          float(radius) if r_arr is None else 0.0, ctypes.byref(out))
        self._check(st)
        res["jets"] = res["jets"][:total]
        res["jet_label"] = res["jet_label"][:total]
        res["n_jets"] = res["n_jets"][:ne]
        if history:
            res["history"] = res["history"][:total]
        if owner:
            res["owner"] = res["owner"][:total]
        return res

    # ---------------------------------------------------------- device memory
    def cluster_batch_device(self, p4, offsets, algo, radius, total=None, history=False, owner=False, out=None,
                             stream=None):
        """Cluster device-resident torch CUDA tensors (asynchronous on the stream).

        p4 float64 [total, 4]; offsets int64 [n_events + 1]; algo/radius scalars
        or int32/float64 tensors.  ``out`` may pass preallocated outputs.
        """
        import torch
        ne = offsets.numel() - 1
        total = p4.shape[0] if total is None else total
        if out is None:
            dev = p4.device
            out = {"jets": torch.empty((max(total, 1), 4), dtype=torch.float64, device=dev),
                   "jet_label": torch.empty(max(total, 1), dtype=torch.int32, device=dev),
                   "n_jets": torch.empty(max(ne, 1), dtype=torch.int32, device=dev)}
            if history:
                out["history"] = torch.empty((max(total, 1), 2), dtype=torch.float64, device=dev)
            if owner:
                out["owner"] = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
        o = _Outputs(out["jets"].data_ptr(), out["jet_label"].data_ptr(), out["n_jets"].data_ptr(),
                     out["history"].data_ptr() if "history" in out else None,
                     out["owner"].data_ptr() if "owner" in out else None)
        a_t = None if isinstance(algo, (int, np.integer)) else algo
        r_t = None if isinstance(radius, (float, int, np.floating)) else radius
        s = _torch_stream(stream, p4.device)
        st = lib().fjg_cluster_batch(self._h, _t_ptr(p4), _t_ptr(offsets), ne, int(total), _t_ptr(a_t),
                                     int(algo) if a_t is None else 0, _t_ptr(r_t),
                                     float(radius) if r_t is None else 0.0, ctypes.byref(o), ctypes.c_void_p(s))
        self._check(st)
        return out

    def capture_batch(self, p4, offsets, algo, radius, total=None, history=False, owner=False, out=None):
        """Capture one batch call on these device tensors as a CUDA graph.

        Returns a ``Graph``; refill the tensors in place (event sizes may
        change as long as the last offset stays <= total) and launch again.
        """
        import torch
        ne = offsets.numel() - 1
        total = p4.shape[0] if total is None else total
        if out is None:
            dev = p4.device
            out = {"jets": torch.empty((max(total, 1), 4), dtype=torch.float64, device=dev),
                   "jet_label": torch.empty(max(total, 1), dtype=torch.int32, device=dev),
                   "n_jets": torch.empty(max(ne, 1), dtype=torch.int32, device=dev)}
            if history:
                out["history"] = torch.empty((max(total, 1), 2), dtype=torch.float64, device=dev)
            if owner:
                out["owner"] = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
        o = _Outputs(out["jets"].data_ptr(), out["jet_label"].data_ptr(), out["n_jets"].data_ptr(),
                     out["history"].data_ptr() if "history" in out else None,
                     out["owner"].data_ptr() if "owner" in out else None)
        a_t = None if isinstance(algo, (int, np.integer)) else algo
        r_t = None if isinstance(radius, (float, int, np.floating)) else radius
        h = ctypes.c_void_p()
        st = lib().fjg_graph_capture_batch(self._h, _t_ptr(p4), _t_ptr(offsets), ne, int(total), _t_ptr(a_t),
                                           int(algo) if a_t is None else 0, _t_ptr(r_t),
                                           float(radius) if r_t is None else 0.0, ctypes.byref(o), ctypes.byref(h))
        self._check(st)
        return Graph(self, h, out, (p4, offsets, a_t, r_t))

    @property
    def tuning(self):
        t = _Tuning()
        self._check(lib().fjg_get_tuning(self._h, ctypes.byref(t)))
        return t.to_dict()

    @tuning.setter
    def tuning(self, d):
        t = _Tuning.from_dict(d)
        self._check(lib().fjg_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, algo=-1, radius=0.4, skip_large=False):
        """Time the compiled kernel shapes per size bucket; keep and return the fastest."""
        t = _Tuning()
        self._check(lib().fjg_autotune(self._h, int(algo), float(radius), FJG_TUNE_SKIP_LARGE if skip_large else 0,
                                       ctypes.byref(t)))
        return t.to_dict()

    def select_jets(self, out, offsets, ptmin=0.0, sort=True, total=None, stream=None):
        """Inclusive jets with pT >= ptmin per event, by decreasing pT (device).

        ``out`` holds a batch's device outputs (``jets``, ``jet_label``,
        ``n_jets``); returns new tensors at the same positions.
        """
        import torch
        ne = offsets.numel() - 1
        total = out["jets"].shape[0] if total is None else total
        dev = out["jets"].device
        res = {"jets": torch.empty_like(out["jets"]), "jet_label": torch.empty_like(out["jet_label"]),
               "n_jets": torch.empty(max(ne, 1), dtype=torch.int32, device=dev)}
        self._check(lib().fjg_select_jets(self._h, _t_ptr(out["jets"]), _t_ptr(out["jet_label"]),
                                          _t_ptr(out["n_jets"]), _t_ptr(offsets), ne, int(total), float(ptmin),
                                          1 if sort else 0, _t_ptr(res["jets"]), _t_ptr(res["jet_label"]),
                                          _t_ptr(res["n_jets"]), ctypes.c_void_p(_torch_stream(stream, dev))))
        return res

    def combine_events(self, offsets, k, stream=None):
        """Offsets of the batch with every k consecutive events merged (k = 0: all)."""
        import torch
        ne = offsets.numel() - 1
        n_out = ctypes.c_int()
        res = torch.empty(max(ne, 1) + 1, dtype=torch.int64, device=offsets.device)
        self._check(lib().fjg_combine_events(self._h, _t_ptr(offsets), ne, int(k), _t_ptr(res),
                                             ctypes.byref(n_out),
                                             ctypes.c_void_p(_torch_stream(stream, offsets.device))))
        return res[: n_out.value + 1]

    def cluster_event(self, p4, algo, radius, history=False, owner=False):
        """The plain path: one event per launch (torch CUDA tensors), synchronous."""
        import torch
        n = p4.shape[0]
        dev = p4.device
        out = {"jets": torch.empty((max(n, 1), 4), dtype=torch.float64, device=dev),
               "jet_label": torch.empty(max(n, 1), dtype=torch.int32, device=dev),
               "n_jets": torch.empty(1, dtype=torch.int32, device=dev)}
        if history:
            out["history"] = torch.empty((max(n, 1), 2), dtype=torch.float64, device=dev)
        if owner:
            out["owner"] = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        self._after_torch(dev)
        st = lib().fjg_cluster_event(self._h, _t_ptr(p4), n, int(algo), float(radius), _t_ptr(out["jets"]),
                                     _t_ptr(out["jet_label"]), _t_ptr(out["n_jets"]),
                                     _t_ptr(out.get("history")), _t_ptr(out.get("owner")))
        self._check(st)
        return out

    def kinematics(self, p4, algo):
        """(rap, phi, w) of device four-momenta (torch CUDA float64 [n, 4]), synchronous."""
        import torch
        n = p4.shape[0]
        rap, phi, w = (torch.empty(max(n, 1), dtype=torch.float64, device=p4.device) for _ in range(3))
        self._after_torch(p4.device)
        self._check(lib().fjg_kinematics(self._h, _t_ptr(p4), n, int(algo), _t_ptr(rap), _t_ptr(phi), _t_ptr(w),
                                         None))
        self.check()
        return rap[:n], phi[:n], w[:n]

    def cluster_pseudojets(self, records, size, algo, radius):
        """In-place clustering of PseudoJet records (cluster.h:6 semantics).

        ``records``: a numpy PSEUDOJET array (host; copied to the device and
        back) or a CUDA torch uint8 tensor of ``size * 40`` bytes (in place).
        """
        import torch
        if isinstance(records, np.ndarray):
            assert records.dtype == PSEUDOJET
            host = records
            dev = torch.from_numpy(records.view(np.uint8).reshape(-1).copy()).cuda(self.device)
        else:
            host, dev = None, records
        self._after_torch(dev.device)
        st = lib().fjg_cluster_pseudojets(self._h, _t_ptr(dev), int(size), int(algo), float(radius), None)
        self._check(st)
        if host is not None:
            host.view(np.uint8).reshape(-1)[:] = dev.cpu().numpy()
        return records


class Graph:
    """A captured batch call (fjg_graph_*): ``launch()`` reruns it on the captured tensors."""

    def __init__(self, ctx, handle, out, keep):
        self.ctx, self._h, self.out, self._keep = ctx, handle, out, keep

    def launch(self, stream=None):
        """Launch on the given stream handle, or torch's current stream."""
        s = _torch_stream(stream, self.out["jets"].device)
        self.ctx._check(lib().fjg_graph_launch(self._h, ctypes.c_void_p(s)))

    def check(self):
        self.ctx._check(lib().fjg_graph_check(self._h))

    def close(self):
        if self._h:
            lib().fjg_graph_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request server on a context (fjg_server_*): submit events one at a time,
    poll for completed ones.  Continuous batching; see fastjet_gb300.h."""

    def __init__(self, ctx, arena_particles=0, max_inflight=0, streams=0, max_batch=0, oversubscribe=0,
                 history=False, device_check=False):
        self.ctx = ctx
        flags = (FJG_SERVE_HISTORY if history else 0) | (FJG_SERVE_DEVICE_CHECK if device_check else 0)
        cfg = _ServerConfig(int(arena_particles), int(max_inflight), int(streams), int(max_batch),
                            int(oversubscribe), flags)
        self._h = ctypes.c_void_p()
        ctx._check(lib().fjg_server_create(ctx._h, ctypes.byref(cfg), ctypes.byref(self._h)))
        self.history = history

    def submit(self, p4, algo, radius):
        p4 = np.ascontiguousarray(p4, dtype=np.float64).reshape(-1, 4)
        t = ctypes.c_uint64()
        self.ctx._check(lib().fjg_server_submit(self._h, _np_ptr(p4), p4.shape[0], int(algo), float(radius),
                                                ctypes.byref(t)))
        return t.value

    def poll(self, max_results=64, timeout_us=0):
        """Completed requests as dicts (results copied, arena ranges released)."""
        buf = (_Served * max_results)()
        n = ctypes.c_int()
        self.ctx._check(lib().fjg_server_poll(self._h, buf, max_results, ctypes.byref(n), int(timeout_us)))
        out = []
        for k in range(n.value):
            r = buf[k]
            nj, npart = r.n_jets, r.n_particles
            d = {"ticket": r.ticket, "status": r.status, "n_jets": nj, "latency_us": r.latency_us,
                 "jets": np.ctypeslib.as_array(r.jets, (max(nj, 1) * 4,))[: 4 * nj].reshape(nj, 4).copy()
                 if nj else np.zeros((0, 4)),
                 "jet_label": np.ctypeslib.as_array(r.jet_label, (max(nj, 1),))[:nj].copy() if nj else
                 np.zeros(0, np.int32)}
            if self.history and npart:
                raw = (ctypes.c_char * (16 * npart)).from_address(r.history)
                d["history"] = np.frombuffer(raw, dtype=STEP, count=npart).copy()
                d["owner"] = np.ctypeslib.as_array(r.owner, (npart,)).copy()
            out.append(d)
            self.ctx._check(lib().fjg_server_release(self._h, r.ticket))
        return out

    @property
    def pending(self):
        return lib().fjg_server_pending(self._h)

    @property
    def launches(self):
        """Clustering kernels launched so far (one per micro-batch)."""
        return int(lib().fjg_server_launches(self._h))

    def replay(self, particles, offsets, algo, radius, arrival_us):
        """Open-loop replay of a trace; returns (latency_us per event, wall_us)."""
        p4 = np.ascontiguousarray(particles, dtype=np.float64)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        a = np.ascontiguousarray(algo, dtype=np.int32)
        r = np.ascontiguousarray(radius, dtype=np.float64)
        t = np.ascontiguousarray(arrival_us, dtype=np.float64)
        lat = np.zeros(off.size - 1)
        wall = ctypes.c_double()
        self.ctx._check(lib().fjg_server_replay(self._h, _np_ptr(p4), _np_ptr(off), off.size - 1, _np_ptr(a),
                                                _np_ptr(r), _np_ptr(t), _np_ptr(lat), ctypes.byref(wall)))
        return lat, wall.value

    def close(self):
        if self._h:
            lib().fjg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = {}


def default_context(device=0):
    if device not in _default_ctx:
        _default_ctx[device] = Context(device)
    return _default_ctx[device]


def cluster(records, size, algo, r):
    """Drop-in for the reference's ``cluster(PseudoJet*, int, Algorithm, double)``."""
    return default_context().cluster_pseudojets(records, size, int(algo), r)


def history_records(t):
    """View a device history tensor (float64 [n, 2]) as numpy STEP records."""
    return t.cpu().numpy().view(STEP).reshape(-1)
