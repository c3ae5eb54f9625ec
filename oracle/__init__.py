"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product path (fastjet_gpu_gb300) never does.  The oracle is
built into oracle/_build/libfjg_oracle.so by :func:`build` (gcc, FP64 without
FMA contraction).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfjg_oracle.so")

KT, CAM, ANTIKT = 1, 0, -1
NN_INCREMENTAL, NN_RECOMPUTE = 0, 1
KIN_PORTABLE = 16  # OR into method: the library's integer kinematics instead of libm

STEP_DTYPE = np.dtype([("a", np.int32), ("b", np.int32), ("d", np.float64)])


def build(force=False):
    """Compile the oracle shared library (gcc -O2 -ffp-contract=off)."""
    src = os.path.join(HERE, "fjg_oracle.c")
    kin_dir = os.path.join(os.path.dirname(HERE), "fastjet_gpu_gb300", "csrc")
    deps = [src, os.path.join(HERE, "fjg_oracle.h"), os.path.join(kin_dir, "fjg_kin.h"),
            os.path.join(kin_dir, "fjg_kin_tables.h")]
    if not force and os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d)
                                                       for d in deps):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I" + kin_dir, "-o", tmp, src, "-lm",
                    "-lpthread"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.fjo_cluster.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, P, P, P, P,
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]
        L.fjo_cluster.restype = ctypes.c_int
        L.fjo_cluster_batch.argtypes = [P, P, ctypes.c_int, P, P, ctypes.c_int, P, P, P, P, P,
                                        ctypes.POINTER(ctypes.c_longlong)]
        L.fjo_cluster_batch.restype = ctypes.c_int
        L.fjo_kinematics.argtypes = [P, ctypes.c_int, P, P, P, P]
        L.fjo_kinematics.restype = None
        for f in ("fjo_kin_log",):
            getattr(L, f).argtypes = [ctypes.c_double]
            getattr(L, f).restype = ctypes.c_double
        for f in ("fjo_kin_atan2", "fjo_kin_div"):
            getattr(L, f).argtypes = [ctypes.c_double, ctypes.c_double]
            getattr(L, f).restype = ctypes.c_double
        L.fjo_kin_f32.argtypes = [ctypes.c_double, ctypes.c_int]
        L.fjo_kin_f32.restype = ctypes.c_float
        L.fjo_kin_kinematics.argtypes = [P, ctypes.c_int, P, P, P]
        L.fjo_kin_kinematics.restype = None
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Result:
    """Clustering result of one event: history, jets (promotion order), labels, owners."""

    def __init__(self, history, jets, jet_label, owner, pair_evals):
        self.history = history
        self.jets = jets
        self.jet_label = jet_label
        self.owner = owner
        self.pair_evals = pair_evals


def cluster(p4, algo, R, method=NN_INCREMENTAL):
    p4 = np.ascontiguousarray(p4, dtype=np.float64).reshape(-1, 4)
    n = p4.shape[0]
    hist = np.zeros(max(n, 1), dtype=STEP_DTYPE)
    jets = np.zeros((max(n, 1), 4), dtype=np.float64)
    lab = np.zeros(max(n, 1), dtype=np.int32)
    own = np.zeros(max(n, 1), dtype=np.int32)
    nj = ctypes.c_int(0)
    ev = ctypes.c_longlong(0)
    rc = lib().fjo_cluster(_ptr(p4), n, int(algo), float(R), int(method), _ptr(hist), _ptr(jets), _ptr(lab),
                           _ptr(own), ctypes.byref(nj), ctypes.byref(ev))
    if rc:
        raise ValueError(f"oracle fjo_cluster failed ({rc})")
    k = nj.value
    return Result(hist[:n], jets[:k], lab[:k], own[:n], ev.value)


def cluster_batch(p4, offsets, algo, R, threads=1, want_history=True, portable=False):
    """Cluster a CSR batch on `threads` host threads; per-event algo/R may be scalars."""
    p4 = np.ascontiguousarray(p4, dtype=np.float64).reshape(-1, 4)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    ne = offsets.size - 1
    algo = np.ascontiguousarray(np.broadcast_to(np.asarray(algo, dtype=np.int32), (ne,)))
    R = np.ascontiguousarray(np.broadcast_to(np.asarray(R, dtype=np.float64), (ne,)))
    total = p4.shape[0]
    hist = np.zeros(max(total, 1), dtype=STEP_DTYPE) if want_history else None
    jets = np.zeros((max(total, 1), 4), dtype=np.float64)
    lab = np.zeros(max(total, 1), dtype=np.int32)
    own = np.zeros(max(total, 1), dtype=np.int32) if want_history else None
    nj = np.zeros(max(ne, 1), dtype=np.int32)
    ev = ctypes.c_longlong(0)
    th = int(threads) | ((KIN_PORTABLE << 16) if portable else 0)
    rc = lib().fjo_cluster_batch(_ptr(p4), _ptr(offsets), ne, _ptr(algo), _ptr(R), th, _ptr(hist),
                                 _ptr(jets), _ptr(lab), _ptr(own), _ptr(nj), ctypes.byref(ev))
    if rc:
        raise ValueError(f"oracle fjo_cluster_batch failed ({rc})")
    return hist, jets, lab, own, nj[:ne], ev.value


def kin_kinematics(p4, algo):
    """(rap, phi, w) from the library's integer kinematics (host build of fjg_kin.h)."""
    p4 = np.ascontiguousarray(p4, dtype=np.float64)
    out = np.zeros(3, dtype=np.float64)
    ptrs = [ctypes.c_void_p(out.ctypes.data + 8 * k) for k in range(3)]
    lib().fjo_kin_kinematics(_ptr(p4), int(algo), *ptrs)
    return tuple(out)


def kinematics(p4, algo):
    """(pt2, phi, rap, w) of one four-vector, as the reference computes them."""
    p4 = np.ascontiguousarray(p4, dtype=np.float64)
    out = np.zeros(4, dtype=np.float64)
    ptrs = [ctypes.c_void_p(out.ctypes.data + 8 * k) for k in range(4)]
    lib().fjo_kinematics(_ptr(p4), int(algo), *ptrs)
    return tuple(out)
