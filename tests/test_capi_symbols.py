"""The C-ABI library builds for sm_103a and exports every symbol its headers declare.

No compute calls: this runs without a GPU.
"""
import ctypes
import os
import re
import subprocess

import pytest

from fastjet_gpu_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for h in ("fastjet_gb300.h",):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fjg_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    return B.build()


def test_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    names = _declared_functions()
    assert "fjg_cluster_batch" in names and "fjg_cluster_pseudojets" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_exports_reference_cpp_symbol(libpath):
    # cluster(PseudoJet*, int, Algorithm, double) from cluster.h:6
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    assert "_Z7clusterP9PseudoJeti9Algorithmd" in out


def test_status_strings(libpath):
    L = ctypes.CDLL(libpath)
    L.fjg_status_string.restype = ctypes.c_char_p
    assert L.fjg_status_string(0) == b"ok"
    assert L.fjg_status_string(4) == b"event too large"


def test_compat_header_matches_reference_layout():
    # PseudoJet.h:4-11 layout: 40 bytes, px at offset 8
    import numpy as np
    import fastjet_gpu_gb300 as F
    assert F.PSEUDOJET.itemsize == 40
    assert F.PSEUDOJET.fields["px"][1] == 8 and F.PSEUDOJET.fields["E"][1] == 32
    assert int(F.Algorithm.Kt) == 1 and int(F.Algorithm.CambridgeAachen) == 0 and int(F.Algorithm.AntiKt) == -1


def test_size_limit_constant_matches_header():
    import fastjet_gpu_gb300 as F
    text = open(os.path.join(ROOT, "include", "fastjet_gb300.h")).read()
    m = re.search(r"#define FJG_MAX_EVENT_PARTICLES (\d+)", text)
    assert m and int(m.group(1)) == F.MAX_EVENT_PARTICLES


def test_host_side_argument_checks():
    """Calls refused before any device work: a null context, a null server,
    and (without a GPU) context creation reports a CUDA error, not a crash."""
    import fastjet_gpu_gb300 as F
    L = F.lib()
    st = L.fjg_cluster_batch(None, None, None, 1, 0, None, -1, None, 0.4, None, None)
    assert st == 1 and b"ctx is null" in L.fjg_last_error(None)
    assert L.fjg_server_pending(None) == 0 and L.fjg_server_launches(None) == 0
    import torch
    if not torch.cuda.is_available():
        h = ctypes.c_void_p()
        st = L.fjg_ctx_create(0, ctypes.byref(h))
        assert st != 0 and not h.value
        assert L.fjg_last_error(None)


def test_noalloc_limits_refused_before_device_work():
    """fjg_cluster_batch_noalloc refuses batches beyond its static scratch
    (more than FJG_NOALLOC_MAX_EVENTS events or FJG_NOALLOC_MAX_PARTICLES
    particles) with FJG_EINVAL before touching a device."""
    import fastjet_gpu_gb300 as F
    text = open(os.path.join(ROOT, "include", "fastjet_gb300.h")).read()
    max_events = int(re.search(r"#define FJG_NOALLOC_MAX_EVENTS (\d+)", text).group(1))
    max_particles = int(re.search(r"#define FJG_NOALLOC_MAX_PARTICLES (\d+)", text).group(1))
    L = F.lib()
    f = L.fjg_cluster_batch_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(F._Outputs), ctypes.c_void_p]
    dummy = ctypes.c_void_p(64)  # never dereferenced: the calls are refused first
    out = F._Outputs(dummy.value, dummy.value, dummy.value, None, None)
    st = f(dummy, dummy, 1, max_particles + 1, None, -1, None, 0.4, ctypes.byref(out), None)
    assert st == 1 and b"FJG_NOALLOC_MAX_PARTICLES" in L.fjg_last_error(None)
    st = f(dummy, dummy, max_events + 1, 10, None, -1, None, 0.4, ctypes.byref(out), None)
    assert st == 1 and b"FJG_NOALLOC_MAX_EVENTS" in L.fjg_last_error(None)
    st = f(dummy, dummy, 1, 10, None, 5, None, 0.4, ctypes.byref(out), None)
    assert st == 1 and b"algorithm" in L.fjg_last_error(None)
