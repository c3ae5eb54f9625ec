"""Build libfastjet_gb300.so (CUDA, sm_103a) and the fjg_cluster driver in-tree.

    python -m fastjet_gpu_gb300.build [--force]

Every translation unit under csrc/ is compiled by nvcc for
``-gencode arch=compute_103a,code=sm_103a`` in parallel, then linked into
fastjet_gpu_gb300/_lib/libfastjet_gb300.so.  The driver (driver/fjg_cluster.cc)
links against that library.  Outputs are git-ignored and rebuilt on the GPU
host, which is a different architecture from the build container.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libfastjet_gb300.so")
DRIVER = os.path.join(LIBDIR, "fjg_cluster")

GENCODE = "arch=compute_103a,code=sm_103a"


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-gencode", GENCODE, "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res


def build(force=False, verbose=False, phase_clocks=False):
    """Compile the CUDA library and the driver; return the library path.

    phase_clocks: a second build, with the kernels' per-step phase counters
    compiled in (-DFJG_PHASE_CLOCKS), into _lib_phases/ (no driver); the
    product build is unaffected.
    """
    libdir, objdir, lib = LIBDIR, OBJDIR, LIB
    flags = list(NVCC_FLAGS)
    if phase_clocks:
        libdir, objdir = os.path.join(PKG, "_lib_phases"), os.path.join(PKG, "_build_phases")
        lib = os.path.join(libdir, "libfastjet_gb300.so")
        flags.append("-DFJG_PHASE_CLOCKS")
    os.makedirs(libdir, exist_ok=True)
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    objs, jobs = [], []
    for src in _sources():
        obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for res in ex.map(_run, jobs):
            if verbose and res.stderr:
                print(res.stderr, file=sys.stderr)
    if force or jobs or _stale(lib, objs):
        tmp = lib + f".tmp{os.getpid()}"
        _run([nvcc, "-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, lib)
    if phase_clocks:
        return lib
    drv_src = os.path.join(PKG, "driver", "fjg_cluster.cc")
    if os.path.exists(drv_src) and (force or _stale(DRIVER, [drv_src, LIB] + headers)):
        cuda = _cuda_home()
        tmp = DRIVER + f".tmp{os.getpid()}"
        _run(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), drv_src, "-o", tmp,
              "-L" + LIBDIR, "-lfastjet_gb300", "-Wl,-rpath,$ORIGIN", "-L" + os.path.join(cuda, "lib64"),
              "-lcudart"])
        os.replace(tmp, DRIVER)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--phase-clocks", action="store_true", help="the phase-counter build, into _lib_phases/")
    args = ap.parse_args()
    print(build(force=args.force, verbose=True, phase_clocks=args.phase_clocks))
