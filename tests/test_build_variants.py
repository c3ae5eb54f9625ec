"""The phase-counter build (-DFJG_PHASE_CLOCKS, python -m fastjet_gpu_gb300.phases)
compiles, into its own directory, and exports the counter entry point; the
product build is a separate library.  CPU only (nvcc cross-compiles)."""
import os
import shutil
import subprocess

import pytest


def test_phase_clock_build_compiles():
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc not found")
    from fastjet_gpu_gb300 import build as B
    lib = B.build(phase_clocks=True)
    assert os.path.basename(os.path.dirname(lib)) == "_lib_phases"
    assert lib != B.LIB
    syms = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True,
                          check=True).stdout
    assert " fjg_phase_clocks" in syms
