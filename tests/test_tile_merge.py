"""The tiled kernel's summary merge (merge_skipped in fjg_cluster_tiled.cuh):
the summary of the new jet's tile is built from the other members' parts and
the new jet's key, and must equal the full summary of the tile.  A host
program (tests/tile_merge_check.cu) includes the kernel header, calls the
shipped function and compares it with a brute-force summary on random tiles
(CPU only; needs nvcc)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_merge_skipped_equals_full_summary(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "tile_merge_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                    "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "fastjet_gpu_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "tile_merge_check.cu"), "-o", exe],
                   check=True, capture_output=True, text=True, timeout=600)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and res.stdout.startswith("ok"), res.stdout + res.stderr
