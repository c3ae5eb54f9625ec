"""The fjg_cluster driver reproduces the reference driver's text output.

tests/golden/driver/<case>.txt holds the reference driver's stdout (timing and
device lines replaced, tests/golden/make_golden.py) for the cases in
DRIVER_CASES; the same command line is run through fjg_cluster and compared
line by line after the same replacement.
"""
import importlib.util
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
DRIVER = os.path.join(ROOT, "fastjet_gpu_gb300", "_lib", "fjg_cluster")


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


MG = _make_golden()


@pytest.mark.parametrize("case,backend,argv,rel", MG.DRIVER_CASES, ids=[c[0] for c in MG.DRIVER_CASES])
def test_driver_matches_reference_text(case, backend, argv, rel):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    with open(os.path.join(GOLD, rel)) as f:
        res = subprocess.run([DRIVER] + argv, stdin=f, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    with open(os.path.join(GOLD, "driver", case + ".txt")) as f:
        expected = f.read().split("\n", 1)[1]  # first line records the reference command
    got = MG.drop_timing(res.stdout)
    assert got == expected


REF_MAIN = os.path.join(ROOT, "oracle", "_ref", "bin", "main_gb300")


@pytest.mark.parametrize("case,backend,argv,rel", MG.DRIVER_CASES, ids=[c[0] for c in MG.DRIVER_CASES])
def test_unmodified_reference_driver_links_against_library(case, backend, argv, rel):
    """The reference's own main.cc (main.cc:118-370), compiled unmodified and
    linked against libfastjet_gb300.so in place of a backend object (the link
    line of INTEGRATION.md, oracle/ref/Makefile target main_gb300), prints the
    reference's text for every driver case."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.access(REF_MAIN, os.X_OK):
        pytest.skip("the reference driver was not built (no staged reference sources)")
    with open(os.path.join(GOLD, rel)) as f:
        res = subprocess.run([REF_MAIN] + argv, stdin=f, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    with open(os.path.join(GOLD, "driver", case + ".txt")) as f:
        expected = f.read().split("\n", 1)[1]
    assert MG.drop_timing(res.stdout) == expected


def test_reference_driver_zero_radius():
    """`-r 0` (accepted by the reference driver, main.cc:159): every particle
    becomes a jet; through the unmodified reference driver and through
    fjg_cluster alike."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rel = "data/354_fastjet.dat"
    outs = []
    for exe in (DRIVER, REF_MAIN):
        if not os.access(exe, os.X_OK):
            continue
        with open(os.path.join(GOLD, rel)) as f:
            res = subprocess.run([exe, "-antikt", "-r", "0", "--csv"], stdin=f, capture_output=True, text=True,
                                 timeout=300)
        assert res.returncode == 0, res.stderr
        outs.append(MG.drop_timing(res.stdout).strip().split("\n")[-1])
    assert outs and all(o == "354,354,<t>" for o in outs), outs
