"""fjg_cluster's command line follows the reference driver (main.cc:129-257):
missing values, negative or unparsable values and unknown options exit with
status 1 and the reference's message, before any GPU work."""
import os
import subprocess

import pytest

from fastjet_gpu_gb300 import build as B


@pytest.fixture(scope="module")
def driver():
    B.build()
    return B.DRIVER


@pytest.mark.parametrize("argv,msg", [
    (["--bogus"], "Unrecognized option --bogus"),
    (["-p"], "Missing argument to option -p"),
    (["--file"], "Missing argument to option --file"),
    (["-r", "-1"], "Error while parsing argument to option -r"),
    (["--ptmin", "abc"], "Error while parsing argument to option --ptmin"),
    (["--repeat", "-2"], "Error while parsing argument to option --repeat"),
    (["-combine", "x"], "Error while parsing argument to option -combine"),
])
def test_bad_options(driver, argv, msg):
    res = subprocess.run([driver] + argv, capture_output=True, text=True, timeout=60)
    assert res.returncode == 1
    assert msg in res.stderr
