"""Helpers to read the committed reference goldens (tests/golden)."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from fastjet_gpu_gb300 import events as E

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ALGO_CODE = {"kt": 1, "cam": 0, "antikt": -1}
FIXTURES = {"354_fastjet": "data/354_fastjet.dat", "808_cms": "data/808_cms.dat",
            "multi-event": "data/multi-event.dat"}


def digests():
    with open(os.path.join(HERE, "ref_digest.json")) as f:
        return json.load(f)


def inputs(name):
    """Events of a golden input: the reference fixtures, or the exact synthetic
    events the reference consumed (inputs/<name>.txt or .npz)."""
    if name in FIXTURES:
        return E.read_events(os.path.join(HERE, FIXTURES[name]))
    path = os.path.join(HERE, "inputs", name + ".txt")
    if os.path.exists(path):
        return E.read_events(path)
    z = np.load(os.path.join(HERE, "inputs", name + ".npz"))
    p, o = z["particles"], z["offsets"]
    return [p[o[e]:o[e + 1]] for e in range(o.size - 1)]


def jets_digest(jets):
    """SHA-256 of sorted hex momenta, the format of ref_digest.json."""
    moms = sorted(" ".join(float(x).hex() for x in j) for j in np.asarray(jets).reshape(-1, 4))
    return hashlib.sha256("\n".join(moms).encode()).hexdigest()


def full_jets(name):
    """{(algo, R, event): sorted list of (px, py, pz, E) tuples} from ref_jets/<name>.txt."""
    out, cur = {}, None
    with open(os.path.join(HERE, "ref_jets", name + ".txt")) as f:
        for line in f:
            if line.startswith("#"):
                _, algo, radius, ev, _n = line.split()
                cur = (algo, radius, int(ev))
                out[cur] = []
            elif line.strip():
                _idx, *p = line.split()
                out[cur].append(tuple(float.fromhex(x) for x in p))
    return {k: sorted(v) for k, v in out.items()}


def cases():
    """Every golden case: (input name, algo name, R string, event index, n_jets, digest)."""
    for name, per in digests().items():
        if name.startswith("_"):
            continue
        for key, (nj, dg, _backends) in per.items():
            algo, radius, ev = key.split()
            yield name, algo, radius, int(ev), nj, dg
