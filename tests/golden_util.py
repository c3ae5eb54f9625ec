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


# ---------------------------------------------------------------- large inputs and reference histories

def large_inputs(name):
    """Events of a large golden input, regenerated bit for bit by
    events.portable_pileup from the committed sizes and seed, and checked
    against the committed SHA-256 of the events the reference read."""
    spec = digests()["_large_inputs"][name]
    evs = E.portable_pileup(spec["sizes"], spec["seed"])
    got = [E.event_sha256(ev) for ev in evs]
    assert got == spec["sha256"], f"{name}: regenerated events differ from the ones the reference read"
    return evs


def history_cases():
    """{case key "<input>.<backend>.<algo>.<R>": summary} of ref_history.json."""
    with open(os.path.join(HERE, "ref_history.json")) as f:
        return json.load(f)


def history_sha256(a, b, d):
    """SHA-256 of a history: int32 a, then int32 b, then float64 d (little-endian)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(a, "<i4").tobytes())
    h.update(np.ascontiguousarray(b, "<i4").tobytes())
    h.update(np.ascontiguousarray(d, "<f8").tobytes())
    return h.hexdigest()


_DD = None


def reference_history(key, oracle_hist):
    """The reference backend's exact history for case `key` (a, b, d arrays
    over the input's events in order), rebuilt from the oracle's portable
    history of the same input and the committed differences; its SHA-256 must
    be the one recorded from the reference's own output."""
    global _DD
    if _DD is None:
        _DD = dict(np.load(os.path.join(HERE, "ref_history_d.npz")))
    summ = history_cases()[key]
    a = np.array(oracle_hist["a"], dtype=np.int32)
    b = np.array(oracle_hist["b"], dtype=np.int32)
    dbits = np.array(oracle_hist["d"], dtype=np.float64).view(np.int64).copy()
    if key + ".labels" in _DD:
        k, ra, rb = _DD[key + ".labels"].T
        a[k], b[k] = ra, rb
    if key + ".dulp" in _DD:
        dbits += _DD[key + ".dulp"].astype(np.int64)
    d = dbits.view(np.float64)
    assert history_sha256(a, b, d) == summ["sha256"], f"{key}: rebuilt history is not the reference's"
    return a, b, d


NEAR_TIE_RTOL = 1e-12


def near_tie_mismatch(a1, b1, d1, a2, b2, d2, rtol=NEAR_TIE_RTOL):
    """First step where history 2 departs from history 1 other than by the
    order of steps inside a near-tie group -- a run of consecutive steps whose
    distances agree within `rtol` relative in either history -- or -1; and the
    number of steps in reordered groups.  The reference evaluates pt^2 and dR^2
    with FMA contraction and CUDA's log/atan2 (nvcc defaults, Makefile:17), this
    library correctly rounded and uncontracted: distances that agree to the
    last bits (e.g. the beam distances of particles of equal pT) may be ordered
    differently; the step multisets of each group must still agree."""
    n, k, reordered = len(a1), 0, 0

    def close(x, y):
        return abs(x - y) <= rtol * max(abs(x), abs(y))

    while k < n:
        m = k
        while m + 1 < n and (close(d1[m], d1[m + 1]) or close(d2[m], d2[m + 1])):
            m += 1
        g1 = sorted(zip(np.asarray(a1[k:m + 1]).tolist(), np.asarray(b1[k:m + 1]).tolist()))
        g2 = sorted(zip(np.asarray(a2[k:m + 1]).tolist(), np.asarray(b2[k:m + 1]).tolist()))
        if g1 != g2:
            return k, reordered
        if m > k and (not np.array_equal(a1[k:m + 1], a2[k:m + 1]) or not np.array_equal(b1[k:m + 1], b2[k:m + 1])):
            reordered += m + 1 - k
        k = m + 1
    return -1, reordered


def tie_aware_mismatch(a1, b1, d1, a2, b2):
    """First step where history 2 departs from history 1 other than by the
    order of steps inside a tie group of history 1 (a run of equal d), or -1;
    and the number of steps in reordered tie groups."""
    n, k, reordered = len(a1), 0, 0
    while k < n:
        if a1[k] == a2[k] and b1[k] == b2[k]:
            k += 1
            continue
        s, m = k, k
        while s > 0 and d1[s - 1] == d1[k]:
            s -= 1
        while m + 1 < n and d1[m + 1] == d1[k]:
            m += 1
        g1 = sorted(zip(np.asarray(a1[s:m + 1]).tolist(), np.asarray(b1[s:m + 1]).tolist()))
        g2 = sorted(zip(np.asarray(a2[s:m + 1]).tolist(), np.asarray(b2[s:m + 1]).tolist()))
        if g1 != g2:
            return k, reordered
        reordered += m + 1 - k
        k = m + 1
    return -1, reordered


def golden_events(name):
    """Events of any golden input (fixtures, committed synthetic, large)."""
    if name in digests().get("_large_inputs", {}):
        return large_inputs(name)
    return inputs(name)
