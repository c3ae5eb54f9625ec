"""Generate the reference golden vectors in tests/golden/.

Runs the reference's own backends (tri_matrix, n_array, grid), compiled from the
reference's unmodified sources by oracle/ref/Makefile, on a GPU host:

  1. inputs  : the reference's fixtures (data/*.dat, copied into
               tests/golden/data) and seeded synthetic events written by this
               script into tests/golden/inputs/ (generator:
               fastjet_gpu_gb300/events.py);
  2. jets    : for every input x backend x algorithm x R, the reference's
               cluster() output slots flagged isJet, in exact hex floats
               (oracle/ref/ref_dump.cc), into RAW/ref_jets/<input>.txt; then
               condensed (all backends must agree bit for bit) into
               tests/golden/ref_jets/<input>.txt (small inputs, full jets) and
               tests/golden/ref_digest.json (every case: jet count and SHA-256
               of the sorted hex momenta, and the backends that produced it);
  3. driver  : the reference driver's stdout for the CLI cases in DRIVER_CASES,
               with the timing-dependent lines dropped, into
               tests/golden/driver/<case>.txt.

  4. history: the history-printing copies of tri_matrix and grid
               (oracle/ref/stage_hist.py: the reference's own commented-out
               step printfs, tri_matrix.cu:235, grid.cu:454,462, enabled) print
               every step's two pseudojets and distance; the steps are replayed
               onto input labels (label = lowest constituent index) into
               RAW/ref_hist/<input>.<backend>.<algo>.<R>.npz.  Condensed here
               against the oracle's portable form into tests/golden/ref_history.json
               (per case: SHA-256 of the reference's exact (a, b, d) sequence,
               the steps whose labels differ from the oracle's) and
               tests/golden/ref_history_d.npz (per case: the reference's d minus
               the oracle's, in units in the last place);
  5. large   : pile-up-like events of 10k-22k particles made by the
               bit-reproducible generator (events.portable_pileup; only their
               SHA-256 is committed), clustered by the reference's grid backend
               (the only one valid at these sizes) for anti-kt R=0.4 and kt R=0.6:
               jets digests into ref_digest.json, histories as in 4.

usage (on a machine with a GPU, after `sh oracle/ref/stage.sh <reference dir>` on
the machine that has the reference sources and `make -f oracle/ref/Makefile` here):
    python tests/golden/make_golden.py [--out DIR] [--phases jets,driver,history,large]
then, on any machine, with the raw directory brought back:
    python tests/golden/make_golden.py --condense-history RAW
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import struct
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from fastjet_gpu_gb300 import events as E  # noqa: E402

BIN = os.path.join(ROOT, "oracle", "_ref", "bin")
ALGOS = {"kt": "-kt", "antikt": "-antikt", "cam": "-cam"}
RADII = ["0.4", "0.6", "0.8", "1.0"]
TRI_MATRIX_MAX_N = 2046  # tri_matrix.cu overflows its block-minimum buffer above this size

# name -> (path relative to tests/golden, max event size, run n_array?)
FIXTURES = {
    "354_fastjet": "data/354_fastjet.dat",
    "808_cms": "data/808_cms.dat",
    "multi-event": "data/multi-event.dat",
}


def synthetic_inputs():
    """Seeded synthetic inputs: (name, list of events)."""
    return [
        ("synth_354", [E.single_event(354, 3, seed=11)]),
        ("synth_808", [E.single_event(808, 4, seed=12)]),
        ("synth_mixed24", [E.mixed_batch(24, 50, 2000, seed=13).event(e) for e in range(24)]),
        ("synth_small", [E.single_event(n, 1, seed=100 + n) for n in (1, 2, 3, 5, 8, 13, 21, 34)]),
    ]


# large events: sizes and generator seed (events.portable_pileup; the events are
# regenerated bit for bit, only their SHA-256 is committed), and the
# configurations of the pile-up workload they are clustered with
LARGE_INPUTS = {"pileup4": ([10000, 13000, 17000, 22000], 40)}
LARGE_CASES = [("antikt", "0.4"), ("kt", "0.6")]


def large_inputs():
    return [(name, E.portable_pileup(sizes, seed)) for name, (sizes, seed) in LARGE_INPUTS.items()]


DRIVER_CASES = [
    # (case name, backend, argv, input fixture)
    ("ak04_p1_808", "tri_matrix", ["-antikt", "-r", "0.4", "-p", "1.0"], "data/808_cms.dat"),
    ("ca04_p1_808", "tri_matrix", ["-cam", "-r", "0.4", "-p", "1.0"], "data/808_cms.dat"),
    ("kt04_p1_808", "tri_matrix", ["-kt", "-r", "0.4", "-p", "1.0"], "data/808_cms.dat"),
    ("ak04_p1_808_grid", "grid", ["-antikt", "-r", "0.4", "-p", "1.0"], "data/808_cms.dat"),
    ("kt10_cart_354", "tri_matrix", ["-kt", "-R", "1.0", "--cartesian"], "data/354_fastjet.dat"),
    ("ca08_polar_multi", "tri_matrix", ["--cambridge-aachen", "-r", "0.8", "--polar", "--sort", "-p", "2"],
     "data/multi-event.dat"),
    ("ak06_combine3_multi", "grid", ["--anti-kt", "-r", "0.6", "--combine", "3", "--ptmin", "5"],
     "data/multi-event.dat"),
    ("ak04_csv_multi", "tri_matrix", ["-antikt", "-r", "0.4", "--csv", "--repeat", "2"], "data/multi-event.dat"),
]


def drop_timing(text):
    """Drop the lines of the reference driver's stdout that depend on the device or timing."""
    keep = []
    for line in text.split("\n"):
        if line.startswith("Running on CUDA device") or line.startswith("  - "):
            continue
        if " ms" in line and (line.startswith("found ") or line.startswith("clustered ")):
            line = line[: line.rfind(" in ")] + " in <t> ms" if " in " in line else line
        m = re.match(r"^(\d+),(\d+),", line)
        if m:
            line = f"{m.group(1)},{m.group(2)},<t>"
        keep.append(line)
    return "\n".join(keep)


def run_dump(backend, algo, radius, text):
    """Jets (slots with isJet) of every event, as (index, px, py, pz, E) hex strings."""
    exe = os.path.join(BIN, backend + "_dump")
    res = subprocess.run([exe, ALGOS[algo], radius], input=text, capture_output=True, text=True, check=True)
    events, cur = [], []
    for line in res.stdout.split("\n"):
        if not line:
            continue
        if line.startswith("end "):
            events.append(cur)
            cur = []
            continue
        slot, index, is_jet, px, py, pz, e = line.split()
        if is_jet == "1":
            cur.append(f"{index} {px} {py} {pz} {e}")
    return events


def _dbl(bits):
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def run_hist(backend, algo, radius, text):
    """Per event: (steps, jets) of a history-printing backend.  A step is
    (slot i, slot j, d bits, 4 momentum bits of i, 4 of j); i == j promotes."""
    exe = os.path.join(BIN, backend + "_hist_dump")
    res = subprocess.run([exe, ALGOS[algo], radius], input=text, capture_output=True, text=True, check=True,
                         timeout=3600)
    events, steps, jets = [], [], []
    for line in res.stdout.split("\n"):
        if not line:
            continue
        if line.startswith("H "):
            f = line.split()
            steps.append((int(f[1]), int(f[2])) + tuple(int(x, 16) for x in f[3:12]))
        elif line.startswith("end "):
            events.append((steps, jets))
            steps, jets = [], []
        else:
            slot, index, is_jet, px, py, pz, e = line.split()
            if is_jet == "1":
                jets.append(f"{index} {px} {py} {pz} {e}")
    return events


def _take(live, key):
    lst = live.get(key)
    if not lst:
        raise SystemExit("replay: a printed pseudojet is not among the live ones")
    lst.sort()
    v = lst.pop(0)
    if not lst:
        del live[key]
    return v


def replay(p4, steps):
    """Labels of a backend's printed steps: the backends compact or re-sort
    their slots, so each printed four-momentum is matched, bit for bit, to the
    live pseudojet that has it (inputs as read; a merge's sum as the backends
    form it, component-wise FP64 addition).  Returns a, b (-1: promotion), d."""
    live = {}
    for s, row in enumerate(np.asarray(p4)):
        live.setdefault(tuple(_bits(float(v)) for v in row), []).append(s)
    n = len(steps)
    a = np.empty(n, np.int32)
    b = np.empty(n, np.int32)
    d = np.empty(n, np.float64)
    for k, st in enumerate(steps):
        ki, kj = st[3:7], st[7:11]
        la = _take(live, ki)
        if st[0] == st[1]:
            a[k], b[k] = la, -1
        else:
            lb = _take(live, kj)
            new = tuple(_bits(_dbl(x) + _dbl(y)) for x, y in zip(ki, kj))
            live.setdefault(new, []).append(min(la, lb))
            a[k], b[k] = min(la, lb), max(la, lb)
        d[k] = _dbl(st[2])
    return a, b, d


def history_sha256(a, b, d):
    """SHA-256 of a history: int32 a, then int32 b, then float64 d (little-endian)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(a, "<i4").tobytes())
    h.update(np.ascontiguousarray(b, "<i4").tobytes())
    h.update(np.ascontiguousarray(d, "<f8").tobytes())
    return h.hexdigest()


def phase_history(raw, inputs):
    """Run the history-printing backends; raw npz per (input, backend, algo, R)."""
    os.makedirs(os.path.join(raw, "ref_hist"), exist_ok=True)
    for name, evs, cases in inputs:
        text = E.write_events(evs)
        max_n = max(ev.shape[0] for ev in evs)
        offsets = np.concatenate([[0], np.cumsum([ev.shape[0] for ev in evs])]).astype(np.int64)
        for backend in ("tri_matrix", "grid"):
            if backend == "tri_matrix" and max_n > TRI_MATRIX_MAX_N:
                continue
            for algo, radius in cases:
                t0 = time.time()
                res = run_hist(backend, algo, radius, text)
                if len(res) != len(evs):
                    raise SystemExit(f"{name} {backend} {algo} {radius}: {len(res)} events out of {len(evs)}")
                A, B, D, J = [], [], [], []
                for e, (ev, (steps, jets)) in enumerate(zip(evs, res)):
                    if len(steps) != ev.shape[0]:
                        raise SystemExit(f"{name} {backend} {algo} {radius} event {e}: {len(steps)} steps "
                                         f"for {ev.shape[0]} particles (printf FIFO too small?)")
                    a, b, d = replay(ev, steps)
                    A.append(a)
                    B.append(b)
                    D.append(d)
                    J.append([len(jets), jets_digest(jets)])
                path = os.path.join(raw, "ref_hist", f"{name}.{backend}.{algo}.{radius}.npz")
                np.savez_compressed(path, a=np.concatenate(A), b=np.concatenate(B), d=np.concatenate(D),
                                    offsets=offsets, jets=np.array(json.dumps(J)))
                print(f"history {name} {backend} {algo} {radius}: {time.time() - t0:.1f} s", flush=True)


def phase_large(raw):
    """Jets of the large events from the unmodified grid backend."""
    os.makedirs(os.path.join(raw, "ref_jets"), exist_ok=True)
    for name, evs in large_inputs():
        text = E.write_events(evs)
        lines = []
        for algo, radius in LARGE_CASES:
            t0 = time.time()
            jets = run_dump("grid", algo, radius, text)
            for e, ev_jets in enumerate(jets):
                lines.append(f"# grid {algo} {radius} {e} {len(ev_jets)}")
                lines.extend(ev_jets)
            print(f"large {name} grid {algo} {radius}: {time.time() - t0:.1f} s", flush=True)
        with open(os.path.join(raw, "ref_jets", name + ".txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
        with open(os.path.join(raw, "ref_jets", name + ".sha256.json"), "w") as f:
            json.dump([E.event_sha256(ev) for ev in evs], f)


def condense_large(raw, out_dir):
    """Add the large inputs' jets digests (and their input SHA-256) to ref_digest.json."""
    path = os.path.join(out_dir, "ref_digest.json")
    with open(path) as f:
        digests = json.load(f)
    digests.pop("_input_sha256", None)
    specs = digests.setdefault("_large_inputs", {})
    for name, evs in large_inputs():
        with open(os.path.join(raw, "ref_jets", name + ".sha256.json")) as f:
            raw_sha = json.load(f)
        mine = [E.event_sha256(ev) for ev in evs]
        if raw_sha != mine:
            raise SystemExit(f"{name}: the events regenerated here differ from the ones the reference read")
        sizes, seed = LARGE_INPUTS[name]
        specs[name] = {"sizes": sizes, "seed": seed, "sha256": mine}
        per_case, cur = {}, None
        for line in open(os.path.join(raw, "ref_jets", name + ".txt")):
            line = line.rstrip("\n")
            if line.startswith("#"):
                _, backend, algo, radius, ev, _n = line.split()
                cur = f"{algo} {radius} {ev}"
                per_case[cur] = []
            elif line:
                per_case[cur].append(line)
        digests[name] = {k: [len(v), jets_digest(v), ["grid"]] for k, v in per_case.items()}
    with open(path, "w") as f:
        json.dump(digests, f, indent=0, sort_keys=True)


def _golden_inputs(name, out_dir):
    """Events of a golden input as the reference read them."""
    if name in FIXTURES:
        with open(os.path.join(out_dir, FIXTURES[name])) as f:
            return E.read_events(f.read())
    for n, evs in large_inputs():
        if n == name:
            return evs
    txt = os.path.join(out_dir, "inputs", name + ".txt")
    if os.path.exists(txt):
        with open(txt) as f:
            return E.read_events(f.read())
    z = np.load(os.path.join(out_dir, "inputs", name + ".npz"))
    p, o = z["particles"], z["offsets"]
    return [p[o[e]:o[e + 1]] for e in range(o.size - 1)]


def tie_aware_mismatch(a1, b1, d1, a2, b2):
    """First step where history 2 departs from history 1 other than by the order
    of steps inside a tie group of history 1 (a run of equal d), or -1; and the
    number of steps in reordered tie groups."""
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
        g1 = sorted(zip(a1[s:m + 1].tolist(), b1[s:m + 1].tolist()))
        g2 = sorted(zip(a2[s:m + 1].tolist(), b2[s:m + 1].tolist()))
        if g1 != g2:
            return k, reordered
        reordered += m + 1 - k
        k = m + 1
    return -1, reordered


NEAR_TIE_RTOL = 1e-12


def near_tie_mismatch(a1, b1, d1, a2, b2, d2, rtol=NEAR_TIE_RTOL):
    """As tie_aware_mismatch, with near-tie groups: runs of consecutive steps
    whose distances agree within `rtol` relative in either history.  Two
    clusterings whose distances differ in the last bits (the reference's
    FMA-contracted FP64 and CUDA libm against correctly rounded, uncontracted
    FP64) may order such steps differently.  Returns (first step where the
    step multisets of a group differ, or -1; steps in reordered groups)."""
    n, k, reordered = len(a1), 0, 0

    def close(x, y):
        return abs(x - y) <= rtol * max(abs(x), abs(y))

    while k < n:
        m = k
        while m + 1 < n and (close(d1[m], d1[m + 1]) or close(d2[m], d2[m + 1])):
            m += 1
        g1 = sorted(zip(a1[k:m + 1].tolist(), b1[k:m + 1].tolist()))
        g2 = sorted(zip(a2[k:m + 1].tolist(), b2[k:m + 1].tolist()))
        if g1 != g2:
            return k, reordered
        if m > k and (not np.array_equal(a1[k:m + 1], a2[k:m + 1]) or not np.array_equal(b1[k:m + 1], b2[k:m + 1])):
            reordered += m + 1 - k
        k = m + 1
    return -1, reordered


def condense_history(raw, out_dir):
    """Committed history goldens: the reference's histories as exact differences
    from the oracle's portable form, pinned by the SHA-256 of the reference's own
    sequence.  Every case's jets must also match the unmodified backends'.

    ref_history.json   per case: steps, SHA-256 of the reference's (a, b, d),
                       the first step (and the number of steps) where the
                       reference's sequence departs from the oracle's beyond
                       exact ties, and beyond near ties, and statistics of the
                       distances
    ref_history_d.npz  per case: "<case>.labels" int32 [m, 3] (step, a, b) where
                       the reference's labels differ from the oracle's, and
                       "<case>.dulp" int16 (int32 if needed) [steps] the
                       reference's d minus the oracle's in units in the last
                       place (omitted when all 0)
    """
    sys.path.insert(0, ROOT)
    import oracle
    with open(os.path.join(out_dir, "ref_digest.json")) as f:
        digests = json.load(f)
    hdir = os.path.join(raw, "ref_hist")
    summary, arrays, cache = {}, {}, {}
    for fn in sorted(os.listdir(hdir)):
        if not fn.endswith(".npz"):
            continue
        key = fn[:-4]
        name, backend, algo, radius = key.split(".", 3)
        z = np.load(os.path.join(hdir, fn))
        ra, rb, rd, offsets = z["a"], z["b"], z["d"], z["offsets"]
        jets = json.loads(str(z["jets"]))
        for e, (nj, dg) in enumerate(jets):
            want = digests[name][f"{algo} {radius} {e}"]
            if [nj, dg] != want[:2]:
                raise SystemExit(f"{key} event {e}: the history-printing build's jets differ from the reference's")
        if name not in cache:
            evs = _golden_inputs(name, out_dir)
            cache[name] = (np.concatenate(evs).reshape(-1, 4), offsets)
        p4, off = cache[name]
        hist = oracle.cluster_batch(p4, off, ALGO_CODE[algo], float(radius), threads=os.cpu_count() or 4,
                                    portable=True)[0]
        oa, ob, od = hist["a"], hist["b"], hist["d"]
        diff = np.flatnonzero((oa != ra) | (ob != rb))
        exact_bad, exact_re, near_bad, near_re = -1, 0, -1, 0
        for e in range(off.size - 1):
            s0, s1 = int(off[e]), int(off[e + 1])
            k, r = tie_aware_mismatch(oa[s0:s1], ob[s0:s1], od[s0:s1], ra[s0:s1], rb[s0:s1])
            exact_re += r
            if k >= 0 and exact_bad < 0:
                exact_bad = s0 + k
            k, r = near_tie_mismatch(oa[s0:s1], ob[s0:s1], od[s0:s1], ra[s0:s1], rb[s0:s1], rd[s0:s1])
            near_re += r
            if k >= 0 and near_bad < 0:
                near_bad = s0 + k
        dd = rd.view(np.int64) - od.view(np.int64)
        if dd.size and np.abs(dd).max() >= 2 ** 31:
            raise SystemExit(f"{key}: a distance differs by more than 2^31 ulp")
        rel = np.abs(rd - od) / np.maximum(np.abs(od), 1e-300)
        summary[key] = {
            "steps": int(ra.size),
            "sha256": history_sha256(ra, rb, rd),
            "label_diff_steps": int(diff.size),
            "first_mismatch_exact_ties": int(exact_bad),
            "exact_tie_reordered_steps": int(exact_re),
            "first_mismatch": int(near_bad),
            "near_tie_reordered_steps": int(near_re),
            "d_bit_identical": int((dd == 0).sum()),
            "d_max_abs_ulp": int(np.abs(dd).max()) if dd.size else 0,
            "d_max_rel": float(rel.max()) if rel.size else 0.0,
        }
        if diff.size:
            arrays[key + ".labels"] = np.stack([diff, ra[diff], rb[diff]], axis=1).astype(np.int32)
        if np.any(dd):
            arrays[key + ".dulp"] = dd.astype(np.int16 if np.abs(dd).max() < 2 ** 15 else np.int32)
        print(key, {k: v for k, v in summary[key].items() if k != "sha256"}, flush=True)
    with open(os.path.join(out_dir, "ref_history.json"), "w") as f:
        json.dump(summary, f, indent=0, sort_keys=True)
    np.savez_compressed(os.path.join(out_dir, "ref_history_d.npz"), **arrays)


ALGO_CODE = {"kt": 1, "cam": 0, "antikt": -1}


# inputs whose jets are committed in full; the others are committed as digests
FULL_JETS = ("354_fastjet", "808_cms", "synth_354", "synth_808", "synth_small")


def jets_digest(lines):
    """SHA-256 of the sorted momenta of one event's jets, as Python float.hex() strings."""
    moms = sorted(" ".join(float.fromhex(x).hex() for x in l.split()[1:]) for l in lines)
    return hashlib.sha256("\n".join(moms).encode()).hexdigest()


def condense(raw_dir, out_dir):
    """Build the committed goldens from raw per-backend dumps.

    ref_jets/<input>.txt   jets of one backend (all backends must agree)
    ref_digest.json        {input: {"algo R event": [n_jets, sha256]}} for every case,
                           plus the list of backends that produced it
    """
    digests = {}
    for name in [n for n in FIXTURES] + [n for n, _ in synthetic_inputs()]:
        path = os.path.join(raw_dir, "ref_jets", name + ".txt")
        cases = {}
        cur = None
        for line in open(path):
            line = line.rstrip("\n")
            if line.startswith("#"):
                _, backend, algo, radius, ev, _n = line.split()
                cur = (backend, algo, radius, int(ev))
                cases[cur] = []
            elif line:
                cases[cur].append(line)
        per_case = {}
        for (backend, algo, radius, ev), lines in cases.items():
            key = f"{algo} {radius} {ev}"
            d = [len(lines), jets_digest(lines)]
            if key in per_case:
                if per_case[key]["result"] != d:
                    raise SystemExit(f"backends disagree: {name} {key} {backend}")
                per_case[key]["backends"].append(backend)
            else:
                per_case[key] = {"result": d, "backends": [backend], "lines": lines}
        digests[name] = {k: v["result"] + [v["backends"]] for k, v in per_case.items()}
        if name in FULL_JETS:
            with open(os.path.join(out_dir, "ref_jets", name + ".txt"), "w") as f:
                for key, v in per_case.items():
                    f.write(f"# {key} {len(v['lines'])}\n")
                    f.write("\n".join(v["lines"]) + ("\n" if v["lines"] else ""))
    with open(os.path.join(out_dir, "ref_digest.json"), "w") as f:
        json.dump(digests, f, indent=0, sort_keys=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--raw", default=None, help="directory for the raw per-backend dumps (default: OUT/raw)")
    ap.add_argument("--phases", default="jets,driver", help="comma list of jets, driver, history, large")
    ap.add_argument("--condense-only", action="store_true", help="rebuild the committed jets files from RAW")
    ap.add_argument("--condense-history", metavar="RAW", help="rebuild ref_history.* and the large digests from RAW")
    args = ap.parse_args()
    raw = args.raw or os.path.join(args.out, "raw")
    for d in ("inputs", "ref_jets", "driver"):
        os.makedirs(os.path.join(args.out, d), exist_ok=True)
    if args.condense_only:
        condense(raw, args.out)
        return
    if args.condense_history:
        condense_large(args.condense_history, args.out)
        condense_history(args.condense_history, args.out)
        return
    phases = set(args.phases.split(","))
    os.makedirs(os.path.join(raw, "ref_jets"), exist_ok=True)

    inputs = []
    for name, rel in FIXTURES.items():
        with open(os.path.join(HERE, rel)) as f:
            text = f.read()
        inputs.append((name, E.read_events(text)))
    for name, evs in synthetic_inputs():
        if "jets" in phases:
            # the exact events the reference consumed are committed: the generator's
            # last bits depend on the host's libm, so they are not regenerated
            if name in FULL_JETS:
                E.write_events(evs, os.path.join(args.out, "inputs", name + ".txt"))
            else:
                b = E._batch_from(evs)
                np.savez_compressed(os.path.join(args.out, "inputs", name + ".npz"), particles=b.particles,
                                    offsets=b.offsets)
            inputs.append((name, evs))
        else:
            inputs.append((name, _golden_inputs(name, args.out)))

    if "jets" in phases:
        for name, evs in inputs:
            text = E.write_events(evs)
            max_n = max(ev.shape[0] for ev in evs)
            lines = []
            for backend in ("tri_matrix", "grid", "n_array"):
                if backend == "tri_matrix" and max_n > TRI_MATRIX_MAX_N:
                    continue
                if backend == "n_array" and max_n > 1000:
                    continue
                for algo in ALGOS:
                    for radius in RADII:
                        jets = run_dump(backend, algo, radius, text)
                        for e, ev_jets in enumerate(jets):
                            lines.append(f"# {backend} {algo} {radius} {e} {len(ev_jets)}")
                            lines.extend(ev_jets)
                print(f"{name}: {backend} done", flush=True)
            with open(os.path.join(raw, "ref_jets", name + ".txt"), "w") as f:
                f.write("\n".join(lines) + "\n")

    if "driver" in phases:
        for case, backend, argv, rel in DRIVER_CASES:
            exe = os.path.join(BIN, backend)
            with open(os.path.join(HERE, rel)) as f:
                res = subprocess.run([exe] + argv, stdin=f, capture_output=True, text=True, check=True)
            with open(os.path.join(args.out, "driver", case + ".txt"), "w") as f:
                f.write(f"# {backend} {' '.join(argv)} < {rel}\n")
                f.write(drop_timing(res.stdout))
            print(f"driver {case} done", flush=True)
    if "jets" in phases:
        condense(raw, args.out)
    if "large" in phases:
        phase_large(raw)
    if "history" in phases:
        all_cases = [(a, r) for a in ALGOS for r in RADII]
        hist_inputs = [(name, evs, all_cases) for name, evs in inputs]
        hist_inputs += [(name, evs, LARGE_CASES) for name, evs in large_inputs()]
        phase_history(raw, hist_inputs)


if __name__ == "__main__":
    main()
