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

usage (on a machine with a GPU, after `sh oracle/ref/stage.sh` on the machine
that has the reference mount and `make -f oracle/ref/Makefile` here):
    python tests/golden/make_golden.py [--out DIR]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import subprocess
import sys

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
    ap.add_argument("--condense-only", action="store_true", help="rebuild the committed files from RAW")
    args = ap.parse_args()
    raw = args.raw or os.path.join(args.out, "raw")
    for d in ("inputs", "ref_jets", "driver"):
        os.makedirs(os.path.join(args.out, d), exist_ok=True)
    if args.condense_only:
        condense(raw, args.out)
        return
    os.makedirs(os.path.join(raw, "ref_jets"), exist_ok=True)

    inputs = []
    for name, rel in FIXTURES.items():
        with open(os.path.join(HERE, rel)) as f:
            text = f.read()
        inputs.append((name, E.read_events(text)))
    for name, evs in synthetic_inputs():
        # the exact events the reference consumed are committed: the generator's
        # last bits depend on the host's libm, so they are not regenerated
        if name in FULL_JETS:
            E.write_events(evs, os.path.join(args.out, "inputs", name + ".txt"))
        else:
            b = E._batch_from(evs)
            np.savez_compressed(os.path.join(args.out, "inputs", name + ".npz"), particles=b.particles,
                                offsets=b.offsets)
        inputs.append((name, evs))

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

    for case, backend, argv, rel in DRIVER_CASES:
        exe = os.path.join(BIN, backend)
        with open(os.path.join(HERE, rel)) as f:
            res = subprocess.run([exe] + argv, stdin=f, capture_output=True, text=True, check=True)
        with open(os.path.join(args.out, "driver", case + ".txt"), "w") as f:
            f.write(f"# {backend} {' '.join(argv)} < {rel}\n")
            f.write(drop_timing(res.stdout))
        print(f"driver {case} done", flush=True)
    condense(raw, args.out)


if __name__ == "__main__":
    main()
