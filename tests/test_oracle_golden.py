"""The CPU oracle reproduces the reference backends' outputs bit for bit.

Goldens: tests/golden/make_golden.py ran the reference's tri_matrix, grid and
n_array backends (built from the reference sources) on the reference fixtures
and on seeded synthetic events, for kt / C-A / anti-kt and R in {0.4, 0.6,
0.8, 1.0}; all backends agreed on every case.
"""
import collections

import numpy as np
import pytest

import oracle
import golden_util as G


def test_full_jets_match_reference():
    checked = 0
    for name in ("354_fastjet", "808_cms", "synth_354", "synth_808", "synth_small"):
        evs = G.inputs(name)
        assert evs is not None
        for (algo, radius, ev), ref in G.full_jets(name).items():
            res = oracle.cluster(evs[ev], G.ALGO_CODE[algo], float(radius))
            mine = sorted(tuple(x) for x in res.jets.tolist())
            assert mine == ref, (name, algo, radius, ev)
            checked += 1
    assert checked == 12 * 4 + 12 * 8


def test_all_digests_match_reference():
    by_input = collections.defaultdict(list)
    for case in G.cases():
        by_input[case[0]].append(case)
    n = 0
    for name, cs in by_input.items():
        evs = G.inputs(name)
        for _, algo, radius, ev, nj, dg in cs:
            res = oracle.cluster(evs[ev], G.ALGO_CODE[algo], float(radius))
            assert len(res.jets) == nj, (name, algo, radius, ev)
            assert G.jets_digest(res.jets) == dg, (name, algo, radius, ev)
            n += 1
    assert n == 552


def test_makefile_run_matrix_jet_counts():
    """The reference Makefile's run targets (Makefile:69-87): 808_cms, R=0.4, ptmin 1.0."""
    ev = G.inputs("808_cms")[0]
    counts = {}
    for algo in ("antikt", "cam", "kt"):
        res = oracle.cluster(ev, G.ALGO_CODE[algo], 0.4)
        pt2 = res.jets[:, 0] ** 2 + res.jets[:, 1] ** 2
        counts[algo] = int((pt2 >= 1.0).sum())
    assert counts["antikt"] == 128  # tests/golden/driver/ak04_p1_808.txt: "found 128 jets above 1 GeV"
