"""Event-text reader: the native multi-threaded fjg_parse_events against the
Python reader (events.read_events), both following the reference driver's
read_next_event (main.cc:34-70).  Runs on the CPU (no GPU needed)."""
import os

import numpy as np
import pytest

from fastjet_gpu_gb300 import events as E

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def F():
    import fastjet_gpu_gb300 as F
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return F


def _csr(events):
    offs = np.zeros(len(events) + 1, np.int64)
    offs[1:] = np.cumsum([e.shape[0] for e in events])
    parts = np.concatenate(events) if events else np.zeros((0, 4))
    return parts, offs


def _same(F, text, threads=(1, 3, 16)):
    ref_p, ref_o = _csr(E.read_events(text))
    for t in threads:
        p, o = F.parse_events(text, threads=t)
        assert np.array_equal(o, ref_o), t
        assert p.shape == ref_p.shape and np.array_equal(p.view(np.uint64), ref_p.view(np.uint64)), t
    return ref_p, ref_o


def _random_text(rng, n_events, max_n, decorate=True):
    out = []
    for e in range(n_events):
        if decorate and rng.random() < 0.3:
            out.append("# event %d" % e)
        if decorate and rng.random() < 0.3:
            out.append("")
        n = int(rng.integers(1, max_n + 1))
        vals = rng.normal(0, 30, (n, 4)) * 10.0 ** rng.integers(-3, 4, (n, 4))
        for row in vals:
            fields = []
            for v in row:
                k = rng.integers(0, 5)
                fields.append("%.17g" % v if k == 0 else "%.6e" % v if k == 1 else "%+.3f" % v if k == 2
                              else repr(float(v)) if k == 3 else "%.17G" % v)
            sep = " " if rng.random() < 0.7 else "\t"
            tail = "" if rng.random() < 0.8 else "  extra tokens 7"
            out.append(sep.join(fields) + tail)
        out.append("" if rng.random() < 0.6 else "#")
    return "\n".join(out) + "\n"


def test_fixtures_match_python_reader(F):
    for name in ("354_fastjet.dat", "808_cms.dat", "multi-event.dat"):
        with open(os.path.join(HERE, "golden", "data", name)) as f:
            text = f.read()
        p, o = _same(F, text)
        assert o[-1] > 0


def test_random_texts_and_chunk_boundaries(F):
    rng = np.random.default_rng(5)
    for k in range(5):
        _same(F, _random_text(rng, 40, 60))
    # several MiB: events cross the thread chunk boundaries
    big = _random_text(rng, 3000, 400, decorate=False)
    assert len(big) > 4 << 20
    _same(F, big, threads=(1, 2, 5, 16))


def test_format_rules(F):
    # runs of separators, comments inside, numbers back to back, '+' signs, extra fields
    text = "#h\n\n\n1 2 3 4\n+5 -6 7e1 8.5 junk\n#c\n\n1-2 3 .5 9\n#\n"
    p, o = _same(F, text)
    assert o.tolist() == [0, 2, 3]
    assert p[1].tolist() == [5.0, -6.0, 70.0, 8.5] and p[2].tolist() == [1.0, -2.0, 3.0, 0.5]
    # a final line without a newline is not read (the reference's getline loop)
    p, o = _same(F, "1 2 3 4\n5 6 7 8")
    assert o.tolist() == [0, 1]
    # empty text, only comments
    for t in ("", "\n", "# nothing\n\n"):
        p, o = _same(F, t)
        assert o.tolist() == [0] and p.shape == (0, 4)


@pytest.mark.parametrize("bad,line", [("1 2 3 4\n \n5 6 7 8\n", 2), ("1 2 3\n", 1), ("#\nabc 1 2 3\n", 2),
                                      ("1 2 3 inf\n", 1), ("1 2 3 nan\n", 1), ("1 2 3 4\n\r\n", 2),
                                      ("1 2 3 4\n\n\n\n1 2 x 4\n", 5)])
def test_rejected_lines(F, bad, line):
    with pytest.raises(ValueError):
        E.read_events(bad)
    with pytest.raises(ValueError, match=f"line {line} "):
        F.parse_events(bad)
    # the error is found whatever the chunking
    filler = "".join("%d 1 2 3\n" % i for i in range(200000))
    with pytest.raises(ValueError, match=f"line {200000 + line} "):
        F.parse_events(filler + bad, threads=8)


def test_capacity_reported(F):
    import ctypes
    text = b"1 2 3 4\n\n5 6 7 8\n9 9 9 9\n"
    parts = np.empty((1, 4))
    offs = np.empty(2, np.int64)
    npart, nev, bad = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    st = F.lib().fjg_parse_events(text, len(text), 1, parts.ctypes.data, 1, offs.ctypes.data, 2,
                                  ctypes.byref(npart), ctypes.byref(nev), ctypes.byref(bad))
    assert st == 4 and npart.value == 3 and nev.value == 2
