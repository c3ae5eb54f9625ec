"""Seeded synthetic event generators and the reference's text event format.

Events are massless (E = |p|) particles in FP64, built from hard jet axes plus
a soft background, following the workload definitions this library is measured
on:

* ``single_event``  -- one event of N particles with ``n_axes`` hard axes
  (eta U[-2.5, 2.5], phi U[-pi, pi), axis pT from a 1/pT^4 spectrum above
  30 GeV, Poisson(15) constituents per axis with Dirichlet(1) momentum
  fractions and Gaussian sigma=0.1 angular offsets) and a soft background
  (pT Exp(mean 0.7 GeV) floored at 0.1 GeV, eta U[-5, 5]).
* ``mixed_batch``   -- particle counts log-uniform in [lo, hi], Poisson(3)+1 axes.
* ``pileup_batch``  -- 10k-60k particles: soft pT Exp(0.6 GeV), eta U[-4, 4],
  plus 2-6 hard axes.
* ``serving_sizes`` -- lognormal sizes (median 1500, sigma 0.8) clipped to
  [100, 20000] and the algorithm mix 70% anti-kt R=0.4, 15% kt R=0.6,
  15% C/A R=0.8.

The text format is the reference driver's input stream (main.cc:34-70): four
numbers ``px py pz E`` per line, an event ends at the first blank line or line
starting with '#'.

A batch is held as CSR: ``particles`` float64 [total, 4] (px, py, pz, E) and
``offsets`` int64 [n_events + 1].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * math.pi


def _massless(pt, eta, phi):
    px = pt * np.cos(phi)
    py = pt * np.sin(phi)
    pz = pt * np.sinh(eta)
    E = pt * np.cosh(eta)
    return np.stack([px, py, pz, E], axis=1)


def _hard_axes(rng, n_axes, n_max, eta_span=2.5):
    """Constituents of ``n_axes`` hard axes, at most ``n_max`` particles."""
    pts, etas, phis = [], [], []
    for _ in range(n_axes):
        axis_pt = 30.0 * rng.random() ** (-1.0 / 3.0)  # dN/dpT ~ pT^-4 above 30 GeV
        axis_eta = rng.uniform(-eta_span, eta_span)
        axis_phi = rng.uniform(-math.pi, math.pi)
        k = int(rng.poisson(15))
        if k == 0:
            continue
        frac = rng.dirichlet(np.ones(k)) if k > 1 else np.ones(1)
        pts.append(axis_pt * frac)
        etas.append(axis_eta + rng.normal(0.0, 0.1, k))
        phis.append(axis_phi + rng.normal(0.0, 0.1, k))
    if not pts:
        return np.zeros(0), np.zeros(0), np.zeros(0)
    pt = np.concatenate(pts)[:n_max]
    eta = np.concatenate(etas)[:n_max]
    phi = np.concatenate(phis)[:n_max]
    return pt, eta, phi


def single_event(n, n_axes, seed, soft_mean=0.7, soft_eta=5.0):
    """One event of exactly ``n`` massless particles, float64 [n, 4]."""
    rng = np.random.default_rng(seed)
    pt_h, eta_h, phi_h = _hard_axes(rng, n_axes, n)
    n_soft = n - pt_h.size
    pt_s = np.maximum(rng.exponential(soft_mean, n_soft), 0.1)
    eta_s = rng.uniform(-soft_eta, soft_eta, n_soft)
    phi_s = rng.uniform(-math.pi, math.pi, n_soft)
    pt = np.concatenate([pt_h, pt_s])
    eta = np.concatenate([eta_h, eta_s])
    phi = np.concatenate([phi_h, phi_s])
    order = rng.permutation(n)
    return np.ascontiguousarray(_massless(pt[order], eta[order], phi[order]))


@dataclass
class Batch:
    particles: np.ndarray  # float64 [total, 4]
    offsets: np.ndarray  # int64 [n_events + 1]

    @property
    def n_events(self):
        return self.offsets.size - 1

    def sizes(self):
        return np.diff(self.offsets)

    def event(self, e):
        return self.particles[self.offsets[e]:self.offsets[e + 1]]


def _batch_from(events):
    sizes = np.array([ev.shape[0] for ev in events], dtype=np.int64)
    offsets = np.zeros(len(events) + 1, dtype=np.int64)
    np.cumsum(sizes, out=offsets[1:])
    parts = np.concatenate(events, axis=0) if events else np.zeros((0, 4))
    return Batch(np.ascontiguousarray(parts, dtype=np.float64), offsets)


def mixed_batch(n_events=4096, lo=50, hi=2000, seed=3):
    """Events with particle counts log-uniform in [lo, hi], Poisson(3)+1 axes."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), n_events)).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    axes = rng.poisson(3, n_events) + 1
    seeds = rng.integers(0, 2**62, n_events)
    return _batch_from([single_event(int(n), int(a), int(s)) for n, a, s in zip(sizes, axes, seeds)])


def pileup_batch(n_events=64, lo=10000, hi=60000, seed=4):
    """Pile-up-like events: soft pT Exp(0.6), eta U[-4, 4], 2-6 hard axes."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, n_events)
    axes = rng.integers(2, 7, n_events)
    seeds = rng.integers(0, 2**62, n_events)
    return _batch_from([single_event(int(n), int(a), int(s), soft_mean=0.6, soft_eta=4.0)
                        for n, a, s in zip(sizes, axes, seeds)])


# ------------------------------------------------- bit-reproducible generator
#
# The generators above call numpy's distributions and libm (cos, sinh, log),
# whose last bits differ between hosts (x86 and Arm here), so events they make
# are committed as consumed.  The one below uses only the raw 64-bit words of
# PCG64 and correctly rounded IEEE operations (+, -, *, /, sqrt, frexp/ldexp,
# rint), each a separate numpy ufunc or Python float operation, so it yields
# the same bits on every host: large events can be regenerated instead of
# committed.  Its logarithm, exponential and sine/cosine are short series,
# accurate to a few ulp -- only their determinism matters.

_LN2 = 0.6931471805599453
_SQRT_HALF = 0.7071067811865476


def _p_uniform(bitgen, n):
    """n doubles in [0, 1): the top 53 bits of each raw PCG64 word."""
    raw = bitgen.random_raw(n)
    return (raw >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _p_log(x):
    """Natural logarithm of positive x: 2 atanh((m-1)/(m+1)) + e ln2."""
    m, e = np.frexp(x)
    low = m < _SQRT_HALF
    m = np.where(low, m * 2.0, m)
    e = np.where(low, e - 1, e).astype(np.float64)
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    acc = np.full_like(s, 1.0 / 31.0)
    for k in range(14, -1, -1):
        acc = acc * s2 + 1.0 / (2 * k + 1)
    return (2.0 * s) * acc + e * _LN2


def _p_exp(x):
    """exp(x) for |x| < 700: x = k ln2 + r, Taylor series of r, scaled by 2^k."""
    k = np.rint(x / _LN2)
    r = x - k * _LN2
    acc = np.full_like(r, 1.0)
    for j in range(24, 0, -1):
        acc = acc * (r / j) + 1.0
    return np.ldexp(acc, k.astype(np.int64))


def _p_sincos(a):
    """(sin a, cos a) for |a| <= 4: series at a/4, then two angle doublings."""
    q = a * 0.25
    q2 = q * q
    s = np.full_like(q, 0.0)
    c = np.full_like(q, 0.0)
    for j in range(12, -1, -1):
        s = s * q2 * (-1.0 / ((2 * j + 2) * (2 * j + 3))) + 1.0
        c = c * q2 * (-1.0 / ((2 * j + 1) * (2 * j + 2))) + 1.0
    s = s * q
    for _ in range(2):
        s, c = 2.0 * s * c, c * c - s * s
    return s, c


def _p_gauss(bitgen, n, sigma):
    """Gaussian(0, sigma) by Box-Muller on the functions above."""
    u1 = 1.0 - _p_uniform(bitgen, n)  # (0, 1]
    u2 = _p_uniform(bitgen, n)
    rad = np.sqrt(-2.0 * _p_log(u1))
    _, c = _p_sincos((u2 - 0.5) * (2.0 * math.pi))
    return sigma * rad * c


def portable_event(n, n_axes, seed, soft_mean=0.6, soft_eta=4.0, eta_span=2.5):
    """One event of exactly ``n`` massless particles, float64 [n, 4], with the
    same bits on every host.

    Hard axes: axis pT = 30 GeV * u^(-1/3) (a 1/pT^4 spectrum above 30 GeV),
    eta U[-eta_span, eta_span], phi U[-pi, pi); 10-20 constituents with
    momentum fractions from normalised Exp(1) draws (Dirichlet(1)) and
    Gaussian sigma=0.1 offsets in eta and phi.  Soft background: pT
    Exp(soft_mean) floored at 0.1 GeV, eta U[-soft_eta, soft_eta], phi
    U[-pi, pi).  E = |p|.  Particles are in a seeded random order.
    """
    bg = np.random.PCG64(seed)
    pts, etas, phis = [], [], []
    room = n
    for _ in range(n_axes):
        u = _p_uniform(bg, 4)
        axis_pt = float(30.0 * _p_exp(_p_log(1.0 - u[0:1]) * (-1.0 / 3.0))[0])
        axis_eta = float(eta_span * (2.0 * u[1] - 1.0))
        axis_phi = float(math.pi * (2.0 * u[2] - 1.0))
        k = min(10 + int(u[3] * 11.0), room)
        if k <= 0:
            continue
        x = -_p_log(1.0 - _p_uniform(bg, k))
        tot = 0.0
        for v in x.tolist():
            tot += v
        pts.append(axis_pt * (x / tot))
        etas.append(axis_eta + _p_gauss(bg, k, 0.1))
        phis.append(axis_phi + _p_gauss(bg, k, 0.1))
        room -= k
    n_soft = room
    pt_s = np.maximum(-soft_mean * _p_log(1.0 - _p_uniform(bg, n_soft)), 0.1)
    eta_s = soft_eta * (2.0 * _p_uniform(bg, n_soft) - 1.0)
    phi_s = math.pi * (2.0 * _p_uniform(bg, n_soft) - 1.0)
    pt = np.concatenate(pts + [pt_s])
    eta = np.concatenate(etas + [eta_s])
    phi = np.concatenate(phis + [phi_s])
    # azimuth: reduce to [-pi, pi] (constituents may sit past the edge)
    phi = np.where(phi > math.pi, phi - 2.0 * math.pi, np.where(phi < -math.pi, phi + 2.0 * math.pi, phi))
    sn, cs = _p_sincos(phi)
    ep = _p_exp(eta)
    em = 1.0 / ep
    px = pt * cs
    py = pt * sn
    pz = pt * ((ep - em) * 0.5)
    E = np.sqrt(px * px + py * py + pz * pz)
    # seeded permutation: sort by raw words (distinct with overwhelming odds)
    order = np.argsort(bg.random_raw(n), kind="stable")
    return np.ascontiguousarray(np.stack([px, py, pz, E], axis=1)[order])


def portable_pileup(sizes, seed=40, n_axes=(2, 6)):
    """Pile-up-like events of the given sizes (portable_event, 2-6 hard axes)."""
    bg = np.random.PCG64(seed)
    raw = bg.random_raw(2 * len(sizes))
    evs = []
    for i, n in enumerate(sizes):
        axes = n_axes[0] + int(raw[2 * i] % np.uint64(n_axes[1] - n_axes[0] + 1))
        evs.append(portable_event(int(n), axes, int(raw[2 * i + 1] >> np.uint64(1))))
    return evs


def event_sha256(p4):
    """SHA-256 of an event's float64 [n, 4] array (little-endian bytes)."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(p4, dtype="<f8").tobytes()).hexdigest()


ALGO_KT, ALGO_CAM, ALGO_ANTIKT = 1, 0, -1


def serving_mix(n_events, seed=5, median=1500.0, sigma=0.8, lo=100, hi=20000):
    """Sizes and (algorithm, R) per request for the served workload."""
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.exp(rng.normal(math.log(median), sigma, n_events)), lo, hi).astype(np.int64)
    u = rng.random(n_events)
    algo = np.where(u < 0.70, ALGO_ANTIKT, np.where(u < 0.85, ALGO_KT, ALGO_CAM)).astype(np.int32)
    radius = np.where(u < 0.70, 0.4, np.where(u < 0.85, 0.6, 0.8))
    axes = rng.poisson(3, n_events) + 1
    seeds = rng.integers(0, 2**62, n_events)
    batch = _batch_from([single_event(int(n), int(a), int(s)) for n, a, s in zip(sizes, axes, seeds)])
    return batch, algo, radius


# ---------------------------------------------------------------- text format

def read_events(path_or_text):
    """Parse the reference driver's event stream into a list of [n, 4] arrays.

    Follows main.cc:34-70: each line holds px py pz E (anything after the
    fourth number is ignored); an event is a maximal run of such lines; an
    empty line or one starting with '#' ends an event; any other line raises
    ValueError (main.cc:55-58 throws); a final line without a newline is not
    read (the reference's getline loop stops at end of file).  Numbers take an
    optional sign and no inf/nan, as istream >> double reads them.
    """
    if "\n" in path_or_text or not path_or_text:
        text = path_or_text
    else:
        with open(path_or_text) as f:
            text = f.read()
    events, cur = [], []
    lines = text.split("\n")[:-1]  # the piece after the last newline is not read
    for line in lines:
        if not line or line[0] == "#":
            if cur:
                events.append(np.array(cur, dtype=np.float64))
                cur = []
            continue
        vals = _particle_line(line)
        if vals is None:
            raise ValueError("Error while parsing particles:\n" + line)
        cur.append(vals)
    if cur:
        events.append(np.array(cur, dtype=np.float64))
    return events


_NUMBER = None


def _particle_line(line):
    """The first four numbers of a line as istream >> double reads them, or None."""
    global _NUMBER
    if _NUMBER is None:
        import re
        _NUMBER = re.compile(r"[ \t\r\v\f]*([+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?)")
    vals, pos = [], 0
    for _ in range(4):
        m = _NUMBER.match(line, pos)
        if not m:
            return None
        vals.append(float(m.group(1)))
        pos = m.end()
    return vals


def write_events(events, path=None):
    """Write events in the reference's text format ('%.17g', exact round trip)."""
    out = []
    for ev in events:
        for px, py, pz, E in ev:
            out.append(f"{px:.17g} {py:.17g} {pz:.17g} {E:.17g}")
        out.append("")
    text = "\n".join(out)
    if path is not None:
        with open(path, "w") as f:
            f.write(text)
    return text
