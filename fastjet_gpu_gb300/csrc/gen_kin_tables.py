"""Generate fjg_kin_tables.h: constant tables of the fixed-point log/atan2 in fjg_kin.h.

    python fastjet_gpu_gb300/csrc/gen_kin_tables.py > fastjet_gpu_gb300/csrc/fjg_kin_tables.h

All values are computed with Python's decimal module at 80 significant digits
and rounded to the fixed-point scales stated below; 128-bit values are split
into a signed high and an unsigned low 64-bit word.

log tables (two-level reduction, Tang's table method):
  level 1, index i = top 7 fraction bits of the mantissa m in [1, 2); for
  i >= 53 the reduction uses m' = m / 2 (so m' lies in [0.707, 1.414)):
    C1[i]      short reciprocal: c1 = C1 / 512 ~ 1 / m'_centre (c1 = 1 for i = 0, 127)
    LOG1[i]    log(1 / c1) at scale 2^-112
  level 2, index j = floor((z1 + 2^-7) * 2^13) for z1 = m' c1 - 1 in [-2^-7, 2^-7):
    C2[j]      c2 = C2 / 2^14 ~ 1 / (1 + z1_centre) (c2 = 1 for j = 63, 64)
    LOG2[j]    log(1 / c2) at scale 2^-112
  LN2 at scale 2^-112; the log1p polynomial -1/2 + z/3 - z^2/4 + z^3/5 - z^4/6
  at scale 2^-63.
atan tables:
  ATAN[k]    atan(k / 256) at scale 2^-120, k = 0..256
  PI_2, PI   at scale 2^-120
  atan small-argument polynomial 1/3 - d/5 + d^2/7 (scale 2^-64) and the
  small-t series 1/3, 1/5, ... 1/15 (scale 2^-64).
"""
from decimal import ROUND_FLOOR, Decimal, getcontext

getcontext().prec = 80
D = Decimal


def atan_dec(x):
    """atan(x) for 0 <= x <= 1 in Decimal (argument halving + Taylor series)."""
    x = D(x)
    halvings = 0
    while x > D("0.05"):
        x = x / (1 + (1 + x * x).sqrt())
        halvings += 1
    s, term, x2, n = D(0), x, x * x, 1
    while True:
        t = term / n
        if abs(t) < D(10) ** -78:
            break
        s += t if (n // 2) % 2 == 0 else -t
        term *= x2
        n += 2
    return s * (2 ** halvings)


def fixed(v, scale_bits):
    return int((v * (D(2) ** scale_bits)).to_integral_value(rounding="ROUND_HALF_EVEN"))


def split128(n):
    n &= (1 << 128) - 1
    hi, lo = n >> 64, n & ((1 << 64) - 1)
    if hi >= 1 << 63:
        hi -= 1 << 64
    return hi, lo


def emit_array(name, ctype, values, per_line=4):
    out = [f"FJK_TABLE {ctype} {name}[{len(values)}] = {{"]
    for k in range(0, len(values), per_line):
        chunk = values[k:k + per_line]
        if ctype.startswith("int64"):
            txt = ", ".join(f"(int64_t){v}LL" if v >= 0 else f"(int64_t)(-{-v}LL)" if v != -(1 << 63)
                            else "(int64_t)(-9223372036854775807LL - 1)" for v in chunk)
        elif ctype.startswith("uint64"):
            txt = ", ".join(f"{v}ULL" for v in chunk)
        else:
            txt = ", ".join(str(v) for v in chunk)
        out.append("    " + txt + ",")
    out.append("};")
    return "\n".join(out)


def main():
    ln2 = D(2).ln()
    c1, log1 = [], []
    for i in range(128):
        m_lo = 1 + D(i) / 128
        m_hi = 1 + D(i + 1) / 128
        s = 1 if i >= 53 else 0
        mc = (m_lo + m_hi) / 2 / (2 ** s)
        c = 512 if i in (0, 127) else int((D(512) / mc).to_integral_value())
        # check the reduced argument stays inside [-2^-7, 2^-7)
        for m in (m_lo, m_hi):
            z = m / (2 ** s) * D(c) / 512 - 1
            assert -D(2) ** -7 <= z <= D(2) ** -7, (i, z)
        c1.append(c)
        log1.append(fixed((D(512) / D(c)).ln(), 112))
    c2, log2 = [], []
    for j in range(256):
        zc = (D(j) + D("0.5")) * D(2) ** -13 - D(2) ** -7
        c = 1 << 14 if j in (63, 64) else int((D(1 << 14) / (1 + zc)).to_integral_value())
        for z1 in (D(j) * D(2) ** -13 - D(2) ** -7, D(j + 1) * D(2) ** -13 - D(2) ** -7):
            z2 = (1 + z1) * D(c) / (1 << 14) - 1
            assert -D(2) ** -13 <= z2 < D(2) ** -13 or (z1 == D(j + 1) * D(2) ** -13 - D(2) ** -7), (j, z2)
        c2.append(c)
        log2.append(fixed((D(1 << 14) / D(c)).ln(), 112))
    pi = 4 * atan_dec(1)
    atan_tab = [fixed(atan_dec(D(k) / 256), 120) for k in range(257)]

    lines = ["// Generated by gen_kin_tables.py -- do not edit.", "#pragma once", ""]
    lines.append(emit_array("FJK_LOG_C1", "uint16_t", c1, 16))
    lines.append(emit_array("FJK_LOG1_HI", "int64_t", [split128(v)[0] for v in log1]))
    lines.append(emit_array("FJK_LOG1_LO", "uint64_t", [split128(v)[1] for v in log1]))
    lines.append(emit_array("FJK_LOG_C2", "uint16_t", c2, 16))
    lines.append(emit_array("FJK_LOG2_HI", "int64_t", [split128(v)[0] for v in log2]))
    lines.append(emit_array("FJK_LOG2_LO", "uint64_t", [split128(v)[1] for v in log2]))
    lines.append(emit_array("FJK_ATAN_HI", "int64_t", [split128(v)[0] for v in atan_tab]))
    lines.append(emit_array("FJK_ATAN_LO", "uint64_t", [split128(v)[1] for v in atan_tab]))
    hi, lo = split128(fixed(ln2, 112))
    lines.append(f"#define FJK_LN2_112_HI ((int64_t){hi}LL)\n#define FJK_LN2_112_LO ({lo}ULL)")
    for name, val in (("PI_120", pi), ("PI_2_120", pi / 2)):
        hi, lo = split128(fixed(val, 120))
        lines.append(f"#define FJK_{name}_HI ((int64_t){hi}LL)\n#define FJK_{name}_LO ({lo}ULL)")
    # log1p polynomial coefficients, scale 2^-63
    for k, v in enumerate([D(-1) / 2, D(1) / 3, D(-1) / 4, D(1) / 5, D(-1) / 6]):
        n = fixed(v, 63)
        lines.append(f"#define FJK_LQ{k} ((int64_t)({n}LL))")
    # atan polynomials, scale 2^-64 (unsigned magnitudes; signs applied in code)
    for k in range(3, 17, 2):
        lines.append(f"#define FJK_AQ{k} ({fixed(D(1) / k, 64)}ULL)")
    print("\n".join(lines))


if __name__ == "__main__":
    main()
